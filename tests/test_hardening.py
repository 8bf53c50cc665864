"""Error paths of the device entry points, checked on the GPU without faulting it.

* A progress wait that gives up: the wait limit is set to 0 polls (give up at the
  first look) on a batch forced into CTA mode, where the passes of a pair wait on
  each other.  The call must return PA_ERR_TIMEOUT (not hang), the affected pairs
  carry PA_RESULT_ERROR, and the same context then aligns the batch exactly.
  This mirrors the reference's only runtime error path, the overflow check that
  throws std::runtime_error (tracker/tracker_global_simd_saturated.hpp:98-100).
* Inconsistent offsets on pa_align_batch_device and pa_align_batch_device_static:
  every index the kernels would compute from them stays inside buffers the test
  allocated (the context's scratch was grown by an earlier, larger call), so the
  check under test is the only thing that changes the outcome.
* Per-pair overflow flags with stats=None, and the bounded graph cache.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(built_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import pairwise_aligner_gb300 as pa
    from pairwise_aligner_gb300 import _lib
    return pa, _lib, torch


def _conf(local=False, match=2, mismatch=-3, gap_open=-5, gap_extension=-1):
    f = bool(local)
    return dict(local=local, match=match, mismatch=mismatch, gap_open=gap_open, gap_extension=gap_extension,
                first_column_free=f, first_row_free=f, last_column_free=f, last_row_free=f, width_hint=0,
                band_mode=0)


def _oracle(oracle, conf, d):
    oc = oracle.make_cfg(conf["match"], conf["mismatch"], conf["gap_open"], conf["gap_extension"],
                         local=conf["local"], first_column_free=conf["first_column_free"],
                         first_row_free=conf["first_row_free"], last_column_free=conf["last_column_free"],
                         last_row_free=conf["last_row_free"])
    return oracle.align_batch(oc, d["seq1"], d["off1"], d["seq2"], d["off2"])


def _device(torch, *arrays):
    dev = torch.device("cuda:0")
    return [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in arrays]


def test_a_wait_that_runs_out_returns_timeout_then_the_context_recovers(env, oracle):
    pa, _lib, torch = env
    from pairwise_aligner_gb300.aligner import Aligner
    rng = np.random.default_rng(31)
    # pairs of 1,500-2,000 rows: several 512-row passes per pair, so the warps of a block wait
    seqs1 = [rng.choice(list(b"ACGT"), size=int(rng.integers(300, 600))).astype(np.uint8).tobytes() for _ in range(24)]
    seqs2 = [rng.choice(list(b"ACGT"), size=int(rng.integers(1500, 2000))).astype(np.uint8).tobytes() for _ in range(24)]
    d = {}
    d["seq1"], d["off1"] = pa.pack(seqs1)
    d["seq2"], d["off2"] = pa.pack(seqs2)
    for local in (True, False):
        conf = _conf(local=local)
        ctx = pa.Context(0)
        ctx.set_cta_threshold(1)                      # every pair on whole blocks (CTA mode)
        ctx.set_team_threshold(0)
        al = Aligner(conf, context=ctx)
        ctx.set_wait_limit(0)
        with pytest.raises(pa.PaError) as e:
            al.compute_arrays(d["seq1"], d["off1"], d["seq2"], d["off2"])
        assert e.value.status == 6                    # PA_ERR_TIMEOUT
        ctx.set_wait_limit(1 << 24)
        res = al.compute_arrays(d["seq1"], d["off1"], d["seq2"], d["off2"])
        sc, e1, e2 = _oracle(oracle, conf, d)
        assert np.array_equal(res["score"], sc)
        assert np.array_equal(res["end1"], e1) and np.array_equal(res["end2"], e2)
        assert not (res["flags"] & _lib.RESULT_ERROR).any()
        ctx.close()


def test_timed_out_pairs_are_flagged_on_the_device_entry(env):
    pa, _lib, torch = env
    from pairwise_aligner_gb300.aligner import Aligner
    rng = np.random.default_rng(32)
    seqs1 = [rng.choice(list(b"ACGT"), size=400).astype(np.uint8).tobytes() for _ in range(16)]
    seqs2 = [rng.choice(list(b"ACGT"), size=1800).astype(np.uint8).tobytes() for _ in range(16)]
    s1, o1 = pa.pack(seqs1)
    s2, o2 = pa.pack(seqs2)
    ctx = pa.Context(0)
    ctx.set_cta_threshold(1)
    ctx.set_team_threshold(0)
    ctx.set_wait_limit(0)
    al = Aligner(_conf(local=True), context=ctx)
    ts1, to1, ts2, to2 = _device(torch, s1, o1.astype(np.int64), s2, o2.astype(np.int64))
    out = torch.zeros(16 * 16, dtype=torch.uint8, device="cuda:0")
    with pytest.raises(pa.PaError) as e:
        al.compute_device(ts1, to1, ts2, to2, out, stats=True)
    assert e.value.status == 6
    got = np.frombuffer(out.cpu().numpy().tobytes(), dtype=pa.RESULT_DTYPE)
    flagged = (got["flags"] & _lib.RESULT_ERROR) != 0
    assert flagged.any()
    assert (got["score"][flagged] == np.iinfo(np.int32).min).all()
    ctx.close()


def test_device_entry_rejects_inconsistent_offsets(env, oracle):
    pa, _lib, torch = env
    from pairwise_aligner_gb300 import workloads as W
    from pairwise_aligner_gb300.aligner import Aligner
    conf = _conf(local=True, match=1, mismatch=-4, gap_open=-6, gap_extension=-1)
    al = Aligner(conf)
    # a first, larger call grows the context's scratch well past every index used below
    big = W.config2(seed=3, n_pairs=4096)
    tb = _device(torch, big["seq1"], big["off1"].astype(np.int64), big["seq2"], big["off2"].astype(np.int64))
    out_big = torch.zeros(4096 * 16, dtype=torch.uint8, device="cuda:0")
    al.compute_device(*tb, out_big, stats=True)
    rng = np.random.default_rng(33)
    buf = rng.choice(list(b"ACGT"), size=4096).astype(np.uint8)
    good1 = np.array([0, 60, 130, 200], dtype=np.int64)
    good2 = np.array([0, 70, 140, 210], dtype=np.int64)
    cases = {
        "decreasing": (np.array([0, 60, 40, 200], dtype=np.int64), good2, 4096, 4096),
        "past seq1_bytes": (good1 + 100, good2, 250, 4096),      # off1[0] != 0 and seq1_bytes too small
        "past seq2_bytes": (good1, good2, 4096, 150),
    }
    ts = _device(torch, buf, buf)
    for name, (o1, o2, b1, b2) in cases.items():
        to1, to2 = _device(torch, o1, o2)
        out = torch.zeros(3 * 16, dtype=torch.uint8, device="cuda:0")
        cfg = al.c_config()
        for with_stats in (True, False):
            st = _lib.PaStats()
            rc = al.context.lib.pa_align_batch_device(al.context.ptr, ctypes.byref(cfg), ts[0].data_ptr(),
                                                      to1.data_ptr(), b1, ts[1].data_ptr(), to2.data_ptr(), b2, 3,
                                                      out.data_ptr(), None, ctypes.byref(st) if with_stats else None)
            torch.cuda.synchronize()
            assert rc == (1 if with_stats else 0), (name, rc)       # PA_ERR_INVALID_ARGUMENT with stats
            got = np.frombuffer(out.cpu().numpy().tobytes(), dtype=pa.RESULT_DTYPE)
            assert (got["score"] == np.iinfo(np.int32).min).all(), name
            assert (got["flags"] & _lib.RESULT_ERROR).all(), name
    # the context still aligns consistent input exactly
    to1, to2 = _device(torch, good1, good2)
    out = torch.zeros(3 * 16, dtype=torch.uint8, device="cuda:0")
    al.compute_device(ts[0], to1, ts[1], to2, out, stats=True)
    got = np.frombuffer(out.cpu().numpy().tobytes(), dtype=pa.RESULT_DTYPE)
    d = dict(seq1=buf, off1=good1.astype(np.uint64), seq2=buf, off2=good2.astype(np.uint64))
    sc, e1, e2 = _oracle(oracle, conf, d)
    assert np.array_equal(got["score"], sc) and np.array_equal(got["end1"], e1) and np.array_equal(got["end2"], e2)


def test_static_entry_flags_inconsistent_offsets(env):
    pa, _lib, torch = env
    from pairwise_aligner_gb300.aligner import Aligner
    lib = _lib.load()
    al = Aligner(_conf(local=True, match=1, mismatch=-4, gap_open=-6, gap_extension=-1))
    cfg = al.c_config()
    rng = np.random.default_rng(34)
    buf = rng.choice(list(b"ACGT"), size=4096).astype(np.uint8)
    # off1[0] != 0 and a seq1_bytes that is too small for the last pair: all reads stay inside
    # the 4,096-byte buffer and all scratch rows inside the static array even without the check
    o1 = np.array([100, 160, 230, 300], dtype=np.int64)
    o2 = np.array([0, 70, 140, 210], dtype=np.int64)
    ts1, ts2, to1, to2 = _device(torch, buf, buf, o1, o2)
    out = torch.zeros(3 * 16, dtype=torch.uint8, device="cuda:0")
    rc = lib.pa_align_batch_device_static(ctypes.byref(cfg), ts1.data_ptr(), to1.data_ptr(), 250, ts2.data_ptr(),
                                          to2.data_ptr(), 4096, 3, out.data_ptr(), None)
    torch.cuda.synchronize()
    assert rc == 0
    got = np.frombuffer(out.cpu().numpy().tobytes(), dtype=pa.RESULT_DTYPE)
    # pairs 0 and 1 end inside the declared 250 bytes; pair 2 ends at 300
    assert not (got["flags"][:2] & _lib.RESULT_ERROR).any()
    assert got["flags"][2] & _lib.RESULT_ERROR and got["score"][2] == np.iinfo(np.int32).min


def test_overflow_pairs_are_flagged_without_stats(env, oracle):
    pa, _lib, torch = env
    from pairwise_aligner_gb300.aligner import Aligner
    conf = _conf(local=False, match=1 << 20, mismatch=-(1 << 20), gap_open=-5, gap_extension=-1)
    al = Aligner(conf)
    s1, o1 = pa.pack(["ACGT" * 300, "ACGT"])
    s2, o2 = pa.pack(["ACGT" * 300, "ACGA"])
    ts1, to1, ts2, to2 = _device(torch, s1, o1.astype(np.int64), s2, o2.astype(np.int64))
    out = torch.zeros(2 * 16, dtype=torch.uint8, device="cuda:0")
    al.compute_device(ts1, to1, ts2, to2, out)        # stats=None: returns once queued
    torch.cuda.synchronize()
    got = np.frombuffer(out.cpu().numpy().tobytes(), dtype=pa.RESULT_DTYPE)
    assert got["flags"][0] & _lib.RESULT_OVERFLOW and got["score"][0] == np.iinfo(np.int32).min
    oc = oracle.make_cfg(1 << 20, -(1 << 20), -5, -1)
    assert not got["flags"][1] & _lib.RESULT_OVERFLOW and got["score"][1] == oracle.align(oc, b"ACGT", b"ACGA")[0]
    with pytest.raises(pa.PaError) as e:               # with stats the call reports it
        al.compute_device(ts1, to1, ts2, to2, out, stats=True)
    assert e.value.status == 4


def test_graph_cache_stays_bounded(env, oracle):
    pa, _lib, torch = env
    from pairwise_aligner_gb300 import workloads as W
    from pairwise_aligner_gb300.aligner import Aligner
    d = W.config2(seed=35, n_pairs=256)
    conf = _conf(local=True, match=1, mismatch=-4, gap_open=-6, gap_extension=-1)
    al = Aligner(conf)
    ts1, to1, ts2, to2 = _device(torch, d["seq1"], d["off1"].astype(np.int64), d["seq2"], d["off2"].astype(np.int64))
    sc, e1, e2 = _oracle(oracle, conf, d)
    outs = [torch.zeros(256 * 16, dtype=torch.uint8, device="cuda:0") for _ in range(50)]
    for k, out in enumerate(outs):                    # 50 buffer sets: 50 distinct captures
        al.compute_device(ts1, to1, ts2, to2, out)
        assert al.context.graph_count() <= 8, k
    torch.cuda.synchronize()
    for out in outs[-10:]:
        got = np.frombuffer(out.cpu().numpy().tobytes(), dtype=pa.RESULT_DTYPE)
        assert np.array_equal(got["score"], sc) and np.array_equal(got["end1"], e1) and np.array_equal(got["end2"], e2)
    assert al.context.graph_count() == 8
