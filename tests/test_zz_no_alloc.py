"""pa_align_batch_device_static: the entry point that allocates nothing.

Callers that cannot allocate device memory when they align (an allocator that
must own every byte, code running inside CUDA-graph capture, latency-critical
paths) use this entry point; its only scratch is a fixed device array inside the
library.  The test calls it through the C ABI on device buffers the test owns and
checks, on two calls in a row, that its scores and end positions equal those of
pa_align_batch_device on the same inputs (exact: the scores are integers).  The
file is named so that pytest collects it last; it also passes on its own in a
fresh process, because the first call on a device does its own set-up.
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
    return pa, _lib, _lib.load(), torch


def _device_batch(torch, d):
    dev = torch.device("cuda:0")
    s1 = torch.from_numpy(np.array(d["seq1"])).to(dev)
    s2 = torch.from_numpy(np.array(d["seq2"])).to(dev)
    o1 = torch.from_numpy(d["off1"].astype(np.int64)).to(dev)
    o2 = torch.from_numpy(d["off2"].astype(np.int64)).to(dev)
    return s1, o1, s2, o2


def _static_call(lib, _lib, cfg, s1, o1, s2, o2, out, n, stream):
    return lib.pa_align_batch_device_static(ctypes.byref(cfg), s1.data_ptr(), o1.data_ptr(), s1.numel(),
                                            s2.data_ptr(), o2.data_ptr(), s2.numel(), n, out.data_ptr(), stream)


def _workload(pa, local: bool):
    from pairwise_aligner_gb300 import workloads as W
    d = W.config2(seed=21, n_pairs=3000)
    extra1, extra2 = ["", "ACGT", "A" * 700, "NNACGTNN", "acgt"], ["ACG", "", "A" * 300, "NACGTN", "ACGT"]
    s1, o1 = pa.pack([bytes(d["seq1"][d["off1"][k]:d["off1"][k + 1]]) for k in range(3000)] + extra1)
    s2, o2 = pa.pack([bytes(d["seq2"][d["off2"][k]:d["off2"][k + 1]]) for k in range(3000)] + extra2)
    return dict(seq1=s1, off1=o1, seq2=s2, off2=o2, local=local)


@pytest.mark.parametrize("local,flags", [(True, (1, 1, 1, 1)), (False, (0, 0, 0, 0)), (False, (1, 0, 1, 1))])
def test_static_entry_matches_the_allocating_entry_twice(env, local, flags):
    pa, _lib, lib, torch = env
    from pairwise_aligner_gb300.aligner import Aligner
    d = _workload(pa, local)
    n = len(d["off1"]) - 1
    conf = dict(local=local, match=1, mismatch=-4, gap_open=-6, gap_extension=-1, first_column_free=flags[0],
                first_row_free=flags[1], last_column_free=flags[2], last_row_free=flags[3], width_hint=0,
                band_mode=0)
    al = Aligner(conf)
    s1, o1, s2, o2 = _device_batch(torch, d)
    want = torch.zeros(n * 16, dtype=torch.uint8, device="cuda:0")
    al.compute_device(s1, o1, s2, o2, want, stream=torch.cuda.current_stream(), stats=True)
    torch.cuda.synchronize()
    want = np.frombuffer(want.cpu().numpy().tobytes(), dtype=pa.RESULT_DTYPE)
    cfg = al.c_config()
    for call in range(2):                       # the second call reuses the static scratch
        out = torch.full((n * 16,), 0xAB, dtype=torch.uint8, device="cuda:0")
        rc = _static_call(lib, _lib, cfg, s1, o1, s2, o2, out, n, None)
        assert rc == 0, _lib.STATUS.get(rc, rc)
        torch.cuda.synchronize()
        got = np.frombuffer(out.cpu().numpy().tobytes(), dtype=pa.RESULT_DTYPE)
        assert np.array_equal(got["score"], want["score"]), f"call {call}: scores differ"
        assert np.array_equal(got["end1"], want["end1"]) and np.array_equal(got["end2"], want["end2"]), call
        assert (got["width"] == 32).all()


def test_static_entry_rejects_sizes_beyond_its_scratch(env):
    pa, _lib, lib, torch = env
    from pairwise_aligner_gb300.aligner import Aligner
    al = Aligner(dict(local=True, match=1, mismatch=-4, gap_open=-6, gap_extension=-1, first_column_free=1,
                      first_row_free=1, last_column_free=1, last_row_free=1))
    cfg = al.c_config()
    dummy = torch.zeros(16, dtype=torch.uint8, device="cuda:0")
    offs = torch.zeros(3, dtype=torch.int64, device="cuda:0")
    out = torch.zeros(32, dtype=torch.uint8, device="cuda:0")
    # 4,194,304 scratch cells: seq1_bytes + n_pairs above that is refused before any launch
    rc = lib.pa_align_batch_device_static(ctypes.byref(cfg), dummy.data_ptr(), offs.data_ptr(), 4194303,
                                          dummy.data_ptr(), offs.data_ptr(), 16, 2, out.data_ptr(), None)
    assert rc == 8                               # PA_ERR_TOO_LARGE
    assert (out.cpu() == 0).all()


def test_static_entry_flags_over_bound_and_empty_pairs(env, oracle):
    """Per-pair flags: a pair over both entries' int32 bounds (match 2^20 on 1,100 bases; the
    allocating entry's bound also counts the column shift of its s16 lanes, so it is the
    stricter of the two) gets INT32_MIN and PA_RESULT_OVERFLOW from both device entries (the
    allocating one without a stats block too); an empty global pair ("", "") carries the same
    flags and border result from both entries, and the oracle's score."""
    pa, _lib, lib, torch = env
    from pairwise_aligner_gb300.aligner import Aligner
    rng = np.random.default_rng(5)
    acgt = np.frombuffer(b"ACGT", np.uint8)
    a = acgt[rng.integers(0, 4, 1100)].tobytes()
    pairs = [(a, a), (b"", b""), (b"ACGTAC", b"ACGAC"), (a[:40], a[:40])]
    s1, o1 = pa.pack([p[0] for p in pairs])
    s2, o2 = pa.pack([p[1] for p in pairs])
    d = dict(seq1=s1, off1=o1, seq2=s2, off2=o2)
    n = len(pairs)
    t1, u1, t2, u2 = _device_batch(torch, d)
    conf = dict(local=False, match=1 << 20, mismatch=-4, gap_open=-6, gap_extension=-1, first_column_free=0,
                first_row_free=0, last_column_free=0, last_row_free=0, width_hint=0, band_mode=0)
    al = Aligner(conf)
    main = torch.zeros(n * 16, dtype=torch.uint8, device="cuda:0")
    al.compute_device(t1, u1, t2, u2, main, stream=torch.cuda.current_stream(), stats=False)
    torch.cuda.synchronize()
    main = np.frombuffer(main.cpu().numpy().tobytes(), dtype=pa.RESULT_DTYPE)
    out = torch.zeros(n * 16, dtype=torch.uint8, device="cuda:0")
    rc = _static_call(lib, _lib, al.c_config(), t1, u1, t2, u2, out, n, None)
    assert rc == 0, _lib.STATUS.get(rc, rc)
    torch.cuda.synchronize()
    got = np.frombuffer(out.cpu().numpy().tobytes(), dtype=pa.RESULT_DTYPE)
    for res in (main, got):
        assert res["score"][0] == np.iinfo(np.int32).min and res["flags"][0] & 0x10
        assert not (res["flags"][1:] & 0x10).any()
    assert got["flags"][1] == main["flags"][1] and got["flags"][1] & 0x08
    oc = oracle.make_cfg(1 << 20, -4, -6, -1)
    for k in (1, 2, 3):
        want = oracle.align(oc, pairs[k][0], pairs[k][1])
        for res in (main, got):
            assert (int(res["score"][k]), int(res["end1"][k]), int(res["end2"][k])) == want, k
