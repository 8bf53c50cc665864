"""GPU parity: the CUDA path through the C ABI against the oracle (bit-exact).

Mirrors the reference's test strategy: the hand-written scalar KATs, the
differential SIMD-vs-scalar cases on its mt19937(42) pairs, and seeded
batches of the benchmark configurations compared with the oracle.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import oracle_cfg_of, rule_of

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pa(built_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import pairwise_aligner_gb300 as pa
    return pa


def _oracle_for(oracle, d):
    return oracle.make_cfg(d["match"], d["mismatch"], d["gap_open"], d["gap_extension"], local=d["local"],
                           first_column_free=d.get("first_column_free", False),
                           first_row_free=d.get("first_row_free", False),
                           last_column_free=d.get("last_column_free", False),
                           last_row_free=d.get("last_row_free", False))


def _aligner_for(pa, d, **kw):
    from pairwise_aligner_gb300.aligner import Aligner
    cfg = dict(local=d["local"], match=d["match"], mismatch=d["mismatch"], gap_open=d["gap_open"],
               gap_extension=d["gap_extension"], first_column_free=d.get("first_column_free", False),
               first_row_free=d.get("first_row_free", False), last_column_free=d.get("last_column_free", False),
               last_row_free=d.get("last_row_free", False), width_hint=kw.pop("width_hint", 0), band_mode=0)
    if d["local"]:
        cfg.update(first_column_free=True, first_row_free=True, last_column_free=True, last_row_free=True)
    ctx = pa.Context(0, **kw) if kw else None
    return Aligner(cfg, context=ctx)


def _check(oracle, d, res, nthreads=None):
    sc, e1, e2 = oracle.align_batch(_oracle_for(oracle, d), d["seq1"], d["off1"], d["seq2"], d["off2"],
                                    nthreads=nthreads)
    bad = np.flatnonzero((res["score"] != sc) | (res["end1"] != e1) | (res["end2"] != e2))
    assert len(bad) == 0, (f"{len(bad)} mismatches; first {bad[:5]}: gpu {res[bad[:5]]} "
                           f"oracle {list(zip(sc[bad[:5]], e1[bad[:5]], e2[bad[:5]]))}")


def test_scalar_kats_through_cfg(pa, kats):
    for c in kats:
        aligner = pa.cfg.configure_aligner(rule_of(c))
        r = aligner.compute(c["seq1"], c["seq2"])
        assert r.score() == c["expected_score"], (c["source"], c["name"], r.score())


def test_reference_differential_cases(pa, oracle, simd_cases):
    for c in simd_cases:
        aligner = pa.cfg.configure_aligner(rule_of(c))
        res = aligner.compute(c["seqs1"], c["seqs2"])
        got = [(r.score(), *r.end_position()) for r in res]
        want = list(zip(c["oracle_scores"], c["oracle_end1"], c["oracle_end2"]))
        assert got == want, c["name"]


@pytest.mark.parametrize("group_threads", [1, 2, 4, 8, 16, 32])
def test_group_sizes_config2_sample(pa, oracle, group_threads):
    from pairwise_aligner_gb300 import workloads as W
    d = W.config2(seed=11, n_pairs=2048)
    res = _aligner_for(pa, d, group_threads=group_threads).compute_arrays(d["seq1"], d["off1"], d["seq2"], d["off2"])
    _check(oracle, d, res)


@pytest.mark.parametrize("local", [True, False])
@pytest.mark.parametrize("use_graphs,variant", [(-1, 0), (1, 1), (-1, 2), (1, 3), (-1, 4)])
def test_launch_paths_and_variants(pa, oracle, use_graphs, variant, local):
    """Direct launches and graph replays, every inner-loop variant: same results, stats filled."""
    from pairwise_aligner_gb300 import workloads as W
    d = W.config2(seed=13, n_pairs=3000)
    if not local:
        d.update(local=False, last_row_free=variant % 2 == 1)
    al = _aligner_for(pa, d, use_graphs=use_graphs, kernel_variant=variant)
    for _ in range(2):
        res = al.compute_arrays(d["seq1"], d["off1"], d["seq2"], d["off2"])
        _check(oracle, d, res)
        assert al.last_stats["device_ms"] > 0 and al.last_stats["dp_ms"] > 0


def test_config1_full(pa, oracle):
    from pairwise_aligner_gb300 import workloads as W
    d = W.config1()
    al = _aligner_for(pa, d)
    res = al.compute_arrays(d["seq1"], d["off1"], d["seq2"], d["off2"])
    _check(oracle, d, res)
    assert al.last_stats["pairs_s16"] == 1024


def test_config2_sample(pa, oracle):
    from pairwise_aligner_gb300 import workloads as W
    d = W.config2(seed=2, n_pairs=16384)
    res = _aligner_for(pa, d).compute_arrays(d["seq1"], d["off1"], d["seq2"], d["off2"])
    _check(oracle, d, res)


def test_config3_sample(pa, oracle):
    from pairwise_aligner_gb300 import workloads as W
    d = W.config3(seed=3, n_pairs=64)
    res = _aligner_for(pa, d).compute_arrays(d["seq1"], d["off1"], d["seq2"], d["off2"])
    _check(oracle, d, res)


@pytest.mark.parametrize("flags", [(1, 0, 1, 0), (0, 1, 0, 1), (1, 1, 1, 1), (0, 0, 1, 0), (0, 0, 0, 1),
                                   (1, 1, 0, 0)])
@pytest.mark.parametrize("width", [0, 32])
def test_end_gap_variants(pa, oracle, flags, width):
    from pairwise_aligner_gb300 import workloads as W
    d = W.config2(seed=5, n_pairs=1024)
    d.update(local=False, match=4, mismatch=-5, gap_open=-10, gap_extension=-1)
    d["first_column_free"], d["first_row_free"], d["last_column_free"], d["last_row_free"] = map(bool, flags)
    res = _aligner_for(pa, d, width_hint=width).compute_arrays(d["seq1"], d["off1"], d["seq2"], d["off2"])
    _check(oracle, d, res)


def test_width_16_and_32_agree_at_full_config2_size(pa):
    """Size-independent property at the full 262,144-pair size: two different kernels agree."""
    from pairwise_aligner_gb300 import workloads as W
    d = W.config2()
    a16 = _aligner_for(pa, d).compute_arrays(d["seq1"], d["off1"], d["seq2"], d["off2"])
    a32 = _aligner_for(pa, d, width_hint=32).compute_arrays(d["seq1"], d["off1"], d["seq2"], d["off2"])
    assert (a16["width"] == 16).all() and (a32["width"] == 32).all()
    assert np.array_equal(a16["score"], a32["score"])
    assert np.array_equal(a16["end1"], a32["end1"]) and np.array_equal(a16["end2"], a32["end2"])
    m = np.diff(d["off1"].astype(np.int64))
    n = np.diff(d["off2"].astype(np.int64))
    assert (a16["score"] >= 0).all()
    assert ((a16["score"] == 0) == ((a16["end1"] == 0) & (a16["end2"] == 0))).all()
    assert (a16["end1"] <= m).all() and (a16["end2"] <= n).all()


def test_rerun_promotes_to_s32(pa, oracle):
    rng = np.random.default_rng(9)
    seqs1 = [rng.choice(list(b"ACGT"), size=20000).astype(np.uint8).tobytes() for _ in range(4)] + [b"ACGT" * 10] * 4
    seqs2 = [rng.choice(list(b"ACGT"), size=40).astype(np.uint8).tobytes() for _ in range(4)] + [b"ACGA" * 10] * 4
    d = dict(local=False, match=2, mismatch=-4, gap_open=-4, gap_extension=-2)
    d["seq1"], d["off1"] = pa.pack(seqs1)
    d["seq2"], d["off2"] = pa.pack(seqs2)
    al = _aligner_for(pa, d)
    res = al.compute_arrays(d["seq1"], d["off1"], d["seq2"], d["off2"])
    _check(oracle, d, res)
    assert al.last_stats["pairs_rerun"] == 4
    assert (res["width"][:4] == 32).all() and (res["flags"][:4] & 1).all()
    assert (res["width"][4:] == 16).all()


def test_edge_cases(pa, oracle):
    seqs1 = ["", "A", "", "ACGT", "N", "acgt", "ACGTNNACGT", "A" * 700, "T", "ACGTACGTAC"]
    seqs2 = ["", "", "C", "ACGT", "N", "ACGT", "ACGTNNACGT", "A" * 300, "T" * 1000, "ACGTACGTAC" * 60]
    for local in (False, True):
        for flags in ((0, 0, 0, 0), (1, 1, 1, 1), (0, 1, 0, 1)):
            d = dict(local=local, match=3, mismatch=-2, gap_open=-4, gap_extension=-1,
                     first_column_free=bool(flags[0]), first_row_free=bool(flags[1]),
                     last_column_free=bool(flags[2]), last_row_free=bool(flags[3]))
            d["seq1"], d["off1"] = pa.pack(seqs1)
            d["seq2"], d["off2"] = pa.pack(seqs2)
            res = _aligner_for(pa, d).compute_arrays(d["seq1"], d["off1"], d["seq2"], d["off2"])
            _check(oracle, d, res)


def test_large_scores_use_the_byte_compare_path(pa, oracle):
    from pairwise_aligner_gb300 import workloads as W
    d = W.config1(seed=4, n_pairs=256)
    d.update(match=300, mismatch=-200, gap_open=-500, gap_extension=-100)
    al = _aligner_for(pa, d)
    res = al.compute_arrays(d["seq1"], d["off1"], d["seq2"], d["off2"])
    _check(oracle, d, res)
    assert al.last_stats["pairs_general"] == 256


def test_one_to_many_and_single(pa, oracle):
    aligner = pa.cfg.configure_aligner(pa.cfg.method_local(pa.cfg.gap_model_affine(
        pa.cfg.score_model_unitary(4, -5), -10, -1)))
    targets = ["TTTTTCTGACACACT", "ACGT", "", "CTGCACACGACGGGGGG"]
    res = aligner.compute("CTGCACACGACGGGGGG", targets)
    cfg = oracle.make_cfg(4, -5, -10, -1, local=True)
    for t, r in zip(targets, res):
        assert (r.score(), *r.end_position()) == oracle.align(cfg, b"CTGCACACGACGGGGGG", t.encode())
    single = aligner.compute("CTGCACACGACGGGGGG", "TTTTTCTGACACACT")
    assert single.score() == 21


def test_device_entry_matches_host_entry(pa):
    import torch
    from pairwise_aligner_gb300 import workloads as W
    d = W.config2(seed=8, n_pairs=4096)
    al = _aligner_for(pa, d)
    host = al.compute_arrays(d["seq1"], d["off1"], d["seq2"], d["off2"])
    dev = torch.device("cuda:0")
    s1 = torch.from_numpy(d["seq1"]).to(dev)
    s2 = torch.from_numpy(d["seq2"]).to(dev)
    o1 = torch.from_numpy(d["off1"].astype(np.int64)).to(dev)
    o2 = torch.from_numpy(d["off2"].astype(np.int64)).to(dev)
    out = torch.zeros(4096 * 16, dtype=torch.uint8, device=dev)
    for _ in range(2):                                   # second call replays the captured graph
        al.compute_device(s1, o1, s2, o2, out, stream=torch.cuda.current_stream(), stats=True)
        torch.cuda.synchronize()
        got = np.frombuffer(out.cpu().numpy().tobytes(), dtype=pa.RESULT_DTYPE)
        assert np.array_equal(got["score"], host["score"])
        assert np.array_equal(got["end1"], host["end1"]) and np.array_equal(got["end2"], host["end2"])


def test_invalid_arguments(pa):
    from pairwise_aligner_gb300.aligner import Aligner
    bad = Aligner(dict(local=False, match=1, mismatch=-1, gap_open=2, gap_extension=-1, first_column_free=0,
                       first_row_free=0, last_column_free=0, last_row_free=0))
    with pytest.raises(pa.PaError) as e:
        bad.compute(["A"], ["A"])
    assert e.value.status == 5
    ok = Aligner(dict(local=False, match=1, mismatch=-1, gap_open=-2, gap_extension=-1, first_column_free=0,
                      first_row_free=0, last_column_free=0, last_row_free=0))
    with pytest.raises(ValueError):
        ok.compute_arrays(*pa.pack(["A", "C"]), *pa.pack(["A"]))


def test_autotune_fills_the_batch_bucket_and_stays_exact(pa, oracle, tmp_path):
    """pa_autotune times the candidates on this batch and keeps the winner in the table entry
    of its method, batch-size class (2,048 pairs: class 0) and pair-size class (mean m*n of
    about 82,000: class 2); the other entries stay untuned; the choice survives a save/load."""
    from pairwise_aligner_gb300 import workloads as W
    d = W.config2(seed=17, n_pairs=2048)
    al = _aligner_for(pa, d)
    ctx = al.context
    before = ctx.tuning()
    t = ctx.autotune(al.c_config(), d["seq1"], d["off1"], d["seq2"], d["off2"])
    e = t["s16"][0][0][2]
    assert 0 <= e["variant"] <= 10 and e["group_threads"] in (1, 2, 4, 8, 16, 32) and e["dp_ms"] > 0
    for mi in range(2):
        for a in range(5):
            for b in range(4):
                if (mi, a, b) != (0, 0, 2):
                    assert t["s16"][mi][a][b] == before["s16"][mi][a][b]
    res = al.compute_arrays(d["seq1"], d["off1"], d["seq2"], d["off2"])
    _check(oracle, d, res)
    path = str(tmp_path / "tuning.json")
    ctx.save_tuning(path)
    fresh = pa.Context(0)
    fresh.load_tuning(path)
    assert fresh.tuning()["s16"] == t["s16"]


@pytest.mark.parametrize("local", [True, False])
def test_every_autotune_candidate_is_exact(pa, oracle, local):
    """Each (kernel variant, group size) pa_autotune can choose: the short-pair kernel with 16
    and 32 rows per thread at G = 4..32, and the general kernel down to G = 1 (one pair per
    lane, two per thread in s16x2 halves)."""
    from pairwise_aligner_gb300 import workloads as W
    d = W.config2(seed=19, n_pairs=1024) if local else W.config4(seed=19, n_pairs=512)
    cands = [(v, g) for v in (9, 10) for g in (4, 8, 16, 32)] + [(7 if local else 4, g) for g in (1, 2, 4, 8, 16, 32)]
    for v, g in cands:
        res = _aligner_for(pa, d, group_threads=g, kernel_variant=v).compute_arrays(
            d["seq1"], d["off1"], d["seq2"], d["off2"])
        _check(oracle, d, res)


def test_config5_stratified_sample(pa, oracle):
    """Mixed global stream: short, long and very long (20-50 kb + structural indels) pairs in one batch."""
    from pairwise_aligner_gb300 import workloads as W
    d = W.config5(seed=5, n_pairs=400, strata=(0.90, 0.085, 0.015))
    al = _aligner_for(pa, d)
    res = al.compute_arrays(d["seq1"], d["off1"], d["seq2"], d["off2"])
    _check(oracle, d, res, nthreads=os.cpu_count())
    st = al.last_stats
    assert st["pairs_s16"] + st["pairs_s32"] == 400


def test_config4_sample(pa, oracle):
    from pairwise_aligner_gb300 import workloads as W
    d = W.config4(seed=4, n_pairs=2048)
    res = _aligner_for(pa, d).compute_arrays(d["seq1"], d["off1"], d["seq2"], d["off2"])
    _check(oracle, d, res)
