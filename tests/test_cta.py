"""CTA and cluster modes: long pairs computed by whole thread blocks (the warps
pipeline the pair's row passes through ring rows with published progress), the
largest by clusters of 4 blocks (flags read through distributed shared memory).

Parity with the oracle for local, global and free-end global alignment, the
byte-compare class, the s16 -> s32 redo of long pairs, the device entry point,
the labeller and band mode -- with the CTA threshold forced down to 1 cell so
that short pairs take the same path, and at the default threshold on long pairs.
"""
import numpy as np
import pytest

from pairwise_aligner_gb300 import workloads

pytestmark = pytest.mark.gpu

ACGT = np.frombuffer(b"ACGT", dtype=np.uint8)


@pytest.fixture(scope="module")
def pa(built_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import pairwise_aligner_gb300 as pa
    return pa


def _cfg(local=False, match=2, mismatch=-3, gap_open=-5, gap_extension=-1, **free):
    c = dict(local=local, match=match, mismatch=mismatch, gap_open=gap_open, gap_extension=gap_extension,
             first_column_free=local, first_row_free=local, last_column_free=local, last_row_free=local)
    c.update(free)
    return c


def _oracle_cfg(oracle, c):
    return oracle.make_cfg(c["match"], c["mismatch"], c["gap_open"], c["gap_extension"], local=c["local"],
                           first_column_free=c["first_column_free"], first_row_free=c["first_row_free"],
                           last_column_free=c["last_column_free"], last_row_free=c["last_row_free"])


def _check(oracle, c, s1, o1, s2, o2, res):
    sc, e1, e2 = oracle.align_batch(_oracle_cfg(oracle, c), s1, o1, s2, o2)
    bad = np.flatnonzero((res["score"] != sc) | (res["end1"] != e1) | (res["end2"] != e2))
    assert len(bad) == 0, (len(bad), bad[:5], res[bad[:5]], list(zip(sc[bad[:5]], e1[bad[:5]], e2[bad[:5]])))


def _pairs(seed, shapes, div=0.1, unrelated=False):
    rng = np.random.default_rng(seed)
    s1, s2 = [], []
    for m, n in shapes:
        a = ACGT[rng.integers(0, 4, m)]
        if unrelated:
            b = ACGT[rng.integers(0, 4, n)]
        else:
            b = a.copy()
            flip = rng.random(len(b)) < div
            b[flip] = ACGT[rng.integers(0, 4, int(flip.sum()))]
            b = np.concatenate([b, ACGT[rng.integers(0, 4, max(0, n - m))]])[:n]
        s1.append(bytes(a))
        s2.append(bytes(b))
    from pairwise_aligner_gb300 import pack
    q, qo = pack(s1)
    t, to = pack(s2)
    return q, qo, t, to


SHORT = [(1, 1), (2, 9), (9, 2), (31, 33), (64, 64), (100, 513), (513, 100), (200, 200), (700, 650), (1025, 1030),
         (1500, 400), (400, 1500), (3, 2000), (2000, 3)]


@pytest.mark.parametrize("c", [_cfg(), _cfg(local=True, match=1, mismatch=-4, gap_open=-6),
                               _cfg(last_row_free=True, last_column_free=True),
                               _cfg(first_column_free=True, last_row_free=True),
                               _cfg(match=3, mismatch=-1, gap_open=-2, gap_extension=-2)])
@pytest.mark.parametrize("width", [0, 32])
def test_cta_forced_on_short_pairs(pa, oracle, c, width):
    q, qo, t, to = _pairs(1, SHORT * 3)
    ctx = pa.Context(0)
    ctx.set_cta_threshold(1)
    al = pa.Aligner(dict(c, width_hint=width), context=ctx)
    res = al.compute_arrays(q, qo, t, to)
    _check(oracle, c, q, qo, t, to, res)


@pytest.mark.parametrize("c", [_cfg(), _cfg(local=True, match=1, mismatch=-4, gap_open=-6),
                               _cfg(last_column_free=True)])
def test_cta_long_pairs_default_threshold(pa, oracle, c):
    shapes = [(2100, 2050), (2600, 2500), (3000, 3100), (2048, 4100), (5000, 1000), (2300, 2300)]
    q, qo, t, to = _pairs(2, shapes)
    al = pa.Aligner(c)
    res = al.compute_arrays(q, qo, t, to)
    _check(oracle, c, q, qo, t, to, res)


def test_cta_byte_compare_class(pa, oracle):
    q, qo, t, to = _pairs(3, [(2500, 2400), (2200, 2600), (300, 300)])
    t = t.copy()
    t[100] = ord("N")
    t[2500] = ord("a")
    c = _cfg()
    res = pa.Aligner(c).compute_arrays(q, qo, t, to)
    _check(oracle, c, q, qo, t, to, res)


def test_cta_s16_redo_in_s32(pa, oracle):
    """Long global pairs whose s16 result reaches the clamp floor are redone in s32 lanes."""
    q, qo, t, to = _pairs(4, [(2500, 20000), (2400, 19000), (2600, 2600)], unrelated=True)
    c = _cfg(gap_open=-5, gap_extension=-2)
    al = pa.Aligner(c)
    res = al.compute_arrays(q, qo, t, to)
    _check(oracle, c, q, qo, t, to, res)
    assert al.last_stats["pairs_rerun"] >= 2


def test_cta_device_entry(pa, oracle):
    import torch
    q, qo, t, to = _pairs(5, [(2500, 2500), (3000, 2000), (100, 120), (4000, 4100)])
    c = _cfg(local=True, match=1, mismatch=-4, gap_open=-6)
    dev = torch.device("cuda:0")
    tens = [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in (q, qo.astype(np.int64), t, to.astype(np.int64))]
    out = torch.zeros((4, 16), dtype=torch.uint8, device=dev)
    al = pa.Aligner(c)
    al.compute_device(*tens, out, stats=True)
    res = out.cpu().numpy().reshape(-1).view(pa.RESULT_DTYPE)
    _check(oracle, c, q, qo, t, to, res)


def test_cta_labels_match_oracle(pa, oracle):
    from pairwise_aligner_gb300 import band
    q, qo, t, to = _pairs(6, [(2500, 2600), (700, 800), (3000, 2900), (50, 60)], div=0.08)
    c = _cfg(match=1, mismatch=-4, gap_open=-6)
    for threshold in (1, 1 << 22):
        ctx = pa.Context(0)
        ctx.set_cta_threshold(threshold)
        al = pa.Aligner(c, context=ctx)
        lab = band.labels(ctx, al.c_config(), q, qo, t, to)
        cfg = oracle.make_cfg(1, -4, -6, -1)
        for k in range(4):
            a = bytes(q[qo[k]:qo[k + 1]])
            b = bytes(t[to[k]:to[k + 1]])
            assert list(lab[k]) == oracle.band_labels(cfg, a, b), (threshold, k)


def test_cta_band_mode_exact(pa, oracle):
    d = workloads.config5(seed=56, n_pairs=120, strata=(0.5, 0.4, 0.1))
    c = _cfg(match=1, mismatch=-4, gap_open=-6)
    for threshold, w0 in ((1, 8), (1 << 22, 64), (1 << 22, 2)):
        ctx = pa.Context(0)
        ctx.set_cta_threshold(threshold)
        ctx.set_band_options(straight_w0=w0, w_min=2, full_frac=0.9)
        al = pa.Aligner(dict(c, band_mode=2), context=ctx)
        res = al.compute_arrays(d["seq1"], d["off1"], d["seq2"], d["off2"])
        _check(oracle, c, d["seq1"], d["off1"], d["seq2"], d["off2"], res)


@pytest.mark.parametrize("c", [_cfg(), _cfg(local=True, match=1, mismatch=-4, gap_open=-6),
                               _cfg(last_row_free=True, last_column_free=True)])
def test_cluster_forced_on_short_pairs(pa, oracle, c):
    q, qo, t, to = _pairs(7, SHORT * 2)
    ctx = pa.Context(0)
    ctx.set_cta_threshold(1)
    ctx.set_cluster_threshold(1, 1)
    al = pa.Aligner(c, context=ctx)
    res = al.compute_arrays(q, qo, t, to)
    _check(oracle, c, q, qo, t, to, res)


@pytest.mark.parametrize("c", [_cfg(), _cfg(local=True, match=1, mismatch=-4, gap_open=-6)])
def test_cluster_mode_largest_pairs(pa, oracle, c):
    """Pairs above the default cluster threshold (2^28 cells, 8192 rows), with smaller ones beside."""
    q, qo, t, to = _pairs(8, [(17000, 16500), (16600, 17100), (3000, 2900), (400, 500)], div=0.06)
    al = pa.Aligner(c)
    res = al.compute_arrays(q, qo, t, to)
    _check(oracle, c, q, qo, t, to, res)


def test_cluster_band_mode_exact(pa, oracle):
    d = workloads.config5(seed=57, n_pairs=60, strata=(0.5, 0.3, 0.2))
    c = _cfg(match=1, mismatch=-4, gap_open=-6)
    for w0 in (4, 64):
        ctx = pa.Context(0)
        ctx.set_cta_threshold(1 << 16)
        ctx.set_cluster_threshold(1 << 20, 1024)
        ctx.set_band_options(straight_w0=w0, w_min=2, full_frac=0.9)
        al = pa.Aligner(dict(c, band_mode=2), context=ctx)
        res = al.compute_arrays(d["seq1"], d["off1"], d["seq2"], d["off2"])
        _check(oracle, c, d["seq1"], d["off1"], d["seq2"], d["off2"], res)


def test_largest_pairs_routed_to_blocks_when_many(pa, oracle):
    """More largest-class units than two waves of clusters: the CTA kernel takes them ahead of
    its own list (the lead list); with few, the clusters take them.  Both must be exact."""
    q, qo, t, to = _pairs(9, SHORT * 30)            # 420 pairs: more than 2 x resident clusters units
    c = _cfg()
    for cells in (1, 1 << 40):
        ctx = pa.Context(0)
        ctx.set_cta_threshold(1)
        ctx.set_cluster_threshold(cells, 1)
        al = pa.Aligner(c, context=ctx)
        res = al.compute_arrays(q, qo, t, to)
        _check(oracle, c, q, qo, t, to, res)


def test_band_teams_of_warps_exact(pa, oracle):
    """Narrow bands on long pairs run with teams of 1-4 warps per pair inside a block."""
    q, qo, t, to = _pairs(10, [(6000, 6100), (5000, 4900), (7000, 7050), (4500, 4600)] * 3, div=0.03)
    c = _cfg(match=1, mismatch=-4, gap_open=-6)
    for w0 in (16, 200, 700, 1500):
        ctx = pa.Context(0)
        ctx.set_band_options(straight_w0=w0, w_min=8, full_frac=0.9)
        al = pa.Aligner(dict(c, band_mode=2), context=ctx)
        res = al.compute_arrays(q, qo, t, to)
        _check(oracle, c, q, qo, t, to, res)


@pytest.mark.parametrize("c", [_cfg(), _cfg(local=True, match=1, mismatch=-4, gap_open=-6),
                               _cfg(last_row_free=True, last_column_free=True),
                               _cfg(first_column_free=True, last_row_free=True)])
def test_team_class_forced(pa, oracle, c):
    """Block-mode pairs with few passes on 4-warp teams (the medium class), forced on short pairs."""
    q, qo, t, to = _pairs(11, SHORT * 3)
    for team_rows in (1 << 30, 600):
        ctx = pa.Context(0)
        ctx.set_cta_threshold(1)
        ctx.set_team_threshold(team_rows)
        res = pa.Aligner(c, context=ctx).compute_arrays(q, qo, t, to)
        _check(oracle, c, q, qo, t, to, res)


def test_team_class_long_pairs_and_redo(pa, oracle):
    """Default block threshold, teams for n <= 4096, byte-compare pairs and s16 -> s32 redo among them."""
    q, qo, t, to = _pairs(12, [(2500, 2400), (3000, 3900), (2100, 5000), (4000, 1200)] * 2, unrelated=True)
    t = t.copy()
    t[50] = ord("N")
    for c in (_cfg(gap_open=-5, gap_extension=-2), _cfg(local=True, match=1, mismatch=-4, gap_open=-6)):
        ctx = pa.Context(0)
        ctx.set_team_threshold(4096)
        res = pa.Aligner(c, context=ctx).compute_arrays(q, qo, t, to)
        _check(oracle, c, q, qo, t, to, res)
