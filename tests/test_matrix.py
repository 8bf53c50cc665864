"""Substitution-matrix scoring (cfg::score_model_matrix, PA_SCORE_MATRIX).

CPU: the rule folds into the configuration and sets the method flag; malformed
matrices are rejected.  GPU: the reference's BLOSUM62 known answers through the
Python rule chain, and random protein pairs against the oracle (global with every
end-gap combination, local; group, CTA and cluster modes; large scores), an unknown
symbol as an error, and band mode refused.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import matrix_of, rule_of


def _pairs_of(m: dict):
    return [(sym, row) for sym, row in zip(m["symbols"], m["scores"])]


# -- CPU ----------------------------------------------------------------------------------------

def test_rule_folds_matrix(matrix_kats):
    from pairwise_aligner_gb300 import _lib, cfg
    from pairwise_aligner_gb300.aligner import Aligner
    m = matrix_kats["matrices"]["blosum62_standard"]
    rule = cfg.score_model_matrix(cfg.method_global(cfg.gap_model_affine(-10, -1)), _pairs_of(m))
    flat = cfg.fold(rule)
    sym, scores = matrix_of(m)
    assert flat["matrix"] == (sym, tuple(scores))
    c = Aligner(flat).c_config()
    assert c.method == _lib.PA_METHOD_GLOBAL | _lib.PA_SCORE_MATRIX
    c = Aligner(cfg.fold(cfg.score_model_matrix(cfg.method_local(cfg.gap_model_affine(-10, -1)),
                                                _pairs_of(m)))).c_config()
    assert c.method == _lib.PA_METHOD_LOCAL | _lib.PA_SCORE_MATRIX


def test_rule_rejects_malformed_matrices():
    from pairwise_aligner_gb300 import cfg
    with pytest.raises(ValueError):
        cfg.score_model_matrix([("A", [1, 2]), ("C", [3])])                  # not square
    with pytest.raises(ValueError):
        cfg.score_model_matrix([("A", [1, 2]), ("A", [3, 4])])               # repeated symbol
    with pytest.raises(ValueError):
        cfg.score_model_matrix([(chr(65 + k), [0] * 33) for k in range(33)])  # more than 32 symbols
    with pytest.raises(TypeError):
        cfg.score_model_matrix([("AB", [1])])                                # not one byte
    with pytest.raises(TypeError):                                            # two score models
        cfg.fold(cfg.score_model_matrix(cfg.score_model_unitary(cfg.gap_model_affine(-1, -1), 1, -1),
                                        [("A", [1])]))


# -- GPU ----------------------------------------------------------------------------------------

AMINO = np.frombuffer(b"ACDEFGHIKLMNPQRSTVWY", dtype=np.uint8)


@pytest.fixture(scope="module")
def pa(built_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import pairwise_aligner_gb300 as pa
    return pa


def _protein_pairs(seed, shapes, div=0.25, alphabet=AMINO):
    from pairwise_aligner_gb300 import pack
    rng = np.random.default_rng(seed)
    s1, s2 = [], []
    for m, n in shapes:
        a = alphabet[rng.integers(0, len(alphabet), m)]
        b = a.copy()
        flip = rng.random(len(b)) < div
        b[flip] = alphabet[rng.integers(0, len(alphabet), int(flip.sum()))]
        keep = rng.random(len(b)) > div / 4                  # deletions
        b = b[keep]
        b = np.concatenate([b, alphabet[rng.integers(0, len(alphabet), max(0, n - len(b)))]])[:n]
        s1.append(a.tobytes())
        s2.append(b.tobytes())
    q, qo = pack(s1)
    t, to = pack(s2)
    return q, qo, t, to


def _cfg(matrix, local=False, gap_open=-10, gap_extension=-1, **free):
    c = dict(local=local, match=0, mismatch=0, gap_open=gap_open, gap_extension=gap_extension,
             first_column_free=local, first_row_free=local, last_column_free=local, last_row_free=local,
             matrix=matrix)
    c.update(free)
    return c


def _check(oracle, c, q, qo, t, to, res):
    ocfg = oracle.make_cfg(0, 0, c["gap_open"], c["gap_extension"], local=c["local"],
                           first_column_free=c["first_column_free"], first_row_free=c["first_row_free"],
                           last_column_free=c["last_column_free"], last_row_free=c["last_row_free"],
                           matrix=c["matrix"])
    sc, e1, e2 = oracle.align_batch(ocfg, q, qo, t, to)
    bad = np.flatnonzero((res["score"] != sc) | (res["end1"] != e1) | (res["end2"] != e2))
    assert len(bad) == 0, (len(bad), bad[:5], res[bad[:5]], list(zip(sc[bad[:5]], e1[bad[:5]], e2[bad[:5]])))


@pytest.fixture(scope="module")
def blosum(matrix_kats):
    return matrix_of(matrix_kats["matrices"]["blosum62_standard"])


@pytest.mark.gpu
def test_matrix_kats_through_rules(pa, matrix_kats):
    for c in matrix_kats["cases"]:
        m = matrix_kats["matrices"][c["matrix"]]
        al = pa.cfg.configure_aligner(rule_of(c, _pairs_of(m)))
        assert al.compute(c["seq1"], c["seq2"]).score() == c["expected_score"], (c["source"], c["name"])


@pytest.mark.gpu
def test_matrix_reference_differential_cases(pa, matrix_kats, matrix_cases):
    """The pairs of the reference's matrix SIMD tests (mt19937(42) draws over the BLOSUM62
    symbols); one-vs-many cases go through the one-to-many entry point."""
    from pairwise_aligner_gb300 import pack
    for c in matrix_cases:
        mat = matrix_of(matrix_kats["matrices"][c["matrix"]])
        local = c["method"] == "local"
        cfgd = _cfg(mat, local=local, gap_open=c["gap_open"], gap_extension=c["gap_extension"],
                    **({} if local else dict(first_column_free=c["first_column"] == "free",
                                             first_row_free=c["first_row"] == "free",
                                             last_column_free=c["last_column"] == "free",
                                             last_row_free=c["last_row"] == "free")))
        al = pa.Aligner(cfgd)
        if c["one_vs_many"]:
            res = al.compute(c["seqs1"][0], c["seqs2"])
            got = [(r.score(), *r.end_position()) for r in res]
        else:
            q, qo = pack(c["seqs1"])
            t, to = pack(c["seqs2"])
            r = al.compute_arrays(q, qo, t, to)
            got = list(zip(r["score"].tolist(), r["end1"].tolist(), r["end2"].tolist()))
        want = list(zip(c["oracle_scores"], c["oracle_end1"], c["oracle_end2"]))
        assert got == want, c["name"]


SHAPES = [(0, 5), (5, 0), (1, 1), (2, 9), (9, 2), (20, 21), (31, 33), (64, 64), (100, 130), (257, 200),
          (400, 380), (600, 650), (1025, 1000), (3, 700), (700, 3)]


@pytest.mark.gpu
@pytest.mark.parametrize("kw", [dict(), dict(local=True), dict(last_row_free=True, last_column_free=True),
                                dict(first_column_free=True, last_row_free=True),
                                dict(first_row_free=True, last_column_free=True),
                                dict(gap_open=-5, gap_extension=-2), dict(local=True, gap_open=-11, gap_extension=-1)])
def test_matrix_random_protein_pairs(pa, oracle, blosum, kw):
    q, qo, t, to = _protein_pairs(11, SHAPES * 4)
    c = _cfg(blosum, **kw)
    res = pa.Aligner(c).compute_arrays(q, qo, t, to)
    _check(oracle, c, q, qo, t, to, res)


@pytest.mark.gpu
@pytest.mark.parametrize("local", [False, True])
def test_matrix_block_and_cluster_modes(pa, oracle, blosum, local):
    q, qo, t, to = _protein_pairs(12, SHAPES * 2)
    c = _cfg(blosum, local=local)
    for cta, cluster in ((1, 1 << 40), (1, 1)):
        ctx = pa.Context(0)
        ctx.set_cta_threshold(cta)
        ctx.set_cluster_threshold(cluster, 1)
        res = pa.Aligner(c, context=ctx).compute_arrays(q, qo, t, to)
        _check(oracle, c, q, qo, t, to, res)


@pytest.mark.gpu
def test_matrix_long_pairs_default_thresholds(pa, oracle, blosum):
    q, qo, t, to = _protein_pairs(13, [(2500, 2400), (2100, 2600), (300, 280), (9000, 9100)], div=0.15)
    for local in (False, True):
        c = _cfg(blosum, local=local)
        res = pa.Aligner(c).compute_arrays(q, qo, t, to)
        _check(oracle, c, q, qo, t, to, res)


@pytest.mark.gpu
def test_matrix_large_and_asymmetric_scores(pa, oracle):
    """Scores far beyond 16 bits and a matrix that is not symmetric (row = sequence1 symbol)."""
    rng = np.random.default_rng(14)
    sym = b"ACDEFGHIKLMNPQRSTVWYBZX*"
    dim = len(sym)
    scores = rng.integers(-40000, 30000, dim * dim)
    scores[:: dim + 1] = rng.integers(20000, 60000, dim)
    alphabet = np.frombuffer(sym, dtype=np.uint8)
    q, qo, t, to = _protein_pairs(15, SHAPES * 2, alphabet=alphabet)
    for kw in (dict(), dict(local=True), dict(last_column_free=True)):
        c = _cfg((sym, [int(x) for x in scores]), gap_open=-50000, gap_extension=-7000, **kw)
        res = pa.Aligner(c).compute_arrays(q, qo, t, to)
        _check(oracle, c, q, qo, t, to, res)


@pytest.mark.gpu
def test_matrix_of_unitary_scores_equals_unitary_model(pa):
    from pairwise_aligner_gb300 import pack
    rng = np.random.default_rng(16)
    acgt = np.frombuffer(b"ACGT", dtype=np.uint8)
    s1 = [acgt[rng.integers(0, 4, rng.integers(1, 500))].tobytes() for _ in range(300)]
    s2 = [acgt[rng.integers(0, 4, rng.integers(1, 500))].tobytes() for _ in range(300)]
    q, qo = pack(s1)
    t, to = pack(s2)
    ctx = pa.Context(0)        # one context, switching between the two score models
    for local in (False, True):
        unit = dict(local=local, match=2, mismatch=-3, gap_open=-5, gap_extension=-1, first_column_free=local,
                    first_row_free=local, last_column_free=local, last_row_free=local)
        mat = dict(unit, matrix=(b"ACGT", [2 if i == j else -3 for i in range(4) for j in range(4)]))
        a = pa.Aligner(unit, context=ctx).compute_arrays(q, qo, t, to).copy()
        b = pa.Aligner(mat, context=ctx).compute_arrays(q, qo, t, to).copy()
        c = pa.Aligner(unit, context=ctx).compute_arrays(q, qo, t, to)
        for f in ("score", "end1", "end2"):
            assert np.array_equal(a[f], b[f]) and np.array_equal(a[f], c[f])


@pytest.mark.gpu
def test_matrix_unknown_symbol_is_an_error(pa, blosum):
    from pairwise_aligner_gb300 import _lib, pack
    q, qo = pack([b"ACDEFG", b"ACDJ"])
    t, to = pack([b"ACDEF", b"ACD"])
    with pytest.raises(_lib.PaError) as e:
        pa.Aligner(_cfg(blosum)).compute_arrays(q, qo, t, to)
    assert e.value.status == 1


@pytest.mark.gpu
def test_matrix_refuses_band_mode_and_missing_matrix(pa, blosum):
    import ctypes
    from pairwise_aligner_gb300 import _lib, pack
    q, qo = pack([b"ACDEFG"])
    t, to = pack([b"ACDEF"])
    with pytest.raises(_lib.PaError) as e:
        pa.Aligner(dict(_cfg(blosum), band_mode=2)).compute_arrays(q, qo, t, to)
    assert e.value.status == 5
    ctx = pa.Context(0)                       # PA_SCORE_MATRIX on a context without a matrix
    cfgc = _lib.PaConfig(_lib.PA_METHOD_GLOBAL | _lib.PA_SCORE_MATRIX, 0, 0, -10, -1, 0, 0, 0, 0, 0, 0)
    out = np.zeros(1, dtype=pa.RESULT_DTYPE)
    rc = ctx.lib.pa_align_batch(ctx.ptr, ctypes.byref(cfgc), q.ctypes.data, qo.ctypes.data, t.ctypes.data,
                                to.ctypes.data, 1, out.ctypes.data, None)
    assert rc == 1
