"""The oracle against the reference's own golden vectors (CPU only).

* every hand-written expected score of the reference's scalar tests
  (test/unit/affine/*_scalar_test.cpp, test/unit/configuration/*.cpp);
* the reference's differential SIMD-vs-scalar cases: the oracle's
  inter-sequence SIMD port must agree with its scalar restatement on the exact
  mt19937(42) pairs the reference's tests align, as the reference's
  SIMD lanes agree with its scalar aligner (alignment_simd_test_template.hpp:195-227);
* local end coordinates follow the documented tie-break.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import matrix_of, oracle_cfg_of


def test_scalar_kats(oracle, kats):
    assert len(kats) >= 22
    for c in kats:
        sc, e1, e2 = oracle.align(oracle_cfg_of(oracle, c), c["seq1"].encode(), c["seq2"].encode())
        assert sc == c["expected_score"], (c["source"], c["name"])


def test_matrix_kats(oracle, matrix_kats):
    """BLOSUM62 global / local expected scores of the reference's matrix tests."""
    assert len(matrix_kats["cases"]) >= 6
    for c in matrix_kats["cases"]:
        cfg = oracle_cfg_of(oracle, c, matrix_of(matrix_kats["matrices"][c["matrix"]]))
        sc, _, _ = oracle.align(cfg, c["seq1"].encode(), c["seq2"].encode())
        assert sc == c["expected_score"], (c["source"], c["name"])


def test_matrix_fixture_scores_are_the_oracles(oracle, matrix_kats, matrix_cases):
    assert len(matrix_cases) >= 40
    for c in matrix_cases[::5]:
        cfg = oracle_cfg_of(oracle, c, matrix_of(matrix_kats["matrices"][c["matrix"]]))
        for a, b, s, e1, e2 in list(zip(c["seqs1"], c["seqs2"], c["oracle_scores"], c["oracle_end1"],
                                        c["oracle_end2"]))[:6]:
            assert oracle.align(cfg, a.encode(), b.encode()) == (s, e1, e2)


def test_matrix_rejects_unknown_symbol(oracle, matrix_kats):
    cfg = oracle_cfg_of(oracle, matrix_kats["cases"][0], matrix_of(matrix_kats["matrices"]["blosum62_standard"]))
    with pytest.raises(RuntimeError):
        oracle.align(cfg, b"ACDJ", b"ACD")


def test_matrix_with_unitary_scores_is_unitary(oracle):
    """A matrix with match on the diagonal and mismatch elsewhere scores as the unitary model."""
    rng = np.random.default_rng(3)
    sym = b"ACGT"
    scores = [2 if i == j else -3 for i in range(4) for j in range(4)]
    for local in (False, True):
        cu = oracle.make_cfg(2, -3, -5, -1, local=local)
        cm = oracle.make_cfg(0, 0, -5, -1, local=local, matrix=(sym, scores))
        for _ in range(20):
            a = rng.choice(np.frombuffer(sym, np.uint8), rng.integers(0, 40)).tobytes()
            b = rng.choice(np.frombuffer(sym, np.uint8), rng.integers(0, 40)).tobytes()
            assert oracle.align(cu, a, b) == oracle.align(cm, a, b)


def test_fixture_scores_are_the_oracles(oracle, simd_cases):
    # the committed expected values are reproducible from the committed sequences
    for c in simd_cases[::7]:
        cfg = oracle_cfg_of(oracle, c)
        for a, b, s, e1, e2 in list(zip(c["seqs1"], c["seqs2"], c["oracle_scores"], c["oracle_end1"],
                                        c["oracle_end2"]))[:8]:
            assert oracle.align(cfg, a.encode(), b.encode()) == (s, e1, e2)


def test_simd_port_matches_scalar_on_reference_cases(oracle, simd_cases):
    from pairwise_aligner_gb300.aligner import pack
    checked = 0
    for c in simd_cases:
        if c["method"] == "global" and (c["last_column"] == "free" or c["last_row"] == "free"):
            continue                    # the SIMD port times the penalised-trailing / local paths only
        cfg = oracle_cfg_of(oracle, c)
        s1, o1 = pack(c["seqs1"])
        s2, o2 = pack(c["seqs2"])
        got = oracle.simd_batch(cfg, s1, o1, s2, o2, nthreads=2)
        assert list(got) == c["oracle_scores"], c["name"]
        checked += 1
    assert checked >= 30


def test_batch_matches_single(oracle, simd_cases):
    from pairwise_aligner_gb300.aligner import pack
    c = simd_cases[3]
    cfg = oracle_cfg_of(oracle, c)
    s1, o1 = pack(c["seqs1"])
    s2, o2 = pack(c["seqs2"])
    sc, e1, e2 = oracle.align_batch(cfg, s1, o1, s2, o2, nthreads=3)
    assert list(sc) == c["oracle_scores"]
    assert list(e1) == c["oracle_end1"] and list(e2) == c["oracle_end2"]


def test_local_end_tie_break(oracle):
    cfg = oracle.make_cfg(1, -1, -2, -1, local=True)
    # two equal maximal cells: (2,2) and (4,2) / (2,4) ... the smallest i wins, then the smallest j
    assert oracle.align(cfg, b"AAXAA", b"AA") == (2, 2, 2)
    assert oracle.align(cfg, b"AA", b"AAXAA") == (2, 2, 2)
    assert oracle.align(cfg, b"C", b"G") == (0, 0, 0)          # score 0 -> (0, 0)
    assert oracle.align(cfg, b"", b"G") == (-2**31, 0, 0)      # empty -> lowest(), (0, 0)


def test_global_free_end_coordinates(oracle):
    # overlap: best cell may end inside the last row / column
    cfg = oracle.make_cfg(4, -5, -10, -1, first_column_free=True, first_row_free=True, last_column_free=True,
                          last_row_free=True)
    sc, e1, e2 = oracle.align(cfg, b"TTTTTCTGACACACT", b"CTGCACACGACGGGGGG")
    assert sc == 16
    assert 0 <= e1 <= 15 and 0 <= e2 <= 17 and (e1 == 15 or e2 == 17)
    std = oracle.make_cfg(4, -5, -10, -1)
    assert oracle.align(std, b"ACGT", b"ACGT") == (16, 4, 4)
    assert oracle.align(std, b"", b"ACG") == (-13, 0, 3)        # H(0, n) = open + 3 * ext
    assert oracle.align(std, b"ACG", b"") == (-13, 3, 0)


@pytest.mark.parametrize("local", [False, True])
def test_oracle_symmetry(oracle, local):
    rng = np.random.default_rng(7)
    cfg = oracle.make_cfg(2, -3, -5, -1, local=local)
    for _ in range(20):
        a = rng.choice(list(b"ACGT"), size=int(rng.integers(1, 40))).astype(np.uint8).tobytes()
        b = rng.choice(list(b"ACGT"), size=int(rng.integers(1, 40))).astype(np.uint8).tobytes()
        assert oracle.align(cfg, a, b)[0] == oracle.align(cfg, b, a)[0]


def test_simd_port_matches_scalar_on_random_configs(oracle):
    """The timed CPU port (int16x8 lanes, int32x4 lanes where int16 could overflow) equals the
    scalar restatement across score models, methods and lengths."""
    from pairwise_aligner_gb300.aligner import pack
    rng = np.random.default_rng(31)
    acgt = np.frombuffer(b"ACGT", dtype=np.uint8)
    for trial in range(24):
        match, mismatch = int(rng.integers(1, 6)), int(-rng.integers(1, 7))
        go, ge = int(-rng.integers(0, 11)), int(-rng.integers(1, 4))
        local = bool(trial % 2)
        fc, fr = (False, False) if local else (bool(rng.integers(0, 2)), bool(rng.integers(0, 2)))
        cfg = oracle.make_cfg(match, mismatch, go, ge, local=local, first_column_free=fc, first_row_free=fr)
        long_pairs = trial % 3 == 0                       # lengths that push some pairs to int32 lanes
        lens = rng.integers(0, 3000 if long_pairs else 300, size=(40, 2))
        s1, s2 = [], []
        for m, n in lens:
            a = acgt[rng.integers(0, 4, int(m))]
            b = a[: int(n)].copy() if rng.random() < 0.5 else acgt[rng.integers(0, 4, int(n))]
            b = np.concatenate([b, acgt[rng.integers(0, 4, max(0, int(n) - len(b)))]])
            flip = rng.random(len(b)) < 0.1
            b[flip] = acgt[rng.integers(0, 4, int(flip.sum()))]
            s1.append(a.tobytes())
            s2.append(b.tobytes())
        q, qo = pack(s1)
        t, to = pack(s2)
        got = oracle.simd_batch(cfg, q, qo, t, to, nthreads=4)
        want, _, _ = oracle.align_batch(cfg, q, qo, t, to, nthreads=4)
        assert list(got) == list(want), (trial, match, mismatch, go, ge, local, fc, fr)


@pytest.mark.parametrize("byte_lanes", [True, False])
def test_simd_port_lane_widths_match_scalar(oracle, simd_cases, byte_lanes):
    """Local cases through the byte lanes (the reference's saturated int8 width) and through
    int16 lanes only: both equal the scalar restatement; the byte lanes really run."""
    from pairwise_aligner_gb300.aligner import pack
    ran8 = 0
    for c in simd_cases:
        if c["method"] != "local":
            continue
        cfg = oracle_cfg_of(oracle, c)
        s1, o1 = pack(c["seqs1"])
        s2, o2 = pack(c["seqs2"])
        counts = [0, 0, 0]
        got = oracle.simd_batch(cfg, s1, o1, s2, o2, nthreads=2, byte_lanes=byte_lanes, counts=counts)
        assert list(got) == c["oracle_scores"], c["name"]
        assert sum(counts) <= len(got) and (byte_lanes or counts[0] == 0)
        ran8 += counts[0]
    assert (ran8 > 0) == byte_lanes


def test_byte_lanes_redo_saturated_pairs_exactly(oracle):
    """Pairs whose local score passes the byte range (long identical runs, large match scores)
    are redone in wider lanes; scores still equal the scalar oracle."""
    from pairwise_aligner_gb300.aligner import pack
    rng = np.random.default_rng(41)
    acgt = np.frombuffer(b"ACGT", dtype=np.uint8)
    for match in (1, 3, 100):
        cfg = oracle.make_cfg(match, -4, -6, -1, local=True)
        s1, s2 = [], []
        for k in range(48):
            n = int(rng.integers(0, 700))
            a = acgt[rng.integers(0, 4, n)]
            b = a.copy() if k % 3 == 0 else acgt[rng.integers(0, 4, int(rng.integers(0, 700)))]
            s1.append(a.tobytes())
            s2.append(b.tobytes())
        s1.append(b"ACGTN")                           # a non-ACGT byte: wider lanes
        s2.append(b"ACGTN")
        q, qo = pack(s1)
        t, to = pack(s2)
        counts = [0, 0, 0]
        got = oracle.simd_batch(cfg, q, qo, t, to, nthreads=3, counts=counts)
        want, _, _ = oracle.align_batch(cfg, q, qo, t, to, nthreads=3)
        assert list(got) == list(want), match
        assert counts[1] + counts[2] > 0, counts      # saturated or non-ACGT pairs went wider
        assert counts[0] > 0 or match == 100, counts   # with match 100 nearly every lane saturates
