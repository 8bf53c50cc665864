"""Traceback: the optimal alignment as begin cell + SAM-style ops.

CPU: the oracle's traceback agrees with its own score DP (score and end cell), its ops
consume exactly the symbols between begin and end, and rescoring the ops gives the score
(global with every end-gap combination, local, a substitution matrix).  GPU: the
kernel's begin cell and ops equal the oracle's byte for byte, its score and end cell
equal pa_align_batch's, on the reference's differential pairs, random pairs of every
shape class (several passes of 256 rows, empty sequences) and a BLOSUM62 matrix.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import matrix_of, oracle_cfg_of

ACGT = np.frombuffer(b"ACGT", dtype=np.uint8)
END_GAPS = [(0, 0, 0, 0), (1, 0, 0, 1), (0, 1, 1, 0), (1, 1, 1, 1), (0, 0, 1, 1), (1, 1, 0, 0)]


def _random_pairs(rng, count, max_len, alphabet=ACGT, related=0.5):
    s1, s2 = [], []
    for _ in range(count):
        a = alphabet[rng.integers(0, len(alphabet), int(rng.integers(0, max_len + 1)))]
        if rng.random() < related and len(a):
            b = a.copy()
            flip = rng.random(len(b)) < 0.15
            b[flip] = alphabet[rng.integers(0, len(alphabet), int(flip.sum()))]
            b = b[rng.random(len(b)) > 0.05]
            cut = int(rng.integers(0, max(1, len(b) // 4)))
            b = b[cut:]
        else:
            b = alphabet[rng.integers(0, len(alphabet), int(rng.integers(0, max_len + 1)))]
        s1.append(a.tobytes())
        s2.append(b.tobytes())
    return s1, s2


def _check_oracle_path(oracle, cfg, a, b):
    sc, b1, b2, e1, e2, ops = oracle.traceback(cfg, a, b)
    assert (sc, e1, e2) == oracle.align(cfg, a, b)
    if cfg.local and (not a or not b or sc <= 0):
        assert ops == b"" and (b1, b2, e1, e2) == (0, 0, 0, 0)
        return
    assert b1 + sum(c in b"=XD" for c in ops) == e1 and b2 + sum(c in b"=XI" for c in ops) == e2
    for c, x, y in _columns(a, b, b1, b2, ops):
        assert (c == "=") == (x == y) if c in "=X" else True
    assert oracle.rescore(cfg, a, b, b1, b2, ops) == sc


def _columns(a, b, i, j, ops):
    for c in ops.decode():
        if c in "=X":
            yield c, a[i], b[j]
            i += 1
            j += 1
        elif c == "D":
            i += 1
        else:
            j += 1


@pytest.mark.parametrize("local", [False, True])
@pytest.mark.parametrize("gaps", END_GAPS)
def test_oracle_traceback_is_consistent(oracle, local, gaps):
    rng = np.random.default_rng(1 + 7 * local + sum(g << k for k, g in enumerate(gaps)))
    for match, mismatch, go, ge in ((2, -3, -5, -1), (1, -4, -6, -1), (3, -1, 0, -2)):
        cfg = oracle.make_cfg(match, mismatch, go, ge, local=local, first_column_free=gaps[0],
                              first_row_free=gaps[1], last_column_free=gaps[2], last_row_free=gaps[3])
        for a, b in zip(*_random_pairs(rng, 40, 40)):
            _check_oracle_path(oracle, cfg, a, b)


def test_oracle_traceback_with_a_matrix(oracle, matrix_kats):
    sym, scores = matrix_of(matrix_kats["matrices"]["blosum62_standard"])
    alphabet = np.frombuffer(sym, dtype=np.uint8)
    rng = np.random.default_rng(3)
    for local in (False, True):
        cfg = oracle.make_cfg(0, 0, -10, -1, local=local, matrix=(sym, scores))
        for a, b in zip(*_random_pairs(rng, 60, 50, alphabet=alphabet)):
            _check_oracle_path(oracle, cfg, a, b)


def test_oracle_traceback_known_paths(oracle):
    """Hand-checked alignments of the tie-break convention."""
    g = oracle.make_cfg(2, -3, -5, -1)
    assert oracle.traceback(g, b"ACGT", b"ACGT")[5] == b"===="
    assert oracle.traceback(g, b"ACGT", b"AGT") == (2 + 2 + 2 - 6, 0, 0, 4, 3, b"=D==")
    assert oracle.traceback(g, b"", b"ACG")[5] == b"III"
    lo = oracle.make_cfg(2, -3, -5, -1, local=True)
    assert oracle.traceback(lo, b"TTACGTTT", b"GGACGGG") == (6, 2, 2, 5, 5, b"===")


def test_cigar_strings():
    from pairwise_aligner_gb300 import cigar
    assert cigar(b"") == "" and cigar(b"===XDDI=") == "3=1X2D1I1="


# -- GPU ------------------------------------------------------------------------------------------

@pytest.fixture(scope="module")
def pa(built_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import pairwise_aligner_gb300 as pa
    return pa


def _gpu_vs_oracle(pa, oracle, conf, s1, s2, matrix=None):
    from pairwise_aligner_gb300 import pack
    q, qo = pack(s1)
    t, to = pack(s2)
    al = pa.Aligner(dict(conf, matrix=matrix) if matrix else conf)
    res, aln, ops, ops_off = al.compute_traceback_arrays(q, qo, t, to)
    plain = al.compute_arrays(q, qo, t, to)
    for f in ("score", "end1", "end2"):
        assert np.array_equal(res[f], plain[f]), f
    cfg = oracle.make_cfg(conf["match"], conf["mismatch"], conf["gap_open"], conf["gap_extension"],
                          local=conf["local"], first_column_free=conf["first_column_free"],
                          first_row_free=conf["first_row_free"], last_column_free=conf["last_column_free"],
                          last_row_free=conf["last_row_free"], matrix=matrix)
    for k, (a, b) in enumerate(zip(s1, s2)):
        sc, b1, b2, e1, e2, want = oracle.traceback(cfg, a, b)
        got = ops[int(ops_off[k]):int(ops_off[k]) + int(aln[k]["n_ops"])].tobytes()
        assert (int(res[k]["score"]), int(aln[k]["begin1"]), int(aln[k]["begin2"]), int(res[k]["end1"]),
                int(res[k]["end2"]), got) == (sc, b1, b2, e1, e2, want), (k, a, b)


def _conf(local=False, gaps=(0, 0, 0, 0), match=2, mismatch=-3, gap_open=-5, gap_extension=-1):
    return dict(local=local, match=match, mismatch=mismatch, gap_open=gap_open, gap_extension=gap_extension,
                first_column_free=bool(gaps[0] or local), first_row_free=bool(gaps[1] or local),
                last_column_free=bool(gaps[2] and not local), last_row_free=bool(gaps[3] and not local))


@pytest.mark.gpu
@pytest.mark.parametrize("local", [False, True])
@pytest.mark.parametrize("gaps", END_GAPS)
def test_traceback_matches_oracle_random(pa, oracle, local, gaps):
    rng = np.random.default_rng(11 + 3 * local + sum(g << k for k, g in enumerate(gaps)))
    s1, s2 = _random_pairs(rng, 300, 300)
    s1 += [b"", b"ACGT", b"", b"A", b"T" * 600]
    s2 += [b"", b"", b"ACG", b"A", b"T" * 300 + b"G" * 290]
    _gpu_vs_oracle(pa, oracle, _conf(local, gaps), s1, s2)


@pytest.mark.gpu
@pytest.mark.parametrize("params", [(1, -4, -6, -1), (3, -1, 0, -2), (5, -4, -10, -1)])
def test_traceback_multi_pass_pairs(pa, oracle, params):
    """Sequence2 longer than one pass of 256 rows (up to 4 passes), both methods."""
    rng = np.random.default_rng(12)
    s1, s2 = _random_pairs(rng, 24, 900)
    for local in (False, True):
        _gpu_vs_oracle(pa, oracle, _conf(local, (0, 0, 0, 0), *params), s1, s2)


@pytest.mark.gpu
def test_traceback_reference_differential_pairs(pa, oracle, simd_cases):
    checked = 0
    for c in simd_cases[::3]:
        conf = _conf(c["method"] == "local",
                     tuple(int(c[k] == "free") for k in ("first_column", "first_row", "last_column", "last_row")),
                     c["match"], c["mismatch"], c["gap_open"], c["gap_extension"])
        _gpu_vs_oracle(pa, oracle, conf, [s.encode() for s in c["seqs1"]], [s.encode() for s in c["seqs2"]])
        checked += 1
    assert checked >= 25


@pytest.mark.gpu
def test_traceback_with_blosum62(pa, oracle, matrix_kats):
    sym, scores = matrix_of(matrix_kats["matrices"]["blosum62_standard"])
    alphabet = np.frombuffer(sym, dtype=np.uint8)
    rng = np.random.default_rng(13)
    s1, s2 = _random_pairs(rng, 200, 400, alphabet=alphabet)
    for local in (False, True):
        _gpu_vs_oracle(pa, oracle, _conf(local, (0, 0, 0, 0), 0, 0, -10, -1), s1, s2, matrix=(sym, scores))


@pytest.mark.gpu
def test_traceback_reference_kats_through_rules(pa, kats, oracle):
    """The reference's scalar known answers: the traceback's score is the KAT and its ops rescore to it."""
    from conftest import rule_of
    for c in kats:
        al = pa.cfg.configure_aligner(rule_of(c))
        r = al.compute_traceback([c["seq1"]], [c["seq2"]])[0]
        assert r.score() == c["expected_score"], (c["source"], c["name"])
        if r.ops():
            cfg = oracle_cfg_of(oracle, c)
            b1, b2 = r.begin_position()
            assert oracle.rescore(cfg, c["seq1"].encode(), c["seq2"].encode(), b1, b2, r.ops()) == r.score()


def _all_alignments(a: bytes, b: bytes):
    """Every op string aligning all of a with all of b (small inputs only)."""
    if not a and not b:
        yield ""
        return
    if a and b:
        for rest in _all_alignments(a[1:], b[1:]):
            yield ("=" if a[0] == b[0] else "X") + rest
    if a:
        for rest in _all_alignments(a[1:], b):
            yield "D" + rest
    if b:
        for rest in _all_alignments(a, b[1:]):
            yield "I" + rest


def test_oracle_traceback_is_optimal_by_enumeration(oracle):
    """Global (penalised ends) and local paths against the best of all alignments, enumerated."""
    rng = np.random.default_rng(21)
    for match, mismatch, go, ge in ((2, -3, -5, -1), (1, -1, 0, -1), (3, -2, -4, -2)):
        g = oracle.make_cfg(match, mismatch, go, ge)
        lo = oracle.make_cfg(match, mismatch, go, ge, local=True)
        for _ in range(25):
            a = ACGT[rng.integers(0, 4, int(rng.integers(0, 5)))].tobytes()
            b = ACGT[rng.integers(0, 4, int(rng.integers(0, 5)))].tobytes()
            best = max(oracle.rescore(g, a, b, 0, 0, ops.encode()) for ops in _all_alignments(a, b))
            sc, b1, b2, e1, e2, ops = oracle.traceback(g, a, b)
            assert sc == best and (b1, b2, e1, e2) == (0, 0, len(a), len(b))
            assert oracle.rescore(g, a, b, 0, 0, ops) == best
            if a and b:                                 # local: the best over all substring pairs
                lbest = max(oracle.rescore(lo, a[i:k], b[j:l], 0, 0, ops.encode())
                            for i in range(len(a)) for k in range(i + 1, len(a) + 1)
                            for j in range(len(b)) for l in range(j + 1, len(b) + 1)
                            for ops in _all_alignments(a[i:k], b[j:l]))
                sc, b1, b2, e1, e2, ops = oracle.traceback(lo, a, b)
                assert sc == max(lbest, 0)
                if sc > 0:
                    assert oracle.rescore(lo, a, b, b1, b2, ops) == sc
