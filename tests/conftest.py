"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU."""
from __future__ import annotations

import gzip
import json
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)
GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libpa_gb300.so")


@pytest.fixture(scope="session")
def kats():
    with open(os.path.join(GOLDEN, "kat_scalar.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def matrix_kats():
    """The reference's substitution-matrix known answers and their matrices."""
    with open(os.path.join(GOLDEN, "kat_matrix.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def matrix_cases():
    """The reference's substitution-matrix SIMD differential cases with oracle results."""
    with gzip.open(os.path.join(GOLDEN, "matrix_differential.json.gz"), "rt") as f:
        return json.load(f)


def matrix_of(m: dict):
    """(symbols bytes, flat dim*dim scores) of a golden-fixture matrix."""
    return "".join(m["symbols"]).encode(), [x for row in m["scores"] for x in row]


@pytest.fixture(scope="session")
def simd_cases():
    with gzip.open(os.path.join(GOLDEN, "simd_differential.json.gz"), "rt") as f:
        return json.load(f)


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def built_lib():
    from pairwise_aligner_gb300 import build
    return build.build()


def oracle_cfg_of(O, c: dict, matrix=None):
    """Oracle configuration from a golden-fixture case (`matrix`: (symbols, scores) or None)."""
    return O.make_cfg(c["match"], c["mismatch"], c["gap_open"], c["gap_extension"], local=c["method"] == "local",
                      first_column_free=c["first_column"] == "free", first_row_free=c["first_row"] == "free",
                      last_column_free=c["last_column"] == "free", last_row_free=c["last_row"] == "free",
                      matrix=matrix)


def rule_of(c: dict, matrix_pairs=None):
    """The cfg rule chain of a golden-fixture case, written like the reference's tests
    (`matrix_pairs`: the (symbol, row) list of cfg.score_model_matrix, or None)."""
    from pairwise_aligner_gb300 import cfg
    if c["method"] == "local":
        base = cfg.method_local(cfg.gap_model_affine(c["gap_open"], c["gap_extension"]))
    else:
        e = cfg.end_gap
        lead = cfg.leading_end_gap(first_column=e.free if c["first_column"] == "free" else e.penalised,
                                   first_row=e.free if c["first_row"] == "free" else e.penalised)
        trail = cfg.trailing_end_gap(last_column=e.free if c["last_column"] == "free" else e.penalised,
                                     last_row=e.free if c["last_row"] == "free" else e.penalised)
        base = cfg.method_global(cfg.gap_model_affine(c["gap_open"], c["gap_extension"]), lead, trail)
    if matrix_pairs is not None:
        return cfg.score_model_matrix(base, matrix_pairs)
    return cfg.score_model_unitary_gpu(base, c["match"], c["mismatch"])
