"""Bit-exact parity at the benchmark sizes: every result against the oracle.

The reference pins its SIMD paths by the differential property "SIMD lane ==
scalar aligner" on seeded random pairs
(test/unit/affine/alignment_simd_test_template.hpp:195-227).  Here that
property is checked at the full sizes of the benchmark workloads: every score
and end position of the CUDA path equals the scalar oracle's (oracle/pa_oracle.c,
all host threads), for

* all 262,144 pairs of the local workload (64-512 bp, +1/-4, open 6 / extend 1);
* all 8,192 long-read pairs of the global workload, at the default block / team /
  cluster routing;
* a stratified sample of the mixed global stream with at least 40 very long pairs
  (20-50 kb plus structural indels);
* the 16,384 held-out pairs of the learned-band workload, plain and in band
  mode 1 with the shipped predictor (band mode may only change speed, never a score).
"""
from __future__ import annotations

import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pa(built_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import pairwise_aligner_gb300 as pa
    return pa


def _conf(d, band_mode=0):
    free = bool(d["local"])
    return dict(local=d["local"], match=d["match"], mismatch=d["mismatch"], gap_open=d["gap_open"],
                gap_extension=d["gap_extension"], first_column_free=free, first_row_free=free,
                last_column_free=free, last_row_free=free, width_hint=0, band_mode=band_mode)


def _assert_exact(oracle, d, res):
    oc = oracle.make_cfg(d["match"], d["mismatch"], d["gap_open"], d["gap_extension"], local=d["local"])
    sc, e1, e2 = oracle.align_batch(oc, d["seq1"], d["off1"], d["seq2"], d["off2"], nthreads=os.cpu_count())
    bad = np.flatnonzero((res["score"] != sc) | (res["end1"] != e1) | (res["end2"] != e2))
    assert len(bad) == 0, (f"{len(bad)} of {len(sc)} differ; first {bad[:5]}: gpu {res[bad[:5]]} "
                           f"oracle {list(zip(sc[bad[:5]], e1[bad[:5]], e2[bad[:5]]))}")


def test_every_local_pair_of_the_262144_pair_batch(pa, oracle):
    from pairwise_aligner_gb300 import workloads as W
    from pairwise_aligner_gb300.aligner import Aligner
    d = W.config2()
    al = Aligner(_conf(d))
    res = al.compute_arrays(d["seq1"], d["off1"], d["seq2"], d["off2"])
    assert len(res) == 262144
    _assert_exact(oracle, d, res)


def test_every_long_read_pair_of_the_8192_pair_batch(pa, oracle):
    from pairwise_aligner_gb300 import workloads as W
    from pairwise_aligner_gb300.aligner import Aligner
    d = W.config3()
    al = Aligner(_conf(d))
    res = al.compute_arrays(d["seq1"], d["off1"], d["seq2"], d["off2"])
    assert len(res) == 8192
    _assert_exact(oracle, d, res)


def test_mixed_stream_stratified_sample_with_very_long_pairs(pa, oracle):
    from pairwise_aligner_gb300 import workloads as W
    from pairwise_aligner_gb300.aligner import Aligner
    d = W.config5(seed=55, n_pairs=4096, strata=(0.86, 0.12, 0.02))
    assert (d["stratum"] == 2).sum() >= 40
    al = Aligner(_conf(d))
    res = al.compute_arrays(d["seq1"], d["off1"], d["seq2"], d["off2"])
    _assert_exact(oracle, d, res)


@pytest.mark.parametrize("band_mode", [0, 1])
def test_learned_band_eval_set_plain_and_banded(pa, oracle, band_mode):
    import torch
    from pairwise_aligner_gb300 import band as BD
    from pairwise_aligner_gb300 import workloads as W
    from pairwise_aligner_gb300.aligner import Aligner
    d = W.config4(seed=424242, n_pairs=16384)
    ctx = pa.Context(0)
    if band_mode == 1:
        model = BD.BandModel(device=torch.device("cuda:0"))
        model.load(os.path.join(os.path.dirname(pa.__file__), "data", "band_model.npz"))
        model.to_context(ctx)
    al = Aligner(_conf(d, band_mode), context=ctx)
    res = al.compute_arrays(d["seq1"], d["off1"], d["seq2"], d["off2"])
    _assert_exact(oracle, d, res)
