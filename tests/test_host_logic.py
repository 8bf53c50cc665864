"""Host-side logic that needs no GPU: argument checks before any device call, the
configuration rules, and the C ABI entry points that are host code (2-bit packing, the
sequence-file reader, status strings)."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest


def _conf(**kw):
    c = dict(local=False, match=2, mismatch=-3, gap_open=-5, gap_extension=-1, first_column_free=False,
             first_row_free=False, last_column_free=False, last_row_free=False)
    c.update(kw)
    return c


def test_batch_shapes_are_checked_before_the_device():
    from pairwise_aligner_gb300 import Aligner, pack
    al = Aligner(_conf())
    q, qo = pack([b"ACGT", b"AC"])
    t, to = pack([b"ACGT"])
    with pytest.raises(ValueError):
        al.compute_arrays(q, qo, t, to)
    with pytest.raises(ValueError):
        al.compute_packed(np.zeros(1, np.uint32), qo, np.zeros(1, np.uint32), to)
    w = np.zeros(1, np.uint32)                    # 16 bases, but the offsets need 17
    with pytest.raises(ValueError):
        al.compute_packed(w, np.array([0, 17], np.uint64), w, np.array([0, 3], np.uint64))
    with pytest.raises(ValueError):
        al.compute_traceback_arrays(q, qo, t, to)
    with pytest.raises(ValueError):
        al.compute_arrays(q, qo, q, qo, out=np.zeros(1, dtype=np.int32))


def test_method_flags_of_the_config():
    from pairwise_aligner_gb300 import Aligner, _lib, cfg
    assert Aligner(_conf()).c_config().method == _lib.PA_METHOD_GLOBAL
    assert Aligner(_conf(local=True)).c_config().method == _lib.PA_METHOD_LOCAL
    c = Aligner(cfg.fold(cfg.band_learned(cfg.method_global(cfg.gap_model_affine(cfg.score_model_unitary(1, -4),
                                                                                   -6, -1))))).c_config()
    assert (c.band_mode, c.match, c.mismatch, c.gap_open, c.gap_extension) == (1, 1, -4, -6, -1)
    c = Aligner(cfg.fold(cfg.width(cfg.method_local(cfg.gap_model_affine(cfg.score_model_unitary(1, -1), -1, -1)),
                                   32))).c_config()
    assert c.width_hint == 32 and c.first_row_free and c.last_column_free == 1


def test_rule_errors_follow_the_reference():
    from pairwise_aligner_gb300 import cfg
    with pytest.raises(TypeError):
        cfg.fold(cfg.method_global(cfg.gap_model_affine(-1, -1)))                # no score model
    with pytest.raises(TypeError):
        cfg.fold(cfg.method_global(cfg.score_model_unitary(1, -1)))             # no gap model
    with pytest.raises(TypeError):
        cfg.fold(cfg.method_local(cfg.method_global(cfg.gap_model_affine(cfg.score_model_unitary(1, -1), -1, -1))))
    with pytest.raises(TypeError):
        cfg.gap_model_affine(1, 2, 3, 4)


def test_host_abi_entry_points(built_lib):
    from pairwise_aligner_gb300 import _lib
    lib = _lib.load()
    for code, name in _lib.STATUS.items():
        assert lib.pa_status_string(code)
    assert lib.pa_abi_version() >= 1
    bad = ctypes.c_uint64()
    assert lib.pa_pack_2bit_host(None, 5, None, ctypes.byref(bad)) == 1           # null buffers
    assert lib.pa_pack_2bit_host(None, 0, None, ctypes.byref(bad)) == 0 and bad.value == 0
    h = ctypes.c_void_p()
    assert lib.pa_seqfile_parse(None, 0, ctypes.byref(h), None, 0) == 0            # empty text: no records
    assert lib.pa_seqfile_count(h) == 0
    lib.pa_seqfile_free(h)
    assert lib.pa_seqfile_read(b"/nonexistent/reads.fq", ctypes.byref(h), None, 0) == 1
    assert lib.pa_seqfile_count(None) == 0 and lib.pa_seqfile_name(None, 0) is None
