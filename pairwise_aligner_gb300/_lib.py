"""ctypes binding of the C ABI in include/pairwise_aligner_gb300.h (libpa_gb300.so).

The shared library is built in-tree by ``pairwise_aligner_gb300.build``.  There is
no CPU fallback: if the library is missing or no CUDA device is present, the
calls raise.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libpa_gb300.so")

PA_METHOD_GLOBAL = 0
PA_METHOD_LOCAL = 1
PA_SCORE_MATRIX = 0x100      # or-ed into PaConfig.method: score with the context's substitution matrix

STATUS = {
    0: "PA_OK", 1: "PA_ERR_INVALID_ARGUMENT", 2: "PA_ERR_CUDA", 3: "PA_ERR_OUT_OF_MEMORY",
    4: "PA_ERR_OVERFLOW", 5: "PA_ERR_UNSUPPORTED", 6: "PA_ERR_TIMEOUT", 7: "PA_ERR_NO_DEVICE",
    8: "PA_ERR_TOO_LARGE",
}

RESULT_RERUN, RESULT_BANDED, RESULT_FULL_DP, RESULT_TRIVIAL, RESULT_OVERFLOW, RESULT_ERROR = 0x01, 0x02, 0x04, 0x08, 0x10, 0x20


class PaConfig(ctypes.Structure):
    _fields_ = [
        ("method", ctypes.c_int32),
        ("match", ctypes.c_int32),
        ("mismatch", ctypes.c_int32),
        ("gap_open", ctypes.c_int32),
        ("gap_extension", ctypes.c_int32),
        ("first_column_free", ctypes.c_uint8),
        ("first_row_free", ctypes.c_uint8),
        ("last_column_free", ctypes.c_uint8),
        ("last_row_free", ctypes.c_uint8),
        ("width_hint", ctypes.c_int32),
        ("band_mode", ctypes.c_int32),
    ]


class PaResult(ctypes.Structure):
    _fields_ = [
        ("score", ctypes.c_int32),
        ("end1", ctypes.c_int32),
        ("end2", ctypes.c_int32),
        ("width", ctypes.c_uint8),
        ("flags", ctypes.c_uint8),
        ("band_rounds", ctypes.c_uint16),
    ]


class PaAlignment(ctypes.Structure):
    _fields_ = [
        ("begin1", ctypes.c_int32),
        ("begin2", ctypes.c_int32),
        ("n_ops", ctypes.c_uint32),
        ("reserved", ctypes.c_uint32),
    ]


class PaOptions(ctypes.Structure):
    _fields_ = [
        ("group_threads", ctypes.c_int32),
        ("rows_per_thread", ctypes.c_int32),
        ("blocks_per_sm", ctypes.c_int32),
        ("use_graphs", ctypes.c_int32),
        ("autotune", ctypes.c_int32),
        ("kernel_variant", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 2),
    ]


class PaStats(ctypes.Structure):
    _fields_ = [
        ("pairs", ctypes.c_uint64),
        ("cells", ctypes.c_uint64),
        ("pairs_s16", ctypes.c_uint64),
        ("pairs_s32", ctypes.c_uint64),
        ("pairs_general", ctypes.c_uint64),
        ("pairs_rerun", ctypes.c_uint64),
        ("pairs_trivial", ctypes.c_uint64),
        ("kernel_launches", ctypes.c_uint64),
        ("device_ms", ctypes.c_double),
        ("dp_ms", ctypes.c_double),
        ("pairs_banded", ctypes.c_uint64),
        ("pairs_full_dp", ctypes.c_uint64),
        ("band_cells", ctypes.c_uint64),
        ("band_rounds", ctypes.c_uint64),
    ]


class PaBandOptions(ctypes.Structure):
    _fields_ = [
        ("margin", ctypes.c_float),
        ("w_min", ctypes.c_int32),
        ("straight_w0", ctypes.c_int32),
        ("full_frac", ctypes.c_float),
        ("max_rounds", ctypes.c_int32),
        ("team_full_frac", ctypes.c_float),
        ("reserved", ctypes.c_int32 * 2),
    ]


TUNE_SIZES, TUNE_SHAPES = 5, 4          # PA_TUNE_SIZES, PA_TUNE_SHAPES


class PaTuneEntry(ctypes.Structure):
    _fields_ = [
        ("variant", ctypes.c_int16),
        ("group_threads", ctypes.c_int16),
        ("dp_ms", ctypes.c_float),
    ]


class PaTuning(ctypes.Structure):
    _fields_ = [
        ("variant_s16", ctypes.c_int32 * 2),
        ("variant_s32", ctypes.c_int32 * 2),
        ("group_threads_s16", ctypes.c_int32 * 2),
        ("group_threads_s32", ctypes.c_int32 * 2),
        ("best_ms", ctypes.c_double * 2),
        ("s16", PaTuneEntry * TUNE_SHAPES * TUNE_SIZES * 2),
    ]


def tuning_to_dict(t: PaTuning) -> dict:
    """A PaTuning as plain lists (the s16 table as [method][size class][pair-size class] dicts)."""
    out = {name: list(getattr(t, name)) for name in ("variant_s16", "variant_s32", "group_threads_s16",
                                                      "group_threads_s32", "best_ms")}
    out["s16"] = [[[{"variant": e.variant, "group_threads": e.group_threads, "dp_ms": e.dp_ms} for e in row]
                   for row in m] for m in t.s16]
    return out


def tuning_from_dict(d: dict) -> PaTuning:
    t = PaTuning()
    for name in ("variant_s16", "variant_s32", "group_threads_s16", "group_threads_s32", "best_ms"):
        getattr(t, name)[:] = d[name]
    for mi, m in enumerate(d.get("s16", [])):
        for a, row in enumerate(m):
            for b, e in enumerate(row):
                t.s16[mi][a][b].variant = int(e["variant"])
                t.s16[mi][a][b].group_threads = int(e["group_threads"])
                t.s16[mi][a][b].dp_ms = float(e["dp_ms"])
    return t


class PaRoofline(ctypes.Structure):
    _fields_ = [
        ("s16x2_cells_per_s", ctypes.c_double),
        ("s32_cells_per_s", ctypes.c_double),
        ("sm_clock_mhz", ctypes.c_double),
        ("sm_count", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("s16x2_local_cells_per_s", ctypes.c_double),
    ]


# Every symbol include/pairwise_aligner_gb300.h declares, with its ctypes signature.
_u8p = ctypes.POINTER(ctypes.c_uint8)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_ctxp = ctypes.c_void_p
SIGNATURES = {
    "pa_create": ([ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.POINTER(PaOptions)], ctypes.c_int),
    "pa_destroy": ([_ctxp], ctypes.c_int),
    "pa_align_batch": ([_ctxp, ctypes.POINTER(PaConfig), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                        ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.POINTER(PaStats)], ctypes.c_int),
    "pa_align_batch_device": ([_ctxp, ctypes.POINTER(PaConfig), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                               ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p,
                               ctypes.c_void_p, ctypes.POINTER(PaStats)], ctypes.c_int),
    "pa_align_batch_device_static": ([ctypes.POINTER(PaConfig), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                                      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64,
                                      ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "pa_align_one_to_many": ([_ctxp, ctypes.POINTER(PaConfig), ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p,
                              ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.POINTER(PaStats)],
                             ctypes.c_int),
    "pa_measure_roofline": ([_ctxp, ctypes.POINTER(PaRoofline)], ctypes.c_int),
    "pa_autotune": ([_ctxp, ctypes.POINTER(PaConfig), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                     ctypes.c_void_p, ctypes.c_uint64, ctypes.POINTER(PaTuning)], ctypes.c_int),
    "pa_band_labels": ([_ctxp, ctypes.POINTER(PaConfig), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                        ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p], ctypes.c_int),
    "pa_band_features_device": ([ctypes.c_void_p] * 4 + [ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p],
                                 ctypes.c_int),
    "pa_mlp_gemm": ([ctypes.c_void_p] * 5 + [ctypes.c_int] * 9 + [ctypes.c_float, ctypes.c_void_p], ctypes.c_int),
    "pa_mlp_mse": ([ctypes.c_void_p] * 3 + [ctypes.c_int] + [ctypes.c_void_p] * 3, ctypes.c_int),
    "pa_mlp_relu_grad": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p], ctypes.c_int),
    "pa_mlp_colsum": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "pa_mlp_adam": ([ctypes.c_void_p] * 5 + [ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                              ctypes.c_float, ctypes.c_int, ctypes.c_float, ctypes.c_void_p],
                    ctypes.c_int),
    "pa_mlp_to_bf16": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p],
                       ctypes.c_int),
    "pa_set_cta_threshold": ([_ctxp, ctypes.c_uint64], ctypes.c_int),
    "pa_set_cluster_threshold": ([_ctxp, ctypes.c_uint64, ctypes.c_uint32], ctypes.c_int),
    "pa_set_team_threshold": ([_ctxp, ctypes.c_uint32], ctypes.c_int),
    "pa_set_wait_limit": ([_ctxp, ctypes.c_uint32], ctypes.c_int),
    "pa_get_graph_count": ([_ctxp, ctypes.POINTER(ctypes.c_uint32)], ctypes.c_int),
    "pa_set_band_options": ([_ctxp, ctypes.POINTER(PaBandOptions)], ctypes.c_int),
    "pa_get_band_options": ([_ctxp, ctypes.POINTER(PaBandOptions)], ctypes.c_int),
    "pa_set_band_model": ([_ctxp] + [ctypes.c_void_p] * 6, ctypes.c_int),
    "pa_set_substitution_matrix": ([_ctxp, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p], ctypes.c_int),
    "pa_align_batch_banded": ([_ctxp, ctypes.POINTER(PaConfig), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                               ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p,
                               ctypes.POINTER(PaStats)], ctypes.c_int),
    "pa_traceback_batch": ([_ctxp, ctypes.POINTER(PaConfig), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                            ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                            ctypes.POINTER(PaStats)], ctypes.c_int),
    "pa_rank_map_device": ([_ctxp, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint64,
                            ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)], ctypes.c_int),
    "pa_pack_2bit_host": ([ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)],
                          ctypes.c_int),
    "pa_pack_2bit_device": ([_ctxp, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p,
                             ctypes.POINTER(ctypes.c_uint64)], ctypes.c_int),
    "pa_unpack_2bit_device": ([_ctxp, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p,
                               ctypes.c_void_p], ctypes.c_int),
    "pa_align_batch_packed": ([_ctxp, ctypes.POINTER(PaConfig), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                               ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.POINTER(PaStats)],
                              ctypes.c_int),
    "pa_seqfile_read": ([ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p, ctypes.c_size_t],
                        ctypes.c_int),
    "pa_seqfile_parse": ([ctypes.c_char_p, ctypes.c_uint64, ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p,
                          ctypes.c_size_t], ctypes.c_int),
    "pa_seqfile_count": ([ctypes.c_void_p], ctypes.c_uint64),
    "pa_seqfile_sequences": ([ctypes.c_void_p], ctypes.c_void_p),
    "pa_seqfile_offsets": ([ctypes.c_void_p], ctypes.c_void_p),
    "pa_seqfile_qualities": ([ctypes.c_void_p], ctypes.c_void_p),
    "pa_seqfile_name": ([ctypes.c_void_p, ctypes.c_uint64], ctypes.c_char_p),
    "pa_seqfile_free": ([ctypes.c_void_p], None),
    "pa_get_tuning": ([_ctxp, ctypes.POINTER(PaTuning)], ctypes.c_int),
    "pa_set_tuning": ([_ctxp, ctypes.POINTER(PaTuning)], ctypes.c_int),
    "pa_status_string": ([ctypes.c_int], ctypes.c_char_p),
    "pa_last_error": ([_ctxp], ctypes.c_char_p),
    "pa_abi_version": ([], ctypes.c_int),
}

_lib = None


class PaError(RuntimeError):
    """A non-OK pa_status; mirrors the reference's std::runtime_error."""

    def __init__(self, status: int, message: str = ""):
        self.status = status
        super().__init__(f"{STATUS.get(status, status)}: {message}" if message else STATUS.get(status, str(status)))


def load(path: str | None = None):
    """Load libpa_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise OSError(f"{p} is missing: build it with pairwise_aligner_gb300.build.build() "
                      "(there is no CPU fallback)")
    lib = ctypes.CDLL(p)
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if path is None:
        _lib = lib
    return lib


def check(status: int, ctx=None):
    if status != 0:
        msg = ""
        if ctx is not None:
            raw = load().pa_last_error(ctx)
            msg = raw.decode() if raw else ""
        raise PaError(status, msg)
