"""ctypes front of the CPU oracle (oracle/pa_oracle.c).

TEST INFRASTRUCTURE ONLY: the checker the GPU path is compared with.  Only
tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline / reference
legs import this module.  The product package never does.

The C file restates the reference's scalar path (see its header for the
file:line citations); this module only builds and loads it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "pa_oracle.c")
_SRC_BYTES = os.path.join(_HERE, "pa_oracle_bytes.cpp")
_LIB = os.path.join(_HERE, "liboracle.so")
_lock = threading.Lock()
_lib = None


class OracleCfg(ctypes.Structure):
    _fields_ = [
        ("match", ctypes.c_int32),
        ("mismatch", ctypes.c_int32),
        ("gap_open", ctypes.c_int32),
        ("gap_extension", ctypes.c_int32),
        ("local", ctypes.c_int32),
        ("first_column_free", ctypes.c_int32),
        ("first_row_free", ctypes.c_int32),
        ("last_column_free", ctypes.c_int32),
        ("last_row_free", ctypes.c_int32),
        ("dim", ctypes.c_int32),
        ("matrix", ctypes.POINTER(ctypes.c_int32)),
        ("rank", ctypes.POINTER(ctypes.c_int16)),
    ]


def build(force: bool = False) -> str:
    """Compile oracle/pa_oracle.c and pa_oracle_bytes.cpp into oracle/liboracle.so (portable
    flags, no -march)."""
    with _lock:
        newest = max(os.path.getmtime(_SRC), os.path.getmtime(_SRC_BYTES))
        if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < newest:
            obj = _LIB + f".bytes{os.getpid()}.o"
            warn = ["-Wall", "-Wextra", "-Wno-psabi", "-fPIC"]
            subprocess.check_call(["g++", "-O3", "-std=c++17", *warn, "-c", _SRC_BYTES, "-o", obj])
            try:
                subprocess.check_call(["gcc", "-O3", "-std=c11", *warn, "-shared", "-pthread", _SRC, obj,
                                       "-o", _LIB + ".tmp"])
            finally:
                os.remove(obj)
            os.replace(_LIB + ".tmp", _LIB)
    return _LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB)
        u8p = ctypes.POINTER(ctypes.c_uint8)
        u64p = ctypes.POINTER(ctypes.c_uint64)
        i64p = ctypes.POINTER(ctypes.c_int64)
        i32p = ctypes.POINTER(ctypes.c_int32)
        L.pa_oracle_align.argtypes = [ctypes.POINTER(OracleCfg), u8p, ctypes.c_uint64, u8p, ctypes.c_uint64,
                                      i64p, i64p, i64p]
        L.pa_oracle_align.restype = ctypes.c_int
        L.pa_oracle_align_batch.argtypes = [ctypes.POINTER(OracleCfg), u8p, u64p, u8p, u64p, ctypes.c_uint64,
                                            i64p, i64p, i64p, ctypes.c_int]
        L.pa_oracle_align_batch.restype = ctypes.c_int
        L.pa_oracle_row.argtypes = [ctypes.POINTER(OracleCfg), u8p, ctypes.c_uint64, u8p, ctypes.c_uint64,
                                    ctypes.c_uint64, i64p]
        L.pa_oracle_row.restype = ctypes.c_int
        L.pa_oracle_simd_batch.argtypes = [ctypes.POINTER(OracleCfg), u8p, u64p, u8p, u64p, ctypes.c_uint64,
                                           i32p, ctypes.c_int]
        L.pa_oracle_simd_batch.restype = ctypes.c_int
        L.pa_oracle_simd_batch_lanes.argtypes = [ctypes.POINTER(OracleCfg), u8p, u64p, u8p, u64p, ctypes.c_uint64,
                                                 i32p, ctypes.c_int, ctypes.c_int, u64p]
        L.pa_oracle_simd_batch_lanes.restype = ctypes.c_int
        L.pa_oracle_traceback.argtypes = [ctypes.POINTER(OracleCfg), u8p, ctypes.c_uint64, u8p, ctypes.c_uint64,
                                          i64p, i64p, i64p, i64p, i64p, u8p, i64p]
        L.pa_oracle_traceback.restype = ctypes.c_int
        _lib = L
    return _lib


def make_cfg(match, mismatch, gap_open, gap_extension, local=False, first_column_free=False,
             first_row_free=False, last_column_free=False, last_row_free=False, matrix=None) -> OracleCfg:
    """`matrix`: optional substitution matrix as (symbols, dim x dim scores) -- row = sequence1 symbol."""
    cfg = OracleCfg(int(match), int(mismatch), int(gap_open), int(gap_extension), int(bool(local)),
                    int(bool(first_column_free)), int(bool(first_row_free)), int(bool(last_column_free)),
                    int(bool(last_row_free)), 0, None, None)
    if matrix is not None:
        symbols, scores = matrix
        dim = len(symbols)
        rank = np.full(256, -1, dtype=np.int16)
        for r, sym in enumerate(symbols):
            rank[sym if isinstance(sym, int) else ord(sym)] = r
        mat = np.ascontiguousarray(np.asarray(scores, dtype=np.int32).reshape(dim, dim))
        cfg.dim = dim
        cfg.matrix = _ptr(mat, ctypes.c_int32)
        cfg.rank = _ptr(rank, ctypes.c_int16)
        cfg._keep = (mat, rank)                     # the arrays live as long as the config
    return cfg


def _ptr(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


def align(cfg: OracleCfg, s1: bytes, s2: bytes):
    """One pair -> (score, end1, end2)."""
    a = np.frombuffer(bytes(s1), dtype=np.uint8) if len(s1) else np.zeros(1, np.uint8)
    b = np.frombuffer(bytes(s2), dtype=np.uint8) if len(s2) else np.zeros(1, np.uint8)
    sc, e1, e2 = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    rc = lib().pa_oracle_align(ctypes.byref(cfg), _ptr(a, ctypes.c_uint8), len(s1), _ptr(b, ctypes.c_uint8),
                               len(s2), ctypes.byref(sc), ctypes.byref(e1), ctypes.byref(e2))
    if rc:
        raise RuntimeError(f"pa_oracle_align failed: {rc}")
    return sc.value, e1.value, e2.value


def align_batch(cfg: OracleCfg, s1: np.ndarray, off1: np.ndarray, s2: np.ndarray, off2: np.ndarray,
                nthreads: int | None = None):
    """Batch over concatenated bytes + (n_pairs+1) uint64 offsets -> (scores, end1, end2) int64 arrays."""
    n = len(off1) - 1
    s1 = np.ascontiguousarray(s1, dtype=np.uint8)
    s2 = np.ascontiguousarray(s2, dtype=np.uint8)
    off1 = np.ascontiguousarray(off1, dtype=np.uint64)
    off2 = np.ascontiguousarray(off2, dtype=np.uint64)
    if s1.size == 0:
        s1 = np.zeros(1, np.uint8)
    if s2.size == 0:
        s2 = np.zeros(1, np.uint8)
    scores = np.empty(n, np.int64)
    e1 = np.empty(n, np.int64)
    e2 = np.empty(n, np.int64)
    nt = nthreads or os.cpu_count() or 1
    rc = lib().pa_oracle_align_batch(ctypes.byref(cfg), _ptr(s1, ctypes.c_uint8), _ptr(off1, ctypes.c_uint64),
                                     _ptr(s2, ctypes.c_uint8), _ptr(off2, ctypes.c_uint64), n,
                                     _ptr(scores, ctypes.c_int64), _ptr(e1, ctypes.c_int64),
                                     _ptr(e2, ctypes.c_int64), nt)
    if rc:
        raise RuntimeError(f"pa_oracle_align_batch failed: {rc}")
    return scores, e1, e2


def simd_batch(cfg: OracleCfg, s1, off1, s2, off2, nthreads: int | None = None, byte_lanes: bool = True,
               counts: list | None = None) -> np.ndarray:
    """Inter-sequence SIMD port (scores only) -- the timed CPU baseline.  Local alignment of
    A/C/G/T pairs runs in 16 byte lanes (``byte_lanes``), the rest in 8 int16 or 4 int32 lanes;
    ``counts`` (a list) receives the pairs finished at each width [byte, int16, int32]."""
    n = len(off1) - 1
    s1 = np.ascontiguousarray(s1, dtype=np.uint8)
    s2 = np.ascontiguousarray(s2, dtype=np.uint8)
    off1 = np.ascontiguousarray(off1, dtype=np.uint64)
    off2 = np.ascontiguousarray(off2, dtype=np.uint64)
    scores = np.empty(max(n, 1), np.int32)
    cnt = np.zeros(3, np.uint64)
    nt = nthreads or os.cpu_count() or 1
    rc = lib().pa_oracle_simd_batch_lanes(ctypes.byref(cfg), _ptr(s1, ctypes.c_uint8), _ptr(off1, ctypes.c_uint64),
                                          _ptr(s2, ctypes.c_uint8), _ptr(off2, ctypes.c_uint64), n,
                                          _ptr(scores, ctypes.c_int32), nt, int(bool(byte_lanes)),
                                          _ptr(cnt, ctypes.c_uint64))
    if rc:
        raise RuntimeError(f"pa_oracle_simd_batch_lanes failed: {rc}")
    if counts is not None:
        counts[:] = [int(v) for v in cnt]
    return scores[:n]


def row(cfg: OracleCfg, s1: bytes, s2: bytes, r: int) -> np.ndarray:
    """H(r, 0..n) of the global recurrence."""
    a = np.frombuffer(bytes(s1), dtype=np.uint8) if len(s1) else np.zeros(1, np.uint8)
    b = np.frombuffer(bytes(s2), dtype=np.uint8) if len(s2) else np.zeros(1, np.uint8)
    out = np.empty(len(s2) + 1, np.int64)
    rc = lib().pa_oracle_row(ctypes.byref(cfg), _ptr(a, ctypes.c_uint8), len(s1), _ptr(b, ctypes.c_uint8), len(s2),
                             r, _ptr(out, ctypes.c_int64))
    if rc:
        raise RuntimeError(f"pa_oracle_row failed: {rc}")
    return out


def traceback(cfg: OracleCfg, s1: bytes, s2: bytes):
    """One pair -> (score, begin1, begin2, end1, end2, ops) with ops a bytes string of '=', 'X',
    'I', 'D' in path order (the conventions are in pa_oracle_traceback's comment)."""
    a = np.frombuffer(bytes(s1), dtype=np.uint8) if len(s1) else np.zeros(1, np.uint8)
    b = np.frombuffer(bytes(s2), dtype=np.uint8) if len(s2) else np.zeros(1, np.uint8)
    ops = np.zeros(len(s1) + len(s2) + 1, dtype=np.uint8)
    v = [ctypes.c_int64() for _ in range(6)]
    rc = lib().pa_oracle_traceback(ctypes.byref(cfg), _ptr(a, ctypes.c_uint8), len(s1), _ptr(b, ctypes.c_uint8),
                                   len(s2), *[ctypes.byref(x) for x in v[:5]], _ptr(ops, ctypes.c_uint8),
                                   ctypes.byref(v[5]))
    if rc:
        raise RuntimeError(f"pa_oracle_traceback failed: {rc}")
    return v[0].value, v[1].value, v[2].value, v[3].value, v[4].value, ops[:v[5].value].tobytes()


def rescore(cfg: OracleCfg, s1: bytes, s2: bytes, begin1: int, begin2: int, ops: bytes) -> int:
    """Score of an op string: substitutions plus open + ext * length per maximal gap run.  With a
    free leading gap the begin offset costs nothing; a penalised leading gap is part of the ops."""
    i, j, total, run = begin1, begin2, 0, None
    for op in ops.decode():
        if op in "=X":
            a, b = s1[i], s2[j]
            if cfg.dim:
                rank = cfg._keep[1]
                total += int(cfg._keep[0][rank[a], rank[b]])
            else:
                total += cfg.match if a == b else cfg.mismatch
            i += 1
            j += 1
            run = None
        else:
            total += cfg.gap_extension + (cfg.gap_open if run != op else 0)
            run = op
            if op == "D":
                i += 1
            else:
                j += 1
    return total


def band_labels(cfg: OracleCfg, s1: bytes, s2: bytes) -> list[int]:
    """The 8 checkpoint diagonals of the optimal global path, as the GPU labeller defines them:
    checkpoint rows r_c = (c+1)*m//9; label = argmax_j (H(r_c, j) + H_rev(m - r_c, n - j)) - r_c,
    j in 0..n-1, smallest j on ties."""
    m, n = len(s1), len(s2)
    if m < 9 or n == 0:
        return [0] * 8
    rs1, rs2 = bytes(s1)[::-1], bytes(s2)[::-1]
    out = []
    for c in range(8):
        r = (c + 1) * m // 9
        hf = row(cfg, s1, s2, r)
        hr = row(cfg, rs1, rs2, m - r)
        tot = hf[:n] + hr[n - np.arange(n)]
        out.append(int(np.argmax(tot)) - r)
    return out


# -- input path -----------------------------------------------------------------------------------

def rank_table(symbols: bytes) -> np.ndarray:
    """The reference's alphabet_rank_map_scalar (alphabet_conversion/alphabet_rank_map_scalar.hpp):
    a 256-entry table, -1 everywhere, then rank r written for symbols[r] in list order (a repeated
    symbol keeps its last rank).  An empty list is an error, as alphabet_rank_map_simd throws
    std::invalid_argument for it (alphabet_rank_map_simd.hpp:61-63)."""
    if len(symbols) == 0:
        raise ValueError("the given set of valid symbols is empty")
    tab = np.full(256, -1, dtype=np.int8)
    for r, b in enumerate(bytes(symbols)):
        tab[b] = r
    return tab


def rank_map(symbols: bytes, data: np.ndarray) -> np.ndarray:
    """Ranks of every byte of `data` (int8, -1 for a byte that is not a symbol)."""
    return rank_table(symbols)[np.asarray(data, dtype=np.uint8)]


def pack_2bit(data: np.ndarray) -> tuple[np.ndarray, int]:
    """2-bit DNA packing restated with numpy: base i at bits 2(i mod 16) of word i // 16, code
    ((b >> 1) ^ (b >> 2)) & 3 (A/a 0, C/c 1, G/g 2, T/t 3); returns (words, count of bytes whose
    b | 0x20 is not one of a c g t)."""
    b = np.asarray(data, dtype=np.uint8)
    n = len(b)
    code = (((b >> 1) ^ (b >> 2)) & 3).astype(np.uint32)
    pad = np.zeros((-n) % 16, dtype=np.uint32)
    c = np.concatenate([code, pad]).reshape(-1, 16)
    words = (c << (2 * np.arange(16, dtype=np.uint32))).sum(axis=1, dtype=np.uint64).astype(np.uint32)
    lower = b | 0x20
    bad = int(np.count_nonzero(~np.isin(lower, np.frombuffer(b"acgt", dtype=np.uint8))))
    return words, bad
