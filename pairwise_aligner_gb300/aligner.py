"""The aligner object returned by ``cfg.configure_aligner`` and its results.

Mirrors the reference's interface objects:
  * ``compute(seqs1, seqs2)`` -> list of results, like
    interface_one_to_one_bulk::compute (interface/interface_one_to_one_bulk.hpp:47-100),
    without the "<= lane count" limit (:55-57);
  * ``compute(seq1, seqs2)`` with a single first sequence -> one-to-many
    (interface/interface_one_to_many_bulk.hpp:47-92);
  * ``compute(seq1, seq2)`` with two single sequences -> one result
    (interface/interface_one_to_one_single.hpp:44-67).
Results expose ``score()``, ``sequence1()``, ``sequence2()`` like
aligner_result_bulk (result/aligner_result_bulk.hpp:43-69), plus
``end_position()``.

Bulk callers that hold their sequences as concatenated bytes + offsets use
``compute_arrays`` (host numpy) or ``compute_device`` (device tensors).
"""
from __future__ import annotations

import ctypes
from typing import Sequence

import numpy as np

from . import _lib


def pack(seqs: Sequence) -> tuple[np.ndarray, np.ndarray]:
    """Concatenate str/bytes sequences -> (uint8 bytes, uint64 offsets of length n+1)."""
    raw = [s.encode() if isinstance(s, str) else bytes(s) for s in seqs]
    lens = np.fromiter((len(r) for r in raw), dtype=np.uint64, count=len(raw))
    off = np.zeros(len(raw) + 1, dtype=np.uint64)
    np.cumsum(lens, out=off[1:])
    data = np.frombuffer(b"".join(raw), dtype=np.uint8) if raw else np.zeros(0, np.uint8)
    return data, off


class Context:
    """Owns one pa_ctx (CUDA stream, device buffers, graph cache) on one device."""

    def __init__(self, device: int = 0, group_threads: int = 0, blocks_per_sm: int = 0, use_graphs: int = 0,
                 kernel_variant: int = -1):
        self.lib = _lib.load()
        self.ptr = ctypes.c_void_p()
        opt = _lib.PaOptions()
        opt.group_threads = group_threads
        opt.blocks_per_sm = blocks_per_sm
        opt.use_graphs = use_graphs
        opt.kernel_variant = kernel_variant
        _lib.check(self.lib.pa_create(ctypes.byref(self.ptr), int(device), ctypes.byref(opt)))
        self.device = device

    def close(self):
        if self.ptr:
            self.lib.pa_destroy(self.ptr)
            self.ptr = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_cta_threshold(self, cells: int):
        """Pairs with at least `cells` m*n cells run on whole thread blocks (1: all pairs)."""
        _lib.check(self.lib.pa_set_cta_threshold(self.ptr, int(cells)), self.ptr)

    def set_cluster_threshold(self, cells: int, min_rows: int = 8192):
        """Of the block-mode pairs, those with at least `cells` cells and `min_rows` rows run on clusters."""
        _lib.check(self.lib.pa_set_cluster_threshold(self.ptr, int(cells), int(min_rows)), self.ptr)

    def set_team_threshold(self, max_rows: int):
        """Block-mode pairs whose sequence2 has at most `max_rows` rows run on 4-warp teams (0: none)."""
        _lib.check(self.lib.pa_set_team_threshold(self.ptr, int(max_rows)), self.ptr)

    def graph_count(self) -> int:
        """Calls this context keeps captured as CUDA graphs (at most 8)."""
        n = ctypes.c_uint32()
        _lib.check(self.lib.pa_get_graph_count(self.ptr, ctypes.byref(n)), self.ptr)
        return n.value

    def set_wait_limit(self, polls: int):
        """Polls a CTA-mode progress wait makes before it gives up (default 2^24; 0: at the first look)."""
        _lib.check(self.lib.pa_set_wait_limit(self.ptr, int(polls)), self.ptr)

    def set_substitution_matrix(self, symbols: bytes, scores):
        """Load the matrix that PA_SCORE_MATRIX calls score with: scores[r1 * dim + r2] for a
        sequence1 symbol of rank r1 (its index in `symbols`) against a sequence2 symbol of rank r2."""
        sym = np.frombuffer(bytes(symbols), dtype=np.uint8).copy()
        sc = np.ascontiguousarray(np.asarray(scores, dtype=np.int64).reshape(-1))
        if sc.size != sym.size * sym.size or np.abs(sc).max(initial=0) > (1 << 20):
            raise ValueError("scores must hold dim * dim values in [-2^20, 2^20]")
        sc = sc.astype(np.int32)
        _lib.check(self.lib.pa_set_substitution_matrix(self.ptr, sym.ctypes.data, int(sym.size), sc.ctypes.data),
                   self.ptr)
        self._matrix = (bytes(symbols), tuple(int(x) for x in sc))

    # -- band mode ----------------------------------------------------------------
    def band_options(self) -> dict:
        o = _lib.PaBandOptions()
        _lib.check(self.lib.pa_get_band_options(self.ptr, ctypes.byref(o)), self.ptr)
        return {name: getattr(o, name) for name, _ in _lib.PaBandOptions._fields_ if name != "reserved"}

    def set_band_options(self, **kw):
        o = _lib.PaBandOptions()
        _lib.check(self.lib.pa_get_band_options(self.ptr, ctypes.byref(o)), self.ptr)
        for k, v in kw.items():
            setattr(o, k, v)
        _lib.check(self.lib.pa_set_band_options(self.ptr, ctypes.byref(o)), self.ptr)

    def set_band_model(self, state: dict):
        """Load the band predictor (FP32 arrays W1 144x256, b1, W2 256x256, b2, W3 256x16, b3 16)."""
        shapes = {"W1": (144, 256), "b1": (256,), "W2": (256, 256), "b2": (256,), "W3": (256, 16), "b3": (16,)}
        arrs = []
        for k, shp in shapes.items():
            a = np.ascontiguousarray(state[k], dtype=np.float32)
            if a.shape != shp:
                raise ValueError(f"{k} must have shape {shp}, got {a.shape}")
            arrs.append(a)
        _lib.check(self.lib.pa_set_band_model(self.ptr, *[a.ctypes.data for a in arrs]), self.ptr)
        self._band_model = arrs          # keep the host copies alive with the context

    # -- kernel choices -------------------------------------------------------
    def tuning(self) -> dict:
        """Kernel choices: per-method defaults and the s16x2 table [method][size class][pair-size class]."""
        t = _lib.PaTuning()
        _lib.check(self.lib.pa_get_tuning(self.ptr, ctypes.byref(t)), self.ptr)
        return _lib.tuning_to_dict(t)

    def set_tuning(self, tuning: dict):
        t = _lib.tuning_from_dict(tuning)
        _lib.check(self.lib.pa_set_tuning(self.ptr, ctypes.byref(t)), self.ptr)

    def autotune(self, c_config, seq1, off1, seq2, off2) -> dict:
        """Time the kernel candidates on this batch and keep the fastest in the table entry of
        the batch's method, batch-size class and pair-size class."""
        seq1 = np.ascontiguousarray(seq1, dtype=np.uint8)
        seq2 = np.ascontiguousarray(seq2, dtype=np.uint8)
        off1 = np.ascontiguousarray(off1, dtype=np.uint64)
        off2 = np.ascontiguousarray(off2, dtype=np.uint64)
        t = _lib.PaTuning()
        _lib.check(self.lib.pa_autotune(self.ptr, ctypes.byref(c_config), seq1.ctypes.data, off1.ctypes.data,
                                        seq2.ctypes.data, off2.ctypes.data, len(off1) - 1, ctypes.byref(t)),
                   self.ptr)
        return _lib.tuning_to_dict(t)

    def save_tuning(self, path: str):
        import json
        with open(path, "w") as f:
            json.dump(self.tuning(), f, indent=1)

    def load_tuning(self, path: str):
        import json
        with open(path) as f:
            self.set_tuning(json.load(f))

    def roofline(self) -> dict:
        r = _lib.PaRoofline()
        _lib.check(self.lib.pa_measure_roofline(self.ptr, ctypes.byref(r)), self.ptr)
        return {"s16x2_cells_per_s": r.s16x2_cells_per_s, "s32_cells_per_s": r.s32_cells_per_s,
                "sm_clock_mhz": r.sm_clock_mhz, "sm_count": r.sm_count,
                "s16x2_local_cells_per_s": r.s16x2_local_cells_per_s}


RESULT_DTYPE = np.dtype([("score", np.int32), ("end1", np.int32), ("end2", np.int32), ("width", np.uint8),
                         ("flags", np.uint8), ("band_rounds", np.uint16)])
assert RESULT_DTYPE.itemsize == ctypes.sizeof(_lib.PaResult)


ALIGNMENT_DTYPE = np.dtype([("begin1", np.int32), ("begin2", np.int32), ("n_ops", np.uint32), ("reserved", np.uint32)])
assert ALIGNMENT_DTYPE.itemsize == ctypes.sizeof(_lib.PaAlignment)


def cigar(ops: bytes) -> str:
    """Run-length form of an op string ('=', 'X', 'I', 'D'), e.g. b'==XI' -> '2=1X1I'."""
    out, prev, run = [], None, 0
    for c in ops.decode() if isinstance(ops, (bytes, bytearray)) else ops:
        if c == prev:
            run += 1
        else:
            if prev is not None:
                out.append(f"{run}{prev}")
            prev, run = c, 1
    if prev is not None:
        out.append(f"{run}{prev}")
    return "".join(out)


class AlignerResult:
    """One alignment result (score only, plus the end position)."""

    __slots__ = ("_seq1", "_seq2", "_score", "_end", "_width", "_flags")

    def __init__(self, seq1, seq2, score, end1, end2, width, flags):
        self._seq1, self._seq2 = seq1, seq2
        self._score, self._end = int(score), (int(end1), int(end2))
        self._width, self._flags = int(width), int(flags)

    def score(self) -> int:
        return self._score

    def sequence1(self):
        return self._seq1

    def sequence2(self):
        return self._seq2

    def end_position(self) -> tuple[int, int]:
        """1-based (end in sequence1, end in sequence2); ties to the smallest first, then second."""
        return self._end

    def width(self) -> int:
        return self._width

    def flags(self) -> int:
        return self._flags

    def __repr__(self):
        return f"AlignerResult(score={self._score}, end={self._end})"


class AlignmentResult(AlignerResult):
    """A result with its alignment (``Aligner.compute_traceback``)."""

    __slots__ = ("_begin", "_ops")

    def __init__(self, seq1, seq2, score, end1, end2, width, flags, begin1, begin2, ops):
        super().__init__(seq1, seq2, score, end1, end2, width, flags)
        self._begin = (int(begin1), int(begin2))
        self._ops = bytes(ops)

    def begin_position(self) -> tuple[int, int]:
        """0-based cell the path starts after (symbols of sequence1 / sequence2 before it)."""
        return self._begin

    def ops(self) -> bytes:
        """One byte per alignment column: '=', 'X', 'D' (sequence1 only), 'I' (sequence2 only)."""
        return self._ops

    def cigar(self) -> str:
        return cigar(self._ops)

    def __repr__(self):
        return f"AlignmentResult(score={self._score}, begin={self._begin}, end={self._end}, cigar={self.cigar()!r})"


class Aligner:
    """Configured aligner; see the module docstring."""

    def __init__(self, config: dict, device: int = 0, context: Context | None = None):
        self.config = dict(config)
        self.device = device
        self._ctx = context
        self.last_stats: dict | None = None

    # -- plumbing -----------------------------------------------------------
    @property
    def context(self) -> Context:
        if self._ctx is None:
            self._ctx = Context(self.device)
        mat = self.config.get("matrix")
        if mat is not None and getattr(self._ctx, "_matrix", None) != mat:
            self._ctx.set_substitution_matrix(*mat)       # a context holds one matrix at a time
        return self._ctx

    def c_config(self) -> _lib.PaConfig:
        c = self.config
        method = _lib.PA_METHOD_LOCAL if c["local"] else _lib.PA_METHOD_GLOBAL
        if c.get("matrix") is not None:
            method |= _lib.PA_SCORE_MATRIX
        return _lib.PaConfig(
            method, c["match"], c["mismatch"],
            c["gap_open"], c["gap_extension"], int(c["first_column_free"]), int(c["first_row_free"]),
            int(c["last_column_free"]), int(c["last_row_free"]), int(c.get("width_hint", 0)),
            int(c.get("band_mode", 0)))

    @staticmethod
    def _stats_dict(st: _lib.PaStats) -> dict:
        return {name: getattr(st, name) for name, _ in _lib.PaStats._fields_}

    # -- bulk entry points ----------------------------------------------------
    def compute_arrays(self, seq1: np.ndarray, off1: np.ndarray, seq2: np.ndarray, off2: np.ndarray,
                       stats: bool = True, out: np.ndarray | None = None) -> np.ndarray:
        """Host arrays in, structured result array (RESULT_DTYPE) out.  Synchronous.

        `out` (RESULT_DTYPE, at least n_pairs long, ideally in pinned memory) receives the results
        instead of a newly allocated array."""
        n = len(off1) - 1
        if len(off2) - 1 != n:
            raise ValueError("both sequence collections must hold the same number of sequences")
        seq1 = np.ascontiguousarray(seq1, dtype=np.uint8)
        seq2 = np.ascontiguousarray(seq2, dtype=np.uint8)
        off1 = np.ascontiguousarray(off1, dtype=np.uint64)
        off2 = np.ascontiguousarray(off2, dtype=np.uint64)
        if out is None:
            out = np.zeros(max(n, 1), dtype=RESULT_DTYPE)
        elif out.dtype != RESULT_DTYPE or len(out) < n or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous RESULT_DTYPE array of at least n_pairs entries")
        st = _lib.PaStats()
        ctx = self.context
        cfg = self.c_config()
        rc = ctx.lib.pa_align_batch(ctx.ptr, ctypes.byref(cfg), seq1.ctypes.data, off1.ctypes.data,
                                    seq2.ctypes.data, off2.ctypes.data, n, out.ctypes.data,
                                    ctypes.byref(st) if stats else None)
        _lib.check(rc, ctx.ptr)
        if stats:
            self.last_stats = self._stats_dict(st)
        return out[:n]

    def compute_packed(self, words1: np.ndarray, off1: np.ndarray, words2: np.ndarray, off2: np.ndarray,
                       stats: bool = True, out: np.ndarray | None = None) -> np.ndarray:
        """As compute_arrays, for 2-bit packed DNA (``seqio.pack_2bit``): offsets count bases."""
        n = len(off1) - 1
        if len(off2) - 1 != n:
            raise ValueError("both sequence collections must hold the same number of sequences")
        words1 = np.ascontiguousarray(words1, dtype=np.uint32)
        words2 = np.ascontiguousarray(words2, dtype=np.uint32)
        off1 = np.ascontiguousarray(off1, dtype=np.uint64)
        off2 = np.ascontiguousarray(off2, dtype=np.uint64)
        for w, o in ((words1, off1), (words2, off2)):
            if n and len(w) * 16 < int(o[-1]):
                raise ValueError("the packed words end before the last offset")
        if out is None:
            out = np.zeros(max(n, 1), dtype=RESULT_DTYPE)
        elif out.dtype != RESULT_DTYPE or len(out) < n or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous RESULT_DTYPE array of at least n_pairs entries")
        st = _lib.PaStats()
        ctx = self.context
        cfg = self.c_config()
        rc = ctx.lib.pa_align_batch_packed(ctx.ptr, ctypes.byref(cfg), words1.ctypes.data, off1.ctypes.data,
                                           words2.ctypes.data, off2.ctypes.data, n, out.ctypes.data,
                                           ctypes.byref(st) if stats else None)
        _lib.check(rc, ctx.ptr)
        if stats:
            self.last_stats = self._stats_dict(st)
        return out[:n]

    def compute_traceback_arrays(self, seq1: np.ndarray, off1: np.ndarray, seq2: np.ndarray, off2: np.ndarray):
        """Host arrays in -> (results RESULT_DTYPE, alignments ALIGNMENT_DTYPE, ops uint8, ops offsets);
        pair k's ops are ops[ops_off[k] : ops_off[k] + alignments[k]['n_ops']]."""
        n = len(off1) - 1
        if len(off2) - 1 != n:
            raise ValueError("both sequence collections must hold the same number of sequences")
        seq1 = np.ascontiguousarray(seq1, dtype=np.uint8)
        seq2 = np.ascontiguousarray(seq2, dtype=np.uint8)
        off1 = np.ascontiguousarray(off1, dtype=np.uint64)
        off2 = np.ascontiguousarray(off2, dtype=np.uint64)
        out = np.zeros(max(n, 1), dtype=RESULT_DTYPE)
        aln = np.zeros(max(n, 1), dtype=ALIGNMENT_DTYPE)
        ops_off = (off1 - off1[0]) + (off2 - off2[0]) if n else np.zeros(1, np.uint64)
        ops = np.zeros(max(int(ops_off[-1]), 1), dtype=np.uint8)
        st = _lib.PaStats()
        ctx = self.context
        cfg = self.c_config()
        rc = ctx.lib.pa_traceback_batch(ctx.ptr, ctypes.byref(cfg), seq1.ctypes.data, off1.ctypes.data,
                                        seq2.ctypes.data, off2.ctypes.data, n, out.ctypes.data, aln.ctypes.data,
                                        ops.ctypes.data, ctypes.byref(st))
        _lib.check(rc, ctx.ptr)
        self.last_stats = self._stats_dict(st)
        return out[:n], aln[:n], ops, ops_off[:n]

    def compute_traceback(self, seqs1, seqs2) -> list:
        """Like compute(seqs1, seqs2), with the alignment of every pair (AlignmentResult)."""
        seqs1, seqs2 = list(seqs1), list(seqs2)
        s1, o1 = pack(seqs1)
        s2, o2 = pack(seqs2)
        res, aln, ops, ops_off = self.compute_traceback_arrays(s1, o1, s2, o2)
        return [AlignmentResult(a, b, r["score"], r["end1"], r["end2"], r["width"], r["flags"], g["begin1"],
                                g["begin2"], ops[int(o):int(o) + int(g["n_ops"])].tobytes())
                for a, b, r, g, o in zip(seqs1, seqs2, res, aln, ops_off)]

    def compute_banded(self, seq1: np.ndarray, off1: np.ndarray, seq2: np.ndarray, off2: np.ndarray,
                       bands: np.ndarray) -> np.ndarray:
        """Band mode with caller-given bands: (n_pairs, 10) int32 rows diag[8], w_start, w_min."""
        n = len(off1) - 1
        seq1 = np.ascontiguousarray(seq1, dtype=np.uint8)
        seq2 = np.ascontiguousarray(seq2, dtype=np.uint8)
        off1 = np.ascontiguousarray(off1, dtype=np.uint64)
        off2 = np.ascontiguousarray(off2, dtype=np.uint64)
        bands = np.ascontiguousarray(bands, dtype=np.int32).reshape(n, 10)
        out = np.zeros(max(n, 1), dtype=RESULT_DTYPE)
        st = _lib.PaStats()
        ctx = self.context
        cfg = self.c_config()
        rc = ctx.lib.pa_align_batch_banded(ctx.ptr, ctypes.byref(cfg), seq1.ctypes.data, off1.ctypes.data,
                                           seq2.ctypes.data, off2.ctypes.data, n, bands.ctypes.data, out.ctypes.data,
                                           ctypes.byref(st))
        _lib.check(rc, ctx.ptr)
        self.last_stats = self._stats_dict(st)
        return out[:n]

    def compute_device(self, seq1, off1, seq2, off2, out, stream=None, stats: bool = False):
        """Device tensors (torch, uint8 / int64 / a 16-byte-per-pair result buffer) in and out.

        Asynchronous on ``stream`` (a torch.cuda.Stream or raw handle) unless stats=True."""
        n = off1.numel() - 1
        st = _lib.PaStats()
        ctx = self.context
        cfg = self.c_config()
        handle = getattr(stream, "cuda_stream", stream)
        if stream is not None and not handle:
            handle = 1          # cudaStreamLegacy: torch's default stream
        handle = handle or None
        rc = ctx.lib.pa_align_batch_device(ctx.ptr, ctypes.byref(cfg), seq1.data_ptr(), off1.data_ptr(),
                                           seq1.numel(), seq2.data_ptr(), off2.data_ptr(), seq2.numel(), n,
                                           out.data_ptr(), handle, ctypes.byref(st) if stats else None)
        _lib.check(rc, ctx.ptr)
        if stats:
            self.last_stats = self._stats_dict(st)
        return out

    # -- reference-shaped entry point ------------------------------------------
    def compute(self, seqs1, seqs2):
        single1 = isinstance(seqs1, (str, bytes, bytearray))
        single2 = isinstance(seqs2, (str, bytes, bytearray))
        if single1 and single2:
            return self.compute([seqs1], [seqs2])[0]
        if single1:
            return self._one_to_many(seqs1, list(seqs2))
        seqs1, seqs2 = list(seqs1), list(seqs2)
        s1, o1 = pack(seqs1)
        s2, o2 = pack(seqs2)
        res = self.compute_arrays(s1, o1, s2, o2)
        return [AlignerResult(a, b, r["score"], r["end1"], r["end2"], r["width"], r["flags"])
                for a, b, r in zip(seqs1, seqs2, res)]

    def _one_to_many(self, query, targets):
        q = query.encode() if isinstance(query, str) else bytes(query)
        qa = np.frombuffer(q, dtype=np.uint8) if q else np.zeros(1, np.uint8)
        s2, o2 = pack(targets)
        n = len(targets)
        out = np.zeros(max(n, 1), dtype=RESULT_DTYPE)
        st = _lib.PaStats()
        ctx = self.context
        cfg = self.c_config()
        rc = ctx.lib.pa_align_one_to_many(ctx.ptr, ctypes.byref(cfg), qa.ctypes.data, len(q), s2.ctypes.data,
                                          o2.ctypes.data, n, out.ctypes.data, ctypes.byref(st))
        _lib.check(rc, ctx.ptr)
        self.last_stats = self._stats_dict(st)
        return [AlignerResult(query, b, r["score"], r["end1"], r["end2"], r["width"], r["flags"])
                for b, r in zip(targets, out[:n])]
