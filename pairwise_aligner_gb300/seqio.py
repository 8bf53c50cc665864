"""The input path around the aligner: FASTA / FASTQ files, symbol ranks and 2-bit DNA.

* ``read_sequences(path)`` / ``parse_sequences(text)`` -- the native reader of
  libpa_gb300.so (``pa_seqfile_*``): concatenated sequence bytes plus offsets,
  names and (FASTQ) qualities, ready for ``Aligner.compute_arrays``.
* ``pack_2bit(seq)`` -- the host 2-bit encoder (A/a 0, C/c 1, G/g 2, T/t 3; base i
  at bits 2(i mod 16) of word i // 16); ``Aligner.compute_packed`` aligns packed
  streams, moving a quarter of the bytes to the device.
* ``rank_map_device`` / ``pack_2bit_device`` / ``unpack_2bit_device`` -- the device
  kernels on torch tensors, asynchronous on torch's current stream unless a count
  is asked for.  The rank map follows the reference's alphabet_rank_map_scalar /
  alphabet_rank_map_simd (alphabet_conversion/alphabet_rank_map_simd.hpp:31-117):
  symbol r of the list gets rank r, every other byte -1.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib


@dataclass
class SeqFile:
    names: list
    seq: np.ndarray            # uint8, all sequences back to back
    off: np.ndarray            # uint64, count + 1 offsets
    qual: np.ndarray | None    # uint8 (FASTQ), same offsets; None for FASTA

    def __len__(self):
        return len(self.names)

    def sequence(self, i: int) -> bytes:
        return self.seq[int(self.off[i]):int(self.off[i + 1])].tobytes()


def _take(lib, handle) -> SeqFile:
    try:
        n = lib.pa_seqfile_count(handle)
        off = np.ctypeslib.as_array(ctypes.cast(lib.pa_seqfile_offsets(handle), ctypes.POINTER(ctypes.c_uint64)),
                                    shape=(n + 1,)).copy()
        total = int(off[-1])
        seq = np.zeros(total, dtype=np.uint8)
        qual = None
        if total:
            ctypes.memmove(seq.ctypes.data, lib.pa_seqfile_sequences(handle), total)
        qp = lib.pa_seqfile_qualities(handle)
        if qp is not None:
            qual = np.zeros(total, dtype=np.uint8)
            if total:
                ctypes.memmove(qual.ctypes.data, qp, total)
        names = [lib.pa_seqfile_name(handle, i).decode("utf-8", "replace") for i in range(n)]
        return SeqFile(names, seq, off, qual)
    finally:
        lib.pa_seqfile_free(handle)


def read_sequences(path: str) -> SeqFile:
    """Read a FASTA or FASTQ file (format from its first non-blank byte)."""
    lib = _lib.load()
    h = ctypes.c_void_p()
    err = ctypes.create_string_buffer(256)
    rc = lib.pa_seqfile_read(str(path).encode(), ctypes.byref(h), err, len(err))
    if rc:
        raise _lib.PaError(rc, err.value.decode())
    return _take(lib, h)


def parse_sequences(text: bytes) -> SeqFile:
    """Parse FASTA / FASTQ text held in memory."""
    lib = _lib.load()
    h = ctypes.c_void_p()
    err = ctypes.create_string_buffer(256)
    buf = bytes(text)
    rc = lib.pa_seqfile_parse(buf, len(buf), ctypes.byref(h), err, len(err))
    if rc:
        raise _lib.PaError(rc, err.value.decode())
    return _take(lib, h)


def pack_2bit(seq) -> tuple[np.ndarray, int]:
    """Host 2-bit encoding of a byte stream -> (uint32 words, number of non-ACGT bytes)."""
    a = np.ascontiguousarray(np.frombuffer(seq, dtype=np.uint8) if isinstance(seq, (bytes, bytearray))
                             else seq, dtype=np.uint8)
    words = np.zeros(max((len(a) + 15) // 16, 1), dtype=np.uint32)
    bad = ctypes.c_uint64()
    _lib.check(_lib.load().pa_pack_2bit_host(a.ctypes.data, len(a), words.ctypes.data, ctypes.byref(bad)))
    return words[:(len(a) + 15) // 16], int(bad.value)


def _stream():
    import torch
    return torch.cuda.current_stream().cuda_stream or 1      # 1: cudaStreamLegacy


def rank_map_device(context, symbols: bytes, d_in, d_out, count_invalid: bool = False):
    """Ranks of the bytes of uint8 tensor `d_in` into int8 tensor `d_out`; returns the number of
    bytes without a rank when `count_invalid` (a synchronous call), else None."""
    sym = np.frombuffer(bytes(symbols), dtype=np.uint8).copy()
    bad = ctypes.c_uint64()
    _lib.check(context.lib.pa_rank_map_device(context.ptr, sym.ctypes.data, len(sym), d_in.data_ptr(), d_in.numel(),
                                              d_out.data_ptr(), _stream(),
                                              ctypes.byref(bad) if count_invalid else None), context.ptr)
    return int(bad.value) if count_invalid else None


def pack_2bit_device(context, d_in, d_words, count_invalid: bool = False):
    """2-bit words of uint8 tensor `d_in` into the int32 tensor `d_words` ((n + 15) // 16 words)."""
    bad = ctypes.c_uint64()
    _lib.check(context.lib.pa_pack_2bit_device(context.ptr, d_in.data_ptr(), d_in.numel(), d_words.data_ptr(),
                                               _stream(), ctypes.byref(bad) if count_invalid else None),
               context.ptr)
    return int(bad.value) if count_invalid else None


def unpack_2bit_device(context, d_words, first_base: int, n: int, d_out):
    """Bases [first_base, first_base + n) of the packed `d_words` as letters into uint8 `d_out`."""
    _lib.check(context.lib.pa_unpack_2bit_device(context.ptr, d_words.data_ptr(), int(first_base), int(n),
                                                 d_out.data_ptr(), _stream()), context.ptr)
