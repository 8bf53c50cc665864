"""Seeded synthetic DNA workloads for the five benchmark configurations.

No public dataset is involved: the reference's own benchmarks draw random DNA
(test/benchmark/affine/alignment_benchmark_fixture.hpp:91-117), and these
generators follow the configuration texts (lengths, mutation rates, indel-length
distributions, scoring).  Everything is numpy, vectorised, seeded.

Mutation model (``mutate``): per source base, a deletion starts with
probability p_del (geometric length, given mean), an insertion of random bases
(geometric length) is placed before it with probability p_ins, and a kept base
is substituted by one of the three other bases with probability p_sub.

Scores follow the reference's sign convention (gap of length k scores
open + k * ext):
    config 1: global, +2/-3, gap_model_affine(-5, -1)
    config 2: local,  +1/-4, gap_model_affine(-6, -1)
    config 3: global, +2/-4, gap_model_affine(-4, -2)
    config 4: global, +1/-4, gap_model_affine(-6, -1)
    config 5: global, +1/-4, gap_model_affine(-6, -1)
"""
from __future__ import annotations

import numpy as np

ACGT = np.frombuffer(b"ACGT", dtype=np.uint8)

SCORING = {
    1: dict(local=False, match=2, mismatch=-3, gap_open=-5, gap_extension=-1),
    2: dict(local=True, match=1, mismatch=-4, gap_open=-6, gap_extension=-1),
    3: dict(local=False, match=2, mismatch=-4, gap_open=-4, gap_extension=-2),
    4: dict(local=False, match=1, mismatch=-4, gap_open=-6, gap_extension=-1),
    5: dict(local=False, match=1, mismatch=-4, gap_open=-6, gap_extension=-1),
}


def _offsets(lens: np.ndarray) -> np.ndarray:
    off = np.zeros(len(lens) + 1, dtype=np.uint64)
    np.cumsum(lens.astype(np.uint64), out=off[1:])
    return off


def _ranges(starts: np.ndarray, lens: np.ndarray) -> np.ndarray:
    """Concatenation of arange(starts[k], starts[k] + lens[k]) over k, vectorised."""
    starts = starts.astype(np.int64)
    lens = lens.astype(np.int64)
    total = int(lens.sum())
    if total == 0:
        return np.zeros(0, np.int64)
    base = np.repeat(starts - (np.cumsum(lens) - lens), lens)
    return base + np.arange(total)


def random_codes(rng: np.random.Generator, lens: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    off = _offsets(lens)
    return rng.integers(0, 4, size=int(off[-1]), dtype=np.uint8), off


def _geom(rng, mean: float, size: int) -> np.ndarray:
    if size == 0:
        return np.zeros(0, np.int64)
    return rng.geometric(1.0 / mean, size=size).astype(np.int64)


def mutate(rng: np.random.Generator, codes: np.ndarray, off: np.ndarray, p_sub: float, p_ins: float,
           p_del: float, indel_mean: float) -> tuple[np.ndarray, np.ndarray]:
    """Apply substitutions / insertions / deletions per pair; returns (codes, offsets)."""
    N = len(codes)
    n_pairs = len(off) - 1
    off64 = off.astype(np.int64)
    pair_of = np.repeat(np.arange(n_pairs), np.diff(off64))
    pair_end = off64[1:][pair_of] if N else np.zeros(0, np.int64)
    u = rng.random(N)
    # deletions
    dstart = np.flatnonzero(u < p_del)
    dlen = _geom(rng, indel_mean, len(dstart))
    dend = np.minimum(dstart + dlen, pair_end[dstart])
    diff = np.zeros(N + 1, dtype=np.int64)
    np.add.at(diff, dstart, 1)
    np.add.at(diff, dend, -1)
    deleted = np.cumsum(diff[:-1]) > 0
    # substitutions
    out_base = codes.copy()
    sub = (u >= p_del) & (u < p_del + p_sub) & ~deleted
    out_base[sub] = (out_base[sub] + rng.integers(1, 4, size=int(sub.sum()), dtype=np.uint8)) % 4
    # insertions before a position
    ins_at = np.flatnonzero(rng.random(N) < p_ins)
    ins_len = np.zeros(N, dtype=np.int64)
    ins_len[ins_at] = _geom(rng, indel_mean, len(ins_at))
    counts = ins_len + (~deleted).astype(np.int64)
    total = int(counts.sum())
    src = np.repeat(np.arange(N), counts)
    start = np.cumsum(counts) - counts
    rank = np.arange(total) - start[src]
    is_ins = rank < ins_len[src]
    out = np.where(is_ins, rng.integers(0, 4, size=total, dtype=np.uint8), out_base[src]).astype(np.uint8)
    # new per-pair offsets
    csum = np.zeros(N + 1, dtype=np.int64)
    np.cumsum(counts, out=csum[1:])
    new_off = csum[off64].astype(np.uint64)
    return out, new_off


def fit_length(rng: np.random.Generator, codes: np.ndarray, off: np.ndarray, target: np.ndarray):
    """Crop each sequence to a random window of length target[k], or pad it with random flanks."""
    n_pairs = len(off) - 1
    off64 = off.astype(np.int64)
    lens = np.diff(off64)
    target = target.astype(np.int64)
    slack = lens - target
    crop_start = np.where(slack > 0, (rng.random(n_pairs) * (np.maximum(slack, 0) + 1)).astype(np.int64), 0)
    pad_left = np.where(slack < 0, (rng.random(n_pairs) * (np.maximum(-slack, 0) + 1)).astype(np.int64), 0)
    new_off = _offsets(target)
    total = int(new_off[-1])
    pair = np.repeat(np.arange(n_pairs), target)
    pos = np.arange(total) - new_off[:-1].astype(np.int64)[pair]
    srcpos = pos + crop_start[pair] - pad_left[pair]
    inside = (srcpos >= 0) & (srcpos < lens[pair])
    src = np.where(inside, off64[:-1][pair] + np.clip(srcpos, 0, None), 0)
    out = np.where(inside, codes[np.minimum(src, max(len(codes) - 1, 0))] if len(codes) else 0,
                   rng.integers(0, 4, size=total, dtype=np.uint8)).astype(np.uint8)
    return out, new_off


def structural_indels(rng: np.random.Generator, codes: np.ndarray, off: np.ndarray, lo: int = 50, hi: int = 500):
    """One or two insertion/deletion runs of lo..hi bases per sequence, placed uniformly."""
    parts, lens = [], []
    off64 = off.astype(np.int64)
    for k in range(len(off64) - 1):
        s = codes[off64[k]:off64[k + 1]]
        for _ in range(int(rng.integers(1, 3))):
            L = int(rng.integers(lo, hi + 1))
            p = int(rng.integers(0, len(s) + 1))
            if rng.random() < 0.5:
                s = np.concatenate([s[:p], rng.integers(0, 4, size=L, dtype=np.uint8), s[p:]])
            else:
                s = np.concatenate([s[:p], s[p + L:]])
        parts.append(s)
        lens.append(len(s))
    return (np.concatenate(parts) if parts else np.zeros(0, np.uint8)), _offsets(np.array(lens, dtype=np.int64))


def _interleave(n_pairs: int, groups):
    """Merge generated groups ((q, qo, t, to, idx) with idx = destination pair ids)."""
    qlen = np.zeros(n_pairs, np.int64)
    tlen = np.zeros(n_pairs, np.int64)
    for q, qo, t, to, idx in groups:
        qlen[idx] = np.diff(qo.astype(np.int64))
        tlen[idx] = np.diff(to.astype(np.int64))
    qoff, toff = _offsets(qlen), _offsets(tlen)
    qs = np.zeros(int(qoff[-1]), np.uint8)
    ts = np.zeros(int(toff[-1]), np.uint8)
    for q, qo, t, to, idx in groups:
        qo64, to64 = qo.astype(np.int64), to.astype(np.int64)
        dst = np.repeat(qoff[:-1].astype(np.int64)[idx] - qo64[:-1], np.diff(qo64)) + np.arange(len(q))
        qs[dst] = q
        dst = np.repeat(toff[:-1].astype(np.int64)[idx] - to64[:-1], np.diff(to64)) + np.arange(len(t))
        ts[dst] = t
    return qs, qoff, ts, toff


def _finish(qs, qoff, ts, toff, cfg: int, name: str):
    d = dict(SCORING[cfg])
    d.update(seq1=ACGT[qs], off1=qoff, seq2=ACGT[ts], off2=toff, name=name, config=cfg)
    return d


def config1(seed: int = 1, n_pairs: int = 1024):
    """1,024 global pairs: query 150 bp uniform; target = query with 8% sub, 1% ins, 1% del (mean 2)."""
    rng = np.random.default_rng(seed)
    q, qo = random_codes(rng, np.full(n_pairs, 150))
    t, to = mutate(rng, q, qo, 0.08, 0.01, 0.01, 2.0)
    return _finish(q, qo, t, to, 1, "config1_global_150bp")


def config2(seed: int = 2, n_pairs: int = 262144):
    """Local pairs, m and n independent U[64,512]; half related (15/2/2%, mean 2), half unrelated.

    A related target is the mutated query cropped to a random window of length n
    (or padded with random flanks), so lengths stay independent and uniform."""
    rng = np.random.default_rng(seed)
    m = rng.integers(64, 513, size=n_pairs)
    n = rng.integers(64, 513, size=n_pairs)
    related = rng.random(n_pairs) < 0.5
    q, qo = random_codes(rng, m)
    idx_r = np.flatnonzero(related)
    idx_u = np.flatnonzero(~related)
    qo64 = qo.astype(np.int64)
    # related targets
    qr = q[_ranges(qo64[idx_r], m[idx_r])]
    qro = _offsets(m[idx_r])
    tr, tro = mutate(rng, qr, qro, 0.15, 0.02, 0.02, 2.0)
    tr, tro = fit_length(rng, tr, tro, n[idx_r])
    tu, tuo = random_codes(rng, n[idx_u])
    tlen = np.zeros(n_pairs, np.int64)
    tlen[idx_r] = np.diff(tro.astype(np.int64))
    tlen[idx_u] = np.diff(tuo.astype(np.int64))
    toff = _offsets(tlen)
    ts = np.zeros(int(toff[-1]), np.uint8)
    for t_, to_, idx in ((tr, tro, idx_r), (tu, tuo, idx_u)):
        to64 = to_.astype(np.int64)
        dst = np.repeat(toff[:-1].astype(np.int64)[idx] - to64[:-1], np.diff(to64)) + np.arange(len(t_))
        ts[dst] = t_
    d = _finish(q, qo, ts, toff, 2, "config2_local_64-512bp")
    d["related"] = related
    return d


def config3(seed: int = 3, n_pairs: int = 8192):
    """Global long reads: query log-normal (median 3000, sigma 0.6, clipped 500..20000); 5/3/3% (mean 1.5)."""
    rng = np.random.default_rng(seed)
    m = np.clip(np.round(np.exp(np.log(3000.0) + 0.6 * rng.standard_normal(n_pairs))), 500, 20000).astype(np.int64)
    q, qo = random_codes(rng, m)
    t, to = mutate(rng, q, qo, 0.05, 0.03, 0.03, 1.5)
    return _finish(q, qo, t, to, 3, "config3_global_longreads")


def config4(seed: int = 4, n_pairs: int = 16384):
    """Config-2 lengths and mutation (global) plus one or two 50-500 bp structural indels per pair."""
    rng = np.random.default_rng(seed)
    m = rng.integers(64, 513, size=n_pairs)
    q, qo = random_codes(rng, m)
    t, to = mutate(rng, q, qo, 0.15, 0.02, 0.02, 2.0)
    t, to = structural_indels(rng, t, to)
    return _finish(q, qo, t, to, 4, "config4_global_sv")


def config5(seed: int = 5, n_pairs: int = 1048576, strata=(0.90, 0.09, 0.01)):
    """Mixed global stream: 90% U[100,300] @10% (8:1:1), 9% U[1000,10000] @8%, 1% U[20000,50000] @6% + SVs."""
    rng = np.random.default_rng(seed)
    kind = rng.choice(3, size=n_pairs, p=list(strata))
    groups = []
    specs = [(100, 300, 0.10, False), (1000, 10000, 0.08, False), (20000, 50000, 0.06, True)]
    for k, (lo, hi, div, sv) in enumerate(specs):
        idx = np.flatnonzero(kind == k)
        if len(idx) == 0:
            continue
        m = rng.integers(lo, hi + 1, size=len(idx))
        q, qo = random_codes(rng, m)
        t, to = mutate(rng, q, qo, div * 0.8, div * 0.1, div * 0.1, 2.0)
        if sv:
            t, to = structural_indels(rng, t, to)
        groups.append((q, qo, t, to, idx))
    qs, qoff, ts, toff = _interleave(n_pairs, groups)
    d = _finish(qs, qoff, ts, toff, 5, "config5_mixed_stream")
    d["stratum"] = kind
    return d


GENERATORS = {1: config1, 2: config2, 3: config3, 4: config4, 5: config5}


def subset(d: dict, idx: np.ndarray) -> dict:
    """A new workload made of pairs idx (in that order)."""
    out = {k: v for k, v in d.items() if k not in ("seq1", "off1", "seq2", "off2", "related", "stratum")}
    for s, o in (("seq1", "off1"), ("seq2", "off2")):
        off = d[o].astype(np.int64)
        lens = off[idx + 1] - off[idx]
        new_off = _offsets(lens)
        out[s] = d[s][_ranges(off[idx], lens)]
        out[o] = new_off
    return out


def concat(ds: list[dict]) -> dict:
    """The pairs of several workloads of one scoring, in order."""
    out = {k: v for k, v in ds[0].items() if k not in ("seq1", "off1", "seq2", "off2", "related", "stratum")}
    for s, o in (("seq1", "off1"), ("seq2", "off2")):
        out[s] = np.concatenate([d[s] for d in ds])
        lens = np.concatenate([np.diff(d[o].astype(np.int64)) for d in ds])
        out[o] = _offsets(lens)
    return out


def cells(d: dict) -> int:
    m = np.diff(d["off1"].astype(np.int64))
    n = np.diff(d["off2"].astype(np.int64))
    return int((m * n).sum())
