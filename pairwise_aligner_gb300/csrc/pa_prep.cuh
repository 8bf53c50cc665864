// pa_prep.cuh -- batch preparation on the device: classify, encode, bucket.
//
// Replaces the reference's per-batch transposition and padding into SIMD lanes
// (include/pairwise_aligner/matrix/dp_vector_bulk.hpp:83-103): here every pair
// keeps its own length; pairs are only grouped so that the lanes and groups of
// one warp get matrices of nearly the same shape.
#pragma once
#include "pa_common.cuh"

namespace pa {

struct ClassCfg {
    int32_t fast_scores;     // match/mismatch fit a signed byte table
    int32_t s16_params;      // gap scores small enough for s16 lanes
    int32_t force32;         // width hint 32
    int32_t local;
    int32_t rows[kClasses];  // rows per pass (G*R) of each DP class
    int32_t gcnt[kClasses];  // G of each class (for the last-pass chunk count)
    int32_t rpt[kClasses];   // R of each class
    int64_t long_cells;      // pairs with m*n at least this (and m <= long_max_m) go to CTA mode
    int64_t huge_cells;      // ... and with m*n at least this and n >= huge_min_n to cluster mode
    int32_t long_max_m;      // the longest sequence1 the ring rows hold
    int32_t huge_min_n;
    int32_t team_max_n;      // CTA-mode pairs with n at most this run on teams of 4 warps (0: none)
    int32_t qtab_s16;        // write class K_S16's score tables (0: its kernel builds its own)
    const int8_t *rank_map;  // substitution-matrix scoring: symbol -> rank (null: unitary scores)
};

struct PrepStats {
    unsigned long long cells;
    unsigned long long n_class[16];
    unsigned long long overflow;    // pairs whose int32 bound fails
    unsigned long long invalid;     // substitution-matrix scoring: pairs with a symbol outside it
    unsigned long long bad_offsets; // pairs whose offsets are decreasing or run past the byte buffers
};

// Result of a pair the DP does not compute (no valid score): INT32_MIN at (0, 0).
__device__ __forceinline__ pa_result error_result(uint8_t flags)
{
    pa_result r;
    r.score = INT32_MIN;
    r.end1 = r.end2 = 0;
    r.width = 32;
    r.flags = flags;
    r.band_rounds = 0;
    return r;
}

__device__ __forceinline__ uint32_t quant_len(uint32_t m)
{
    if (m < 32u) return m;
    const uint32_t e = 31u - __clz(m);
    return min(1023u, 32u + (e - 5u) * 32u + ((m >> (e - 5u)) & 31u));
}

__device__ __forceinline__ uint32_t quant_shape(uint32_t s)
{
    if (s < 32u) return s;
    const uint32_t e = 31u - __clz(s);
    return min(63u, 32u + (e - 5u) * 4u + ((s >> (e - 2u)) & 3u));
}

// Result of a pair with an empty sequence (no DP needed); same candidate rules as the DP.
__device__ void trivial_result(const DpParams &P, int32_t m, int32_t n, pa_result &r)
{
    r.width = 32;
    r.flags = PA_RESULT_TRIVIAL;
    r.band_rounds = 0;
    if (P.local) { r.score = INT32_MIN; r.end1 = 0; r.end2 = 0; return; }
    int32_t s, i, j;
    if (m == 0) { s = border(P, P.first_row_free, n); i = 0; j = n; }
    else { s = border(P, P.first_column_free, m); i = m; j = 0; }
    auto take = [&](int32_t x, int32_t xi, int32_t xj) {
        if (x > s || (x == s && (xi < i || (xi == i && xj < j)))) { s = x; i = xi; j = xj; }
    };
    if (m == 0 && P.last_row_free) take(0, 0, 0);        // H(0, 0..n): the maximum is H(0,0)
    if (n == 0 && P.last_column_free) take(0, 0, 0);     // H(0..m, 0): likewise
    r.score = s; r.end1 = i; r.end2 = j;
}

// One warp per pair: check the pair's offsets against the byte buffers and sequence2's
// alphabet, pick the class, write the bucket key, the score tables of sequence1 and the
// results of pairs the DP does not compute: empty sequences (their border result),
// inconsistent offsets, scores that could exceed int32 and, with a substitution matrix,
// symbols outside it (INT32_MIN and a PA_RESULT_* flag).  Sequence bytes and scratch
// indices are touched only for pairs whose offsets passed the check.
__global__ void k_classify(const uint8_t *__restrict__ seq1, const uint64_t *__restrict__ off1, uint64_t seq1_bytes,
                           const uint8_t *__restrict__ seq2, const uint64_t *__restrict__ off2, uint64_t seq2_bytes,
                           uint64_t n_pairs, DpParams P, ClassCfg C, uint32_t *__restrict__ keys,
                           uint32_t *__restrict__ hist, uint32_t *__restrict__ qtab, pa_result *__restrict__ out,
                           PrepStats *__restrict__ st)
{
    const int lane = threadIdx.x & 31;
    const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint32_t match4 = (uint8_t)(P.match - P.shift) * 0x01010101u;     // scores of H - shift * column
    const uint32_t mis4 = (uint8_t)(P.mismatch - P.shift) * 0x01010101u;
    // statistics: per lane 0 in registers (cells, overflow, bad offsets) and per block in
    // shared memory (class sizes), added to the global counters once per block
    __shared__ unsigned long long sh[19];
    if (threadIdx.x < 19) sh[threadIdx.x] = 0;
    __syncthreads();
    unsigned long long my_cells = 0, my_overflow = 0, my_bad = 0;
    for (uint64_t p = warp; p < n_pairs; p += nwarps) {
        const uint64_t q0 = off1[p], q1 = off1[p + 1], t0 = off2[p], t1 = off2[p + 1];
        if (q0 > q1 || q1 > seq1_bytes || t0 > t1 || t1 > seq2_bytes) {
            if (lane == 0) {
                out[p] = error_result(PA_RESULT_ERROR);
                keys[p] = (uint32_t)K_NONE << kClassShift;
                ++my_bad;
            }
            continue;
        }
        const int64_t m = (int64_t)(q1 - q0), n = (int64_t)(t1 - t0);
        bool dna = true;
#pragma unroll 4
        for (int64_t j = 4 * lane; j < n; j += 128) {     // four independent loads per lane
            const uint8_t *q = seq2 + t0 + j;
            const int64_t left = n - j;
            dna &= dna_valid(q[0]);
            if (left > 1) dna &= dna_valid(q[1]);
            if (left > 2) dna &= dna_valid(q[2]);
            if (left > 3) dna &= dna_valid(q[3]);
        }
        dna = __all_sync(0xffffffffu, dna);
        bool symbols_ok = true;
        if (C.rank_map) {                                 // every symbol needs a rank
            for (int64_t j = lane; j < n; j += 32) symbols_ok &= C.rank_map[seq2[t0 + j]] >= 0;
            for (int64_t i = lane; i < m; i += 32) symbols_ok &= C.rank_map[seq1[q0 + i]] >= 0;
            symbols_ok = __all_sync(0xffffffffu, symbols_ok);
            if (!symbols_ok && lane == 0) atomicAdd(&st->invalid, 1ull);
        }
        const int64_t sa = P.match < 0 ? -(int64_t)P.match : P.match;
        const int64_t sb = P.mismatch < 0 ? -(int64_t)P.mismatch : P.mismatch;
        const int64_t go = -(int64_t)P.gap_open, ge = -(int64_t)P.gap_ext;
        const bool overflow =
            (sa + sb) * min(m, n) + (go + ge) * (m + n + 2) + 2 * go + (int64_t)P.shift * (m + n) >= (1ll << 30);
        if (m > 0 && n > 0 && (overflow || !symbols_ok)) {
            // no DP: the pair's scores could exceed int32, or a symbol has no rank
            if (lane == 0) {
                out[p] = error_result(overflow ? PA_RESULT_OVERFLOW : PA_RESULT_ERROR);
                keys[p] = (uint32_t)K_NONE << kClassShift;
                if (overflow) ++my_overflow;
            }
            continue;
        }
        uint32_t klass;
        if (m == 0 || n == 0) klass = K_NONE;
        else if (!C.fast_scores || !dna) klass = K_GEN;
        // s16 lanes: local scores stay in [0, smax min(m, n)]; global lanes hold H - smax * column,
        // which is at most 0, and a result is exact when that value of its end cell is above
        // the clamp floor (checked after the DP), so any length may try s16 first
        else if (!C.force32 && C.s16_params && (!C.local || (int64_t)P.smax * min(m, n) <= 30000)) klass = K_S16;
        else klass = K_S32;
        if (klass != K_NONE && m * n >= C.long_cells && m <= C.long_max_m && n <= (1 << 20))
            klass += (m * n >= C.huge_cells && n >= C.huge_min_n) ? kHugeOffset
                     : (n <= C.team_max_n)                        ? kMediumOffset
                                                                  : kLongOffset;
        if ((klass == K_S16 && C.qtab_s16) || klass == K_S32 || klass == K_S16L || klass == K_S32L ||
            klass == K_S16H || klass == K_S32H || klass == K_S16M || klass == K_S32M) {
            uint32_t *qt = qtab + q0 + p;
            for (int64_t i = 4 * lane; i <= m; i += 128) {
                const uint8_t *a = seq1 + q0 + i;
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (i + u <= m) qt[i + u] = (i + u < m) ? score_table(a[u], match4, mis4) : 0x80808080u;
            }
        }
        if (lane == 0) {
            uint32_t key;
            if (klass == K_NONE) {
                pa_result r;
                trivial_result(P, (int32_t)m, (int32_t)n, r);
                out[p] = r;
                key = (uint32_t)K_NONE << kClassShift;
            } else {
                // the pass shape, (passes - 1) * R/4 + (chunks of 4G rows in the last pass - 1), is
                // ceil(n / 4G) - 1 because a pass holds G*R rows, a multiple of 4G; G is a power of two
                const uint32_t G = (uint32_t)C.gcnt[klass];
                const uint64_t shape = (uint64_t)(n - 1) >> (2 + (31 - __clz(G)));
                key = (klass << kClassShift) | (quant_shape(shape > 0xffffffffull ? 0xffffffffu : (uint32_t)shape) << 10) |
                      quant_len((uint32_t)m);
                my_cells += (unsigned long long)(m * n);
            }
            keys[p] = key;
            atomicAdd(&hist[key], 1u);
            atomicAdd(&sh[1 + klass], 1ull);
        }
    }
    if (lane == 0) {
        if (my_cells) atomicAdd(&sh[0], my_cells);
        if (my_overflow) atomicAdd(&sh[17], my_overflow);
        if (my_bad) atomicAdd(&sh[18], my_bad);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (sh[0]) atomicAdd(&st->cells, sh[0]);
        for (int k = 0; k < 16; ++k)
            if (sh[1 + k]) atomicAdd(&st->n_class[k], sh[1 + k]);
        if (sh[17]) atomicAdd(&st->overflow, sh[17]);
        if (sh[18]) atomicAdd(&st->bad_offsets, sh[18]);
    }
}

// Exclusive scan of kBuckets counters in three kernels (1024 counters per block).
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *sh, uint32_t &total)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[w] = x;
    __syncthreads();
    if (w == 0) {
        uint32_t s = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        sh[lane] = s;
    }
    __syncthreads();
    total = sh[(blockDim.x >> 5) - 1];
    const uint32_t before = (w > 0) ? sh[w - 1] : 0u;
    __syncthreads();
    return before + x - v;
}

__global__ void k_scan_blocks(const uint32_t *__restrict__ hist, uint32_t *__restrict__ starts,
                              uint32_t *__restrict__ sums)
{
    __shared__ uint32_t sh[32];
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t total;
    const uint32_t ex = block_exclusive_scan(hist[x], sh, total);
    starts[x] = ex;
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void k_scan_sums(uint32_t *__restrict__ sums, uint32_t nblocks)
{
    __shared__ uint32_t sh[32];
    uint32_t total;
    const uint32_t v = threadIdx.x < nblocks ? sums[threadIdx.x] : 0u;
    const uint32_t ex = block_exclusive_scan(v, sh, total);
    if (threadIdx.x < nblocks) sums[threadIdx.x] = ex;
}

__global__ void k_scan_add(uint32_t *__restrict__ starts, uint32_t *__restrict__ cursor,
                           const uint32_t *__restrict__ sums, uint32_t *__restrict__ ranges)
{
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t s = starts[x] + sums[blockIdx.x];
    starts[x] = s;
    cursor[x] = s;
    if ((x & ((1u << kClassShift) - 1u)) == 0u) ranges[x >> kClassShift] = s;   // class begin
}

// A batch with inconsistent offsets is not aligned at all: the pairs' scratch regions
// (at off1[k] + k) could overlap when the offsets decrease somewhere, so every class is
// left empty and every pair gets an error result.
__global__ void k_scatter(const uint32_t *__restrict__ keys, uint64_t n_pairs, uint32_t *__restrict__ cursor,
                          uint32_t *__restrict__ order, const uint32_t *__restrict__ ranges,
                          uint32_t *__restrict__ counts, const PrepStats *__restrict__ st, pa_result *__restrict__ out)
{
    const uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const bool bad = st->bad_offsets != 0;
    if (p == 0) {
        // class sizes from the class begins (classes 7 and 11.. hold no keys)
        for (int c = 0; c < kClasses; ++c) counts[c] = bad ? 0u : ranges[c + 1] - ranges[c];
    }
    if (p >= n_pairs) return;
    if (bad) {
        out[p] = error_result(PA_RESULT_ERROR);
        return;
    }
    const uint32_t key = keys[p];
    if ((key >> kClassShift) == K_NONE) return;
    const uint32_t pos = atomicAdd(&cursor[key], 1u);
    order[pos] = (uint32_t)p;
}

// Who computes the largest pairs: clusters of blocks when their units fit in two waves of
// the clusters that can be resident (their run time would otherwise be one block's), else
// the CTA-mode kernel, ahead of the long pairs (more units than clusters: blocks, which
// quantise a pair's passes more finely, keep the GPU as busy).  words[0..2] are the
// cluster kernels' counts of K_S16H, K_S32H, K_GENH, words[3..5] the CTA kernels' lead counts.
__global__ void k_route_huge(const uint32_t *__restrict__ counts, uint32_t cluster_slots, uint32_t *__restrict__ words)
{
    const uint32_t c16 = counts[K_S16H], c32 = counts[K_S32H], cg = counts[K_GENH];
    const bool clusters = (c16 + 1) / 2 + c32 + cg <= 2 * cluster_slots;
    words[0] = clusters ? c16 : 0u;
    words[1] = clusters ? c32 : 0u;
    words[2] = clusters ? cg : 0u;
    words[3] = clusters ? 0u : c16;
    words[4] = clusters ? 0u : c32;
    words[5] = clusters ? 0u : cg;
}

}  // namespace pa
