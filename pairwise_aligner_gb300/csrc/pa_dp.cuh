// pa_dp.cuh -- the affine-gap (Gotoh) score DP kernel for sm_103a.
//
// One "group" of G consecutive lanes of a warp (G = 1, 2, ..., 32) computes the
// DP matrix of one pair (s32 lanes) or of two pairs at once (s16x2 lanes: pair A
// in the low halfword, pair B in the high halfword of every register).  The
// recurrence is the reference's compute_cell
// (include/pairwise_aligner/affine/affine_dp_algorithm.hpp:149-155):
//     best = max(diag + s(a,b), vgap, hgap)          [local: max(diag + s, 0) first,
//                                                     dp_matrix_local.hpp:39-47]
//     vgap' = max(vgap + ext, best + open + ext);  hgap' = max(hgap + ext, best + open + ext)
// with the border cells of affine_initialisation_strategy.hpp:38-51.
//
// Layout of the work: sequence2 ("held") runs down the rows, sequence1
// ("streamed") along the columns.  Thread t of a group holds rows
// [t*R, t*R + R) of the current pass in registers (H and the rightward gap per
// row, plus a byte-permute selector that encodes the row's base); the group
// sweeps the columns as an anti-diagonal wavefront: at step s thread t computes
// column s - t + 1 and hands the bottom H and downward gap of its strip to
// thread t+1 with __shfl_up_sync.  Rows beyond G*R are covered by further
// passes; the last thread spills its bottom row per column to the pass-boundary
// scratch (8 bytes per column), where thread 0 of the next pass reads it.
//
// Scores: the streamed base of each lane selects a 4-byte table
// (match in the byte of its 2-bit code, mismatch elsewhere); one PRMT with the
// row's selector yields the packed, sign-extended scores of both lanes.
// Arithmetic: DPX __viaddmax / __vimax3(_relu) in s16x2 or s32 form.
//
// Tracking (the reference trackers, tracker/*.hpp):
//   local  -- running column maximum per strip; on a strict improvement the
//             strip's H column is kept, so the end is the smallest column i,
//             then the smallest row j of the maximum (order independent).
//   global -- H(m, n) is read where it is computed; free trailing gaps also
//             scan the last row (i = m) and the last column (j = n).
// s16 global lanes clamp every H at `floor16` from below, which keeps all adds
// inside int16; a result above floor16 + smax * min(m, n) cannot have been
// influenced by a clamp and is exact, anything else is recomputed in s32.
#pragma once
#include "pa_common.cuh"

namespace pa {

enum Mode : int { M_LOCAL = 0, M_GLOBAL = 1, M_GLOBAL_FREE = 2 };

// ---- lane arithmetic policies ------------------------------------------------
struct L16 {
    static constexpr int LANES = 2;
    static constexpr uint8_t WIDTH = 16;
    static __device__ __forceinline__ uint32_t splat(int32_t x)
    {
        uint32_t h = (uint16_t)(int16_t)x;
        return h | (h << 16);
    }
    static __device__ __forceinline__ int32_t get(uint32_t v, int l)
    {
        return l ? (int32_t)(int16_t)(v >> 16) : (int32_t)(int16_t)(v & 0xffffu);
    }
    static __device__ __forceinline__ uint32_t addmax(uint32_t a, uint32_t b, uint32_t c)
    {
        return __viaddmax_s16x2(a, b, c);
    }
    static __device__ __forceinline__ uint32_t add(uint32_t a, uint32_t b)
    {
        return __viaddmax_s16x2(a, b, 0x80008000u);
    }
    static __device__ __forceinline__ uint32_t hmax_local(uint32_t t, uint32_t e, uint32_t)
    {
        return __vimax_s16x2_relu(t, e);
    }
    static __device__ __forceinline__ uint32_t hmax_global(uint32_t t, uint32_t e, uint32_t fl)
    {
        return __vimax3_s16x2(t, e, fl);
    }
    static __device__ __forceinline__ uint32_t max3(uint32_t a, uint32_t b, uint32_t c)
    {
        return __vimax3_s16x2(a, b, c);
    }
    // best = max(best, c) per lane; returns an all-ones mask over the lanes where c > old best.
    static __device__ __forceinline__ uint32_t improve(uint32_t &best, uint32_t c)
    {
        const uint32_t gt = __vcmpgts2(c, best);   // 0xffff per halfword where c > best
        best = __vmaxs2(best, c);
        return gt;
    }
    static __device__ __forceinline__ bool lane_bit(uint32_t mask, int l) { return (mask >> (16 * l)) & 1u; }
    // Byte-permute selector of a held row.  Low halfword <- table byte `ca` of lane A
    // (bytes 0-3) sign-extended, high halfword <- byte 4+cb of lane B.  A padded row
    // (code < 0) replicates the sign of a table byte: its score is 0 or -1.
    static __device__ __forceinline__ uint32_t selector(int ca, int cb)
    {
        uint32_t lo = ca < 0 ? 0x88u : ((uint32_t)ca | (((uint32_t)ca | 8u) << 4));
        uint32_t hi = cb < 0 ? 0xCCu : ((4u + (uint32_t)cb) | (((4u + (uint32_t)cb) | 8u) << 4));
        return lo | (hi << 8);
    }
};

struct L32 {
    static constexpr int LANES = 1;
    static constexpr uint8_t WIDTH = 32;
    static __device__ __forceinline__ uint32_t splat(int32_t x) { return (uint32_t)x; }
    static __device__ __forceinline__ int32_t get(uint32_t v, int) { return (int32_t)v; }
    static __device__ __forceinline__ uint32_t addmax(uint32_t a, uint32_t b, uint32_t c)
    {
        return (uint32_t)__viaddmax_s32((int)a, (int)b, (int)c);
    }
    static __device__ __forceinline__ uint32_t add(uint32_t a, uint32_t b) { return a + b; }
    static __device__ __forceinline__ uint32_t hmax_local(uint32_t t, uint32_t e, uint32_t)
    {
        return (uint32_t)__vimax_s32_relu((int)t, (int)e);
    }
    static __device__ __forceinline__ uint32_t hmax_global(uint32_t t, uint32_t e, uint32_t)
    {
        return (uint32_t)max((int)t, (int)e);
    }
    static __device__ __forceinline__ uint32_t max3(uint32_t a, uint32_t b, uint32_t c)
    {
        return (uint32_t)__vimax3_s32((int)a, (int)b, (int)c);
    }
    static __device__ __forceinline__ uint32_t improve(uint32_t &best, uint32_t c)
    {
        const bool gt = (int)c > (int)best;
        best = gt ? c : best;
        return gt ? 0xffffffffu : 0u;
    }
    static __device__ __forceinline__ bool lane_bit(uint32_t mask, int) { return mask != 0u; }
    static __device__ __forceinline__ uint32_t selector(int ca, int)
    {
        if (ca < 0) return 0x8888u;
        uint32_t c = (uint32_t)ca, s = c | 8u;
        return c | (s << 4) | (s << 8) | (s << 12);
    }
};

// (score, end1, end2) candidate order: higher score, then smaller end1, then smaller end2.
__device__ __forceinline__ bool better(int32_t s, int32_t i, int32_t j, int32_t bs, int32_t bi, int32_t bj)
{
    return s > bs || (s == bs && (i < bi || (i == bi && j < bj)));
}

constexpr int kChunk = 4;   // rows per guarded chunk of the register strip

// GEN = byte-compare scoring (any bytes, any int32 scores), always with L32 lanes.
template <class V, int R, int MODE, bool GEN>
__global__ void __launch_bounds__(256) dp_kernel(DpLaunch L, DpParams P)
{
    static_assert(R % kChunk == 0, "R must be a multiple of the chunk");
    constexpr int NL = V::LANES;
    constexpr int NCH = R / kChunk;
    const int lane = threadIdx.x & 31;
    const int G = L.G;
    const int t = lane & (G - 1);
    const int g = lane / G;
    const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (g * G));
    const uint32_t count = *L.count_ptr;
    const uint32_t *order = L.order + *L.begin_ptr;
    const uint32_t ppw = (uint32_t)(32 / G) * NL;   // pairs per warp unit
    const uint32_t n_units = (count + ppw - 1) / ppw;

    const uint32_t GOE = V::splat(P.gap_open + P.gap_ext);
    const uint32_t EXT = V::splat(P.gap_ext);
    const uint32_t FLOOR = V::splat(P.floor16);
    const bool clamp16 = (NL == 2) && MODE != M_LOCAL;
    const uint32_t PADTAB = 0x80808080u;

    for (;;) {
        uint32_t u = 0;
        if (lane == 0) u = atomicAdd(L.unit_counter, 1u);
        u = __shfl_sync(0xffffffffu, u, 0);
        if (u >= n_units) break;
        u = n_units - 1 - u;                         // largest shapes first
        const uint32_t first = u * ppw + (uint32_t)g * NL;
        if (first >= count) continue;                // idle group in the last unit

        uint32_t id[2];
        id[0] = order[first];
        const bool has_b = NL == 2 && first + 1 < count;
        id[1] = has_b ? order[first + 1] : id[0];
        uint64_t qoff[2], toff[2];
        int32_t m[2], n[2];
#pragma unroll
        for (int l = 0; l < 2; ++l) {
            qoff[l] = L.off1[id[l]];
            m[l] = (int32_t)(L.off1[id[l] + 1] - qoff[l]);
            toff[l] = L.off2[id[l]];
            n[l] = (int32_t)(L.off2[id[l] + 1] - toff[l]);
        }
        const int32_t ms = NL == 2 ? max(m[0], m[1]) : m[0];
        const int32_t nh = NL == 2 ? max(n[0], n[1]) : n[0];
        const int32_t rows_full = G * R;
        const int32_t passes = (nh + rows_full - 1) / rows_full;
        const int owner = (NL == 2 && m[1] > m[0]) ? 1 : 0;
        Cell *buf = L.boundary + (L.off1[id[owner]] + id[owner]);
        const uint32_t *qt[2];
#pragma unroll
        for (int l = 0; l < 2; ++l) qt[l] = L.qtab + qoff[l] + id[l];

        int32_t cs[2], ci[2], cj[2];
#pragma unroll
        for (int l = 0; l < 2; ++l) { cs[l] = MODE == M_LOCAL ? 0 : INT32_MIN; ci[l] = 0; cj[l] = 0; }

        for (int p = 0; p < passes; ++p) {
            // rows of this pass: the last pass keeps only the chunks it needs
            const int32_t rem = nh - p * rows_full;
            const int32_t rpt = rem >= rows_full ? R : ((rem + G * kChunk - 1) / (G * kChunk)) * kChunk;
            const int32_t nch = rpt / kChunk;
            const int32_t pass_base = p * rows_full;
            const int32_t j0 = pass_base + t * rpt;   // rows j0+1 .. j0+rpt (1-based)

            uint32_t H[R], Fr[R], Sel[R], Snap[R];
#pragma unroll
            for (int k = 0; k < R; ++k) {
                const int32_t j = j0 + k;              // 0-based index into sequence2
                int c[2];
#pragma unroll
                for (int l = 0; l < 2; ++l) {
                    if (GEN) c[l] = (k < rpt && j < n[l]) ? (int)L.seq2[toff[l] + j] : 0x100;
                    else c[l] = (k < rpt && j < n[l]) ? (int)dna_code(L.seq2[toff[l] + j]) : -1;
                }
                Sel[k] = GEN ? (uint32_t)c[0] : V::selector(c[0], c[1]);
                int32_t h = border(P, P.first_row_free, (int64_t)j + 1);
                if (clamp16) h = max(h, P.floor16);
                H[k] = V::splat(h);
                Fr[k] = V::add(H[k], GOE);
                Snap[k] = 0;
            }
            int32_t hp = border(P, P.first_row_free, j0);
            if (clamp16) hp = max(hp, P.floor16);
            uint32_t prevH = V::splat(hp);
            uint32_t outH = 0, outE = 0, best = 0;
            int32_t bi[2] = {0, 0};
            int32_t own_k[2], own_t[2], own_p[2];
#pragma unroll
            for (int l = 0; l < 2; ++l) {            // where row n[l] lives
                own_p[l] = (n[l] - 1) / rows_full;
                const int32_t r = (n[l] - 1) - own_p[l] * rows_full;
                const int32_t rr = (own_p[l] == p) ? rpt : R;
                own_t[l] = r / rr;
                own_k[l] = r - own_t[l] * rr;
            }

            const int32_t steps = ms + G - 1;
            for (int s = 0; s < steps; ++s) {
                const int32_t i = s - t + 1;          // 1-based column of this thread
                uint32_t upH = __shfl_up_sync(gmask, outH, 1, G);
                uint32_t upE = __shfl_up_sync(gmask, outE, 1, G);
                if (i < 1 || i > ms) continue;
                if (t == 0) {
                    if (p == 0) {
                        int32_t h = border(P, P.first_column_free, i);
                        if (clamp16) h = max(h, P.floor16);
                        upH = V::splat(h);
                        upE = V::add(upH, GOE);
                    } else {
                        const Cell c = buf[i];
                        upH = c.h;
                        upE = c.e;
                    }
                }
                // streamed base of each lane -> score table (or raw byte for GEN)
                uint32_t ta, tb;
                if (GEN) {
                    ta = (i <= m[0]) ? (uint32_t)L.seq1[qoff[0] + i - 1] : 0x200u;
                    tb = ta;
                } else {
                    ta = __ldg(qt[0] + min(i - 1, m[0]));
                    tb = NL == 2 ? __ldg(qt[1] + min(i - 1, m[1])) : ta;
                }
                uint32_t diag = prevH, Ed = upE;
#pragma unroll
                for (int k = 0; k < R; ++k) {
                    if (k % kChunk == 0 && k / kChunk >= nch) break;
                    uint32_t sc;
                    if (GEN) {
                        const uint32_t x = Sel[k];
                        sc = (x == ta) ? (uint32_t)P.match
                                       : (((x | ta) >> 8) ? (uint32_t)P.spad : (uint32_t)P.mismatch);
                    } else {
                        sc = prmt(ta, tb, Sel[k]);
                    }
                    const uint32_t tt = V::addmax(diag, sc, Fr[k]);
                    const uint32_t h = MODE == M_LOCAL ? V::hmax_local(tt, Ed, FLOOR) : V::hmax_global(tt, Ed, FLOOR);
                    diag = H[k];
                    H[k] = h;
                    const uint32_t hoe = V::add(h, GOE);
                    Fr[k] = V::addmax(Fr[k], EXT, hoe);
                    Ed = V::addmax(Ed, EXT, hoe);
                }
                prevH = upH;
                uint32_t last = H[R - 1];
#pragma unroll
                for (int c = 1; c < NCH; ++c)
                    if (nch == c) last = H[c * kChunk - 1];
                outH = last;
                outE = Ed;
                if (t == G - 1 && p + 1 < passes) buf[i] = Cell{outH, outE};

                if (MODE == M_LOCAL) {
                    uint32_t cm = 0;                  // local H >= 0
#pragma unroll
                    for (int c = 0; c < NCH; ++c) {
                        if (c >= nch) break;
                        cm = V::max3(cm, H[c * kChunk], H[c * kChunk + 1]);
                        cm = V::max3(cm, H[c * kChunk + 2], H[c * kChunk + 3]);
                    }
                    const uint32_t mask = V::improve(best, cm);
#pragma unroll
                    for (int k = 0; k < R; ++k) {
                        if (k % kChunk == 0 && k / kChunk >= nch) break;
                        Snap[k] = (H[k] & mask) | (Snap[k] & ~mask);
                    }
#pragma unroll
                    for (int l = 0; l < NL; ++l)
                        if (V::lane_bit(mask, l)) bi[l] = i;
                } else {
#pragma unroll
                    for (int l = 0; l < NL; ++l) {
                        if (l == 1 && !has_b) continue;
                        if (MODE == M_GLOBAL_FREE && P.last_column_free && p == own_p[l] && t == own_t[l] &&
                            i <= m[l]) {
                            uint32_t v = H[0];
#pragma unroll
                            for (int k = 1; k < R; ++k)
                                if (own_k[l] == k) v = H[k];
                            const int32_t x = V::get(v, l);
                            if (better(x, i, n[l], cs[l], ci[l], cj[l])) { cs[l] = x; ci[l] = i; cj[l] = n[l]; }
                        }
                        if (i == m[l]) {
                            if (MODE == M_GLOBAL_FREE && P.last_row_free) {
#pragma unroll
                                for (int k = 0; k < R; ++k) {
                                    const int32_t j = j0 + k + 1;
                                    if (k < rpt && j <= n[l]) {
                                        const int32_t x = V::get(H[k], l);
                                        if (better(x, i, j, cs[l], ci[l], cj[l])) { cs[l] = x; ci[l] = i; cj[l] = j; }
                                    }
                                }
                            } else if (p == own_p[l] && t == own_t[l]) {
                                uint32_t v = H[0];
#pragma unroll
                                for (int k = 1; k < R; ++k)
                                    if (own_k[l] == k) v = H[k];
                                const int32_t x = V::get(v, l);
                                if (better(x, i, n[l], cs[l], ci[l], cj[l])) { cs[l] = x; ci[l] = i; cj[l] = n[l]; }
                            }
                        }
                    }
                }
            }
            if (MODE == M_LOCAL) {
#pragma unroll
                for (int l = 0; l < NL; ++l) {
                    const int32_t b = V::get(best, l);
                    if (b > 0) {
                        int32_t kk = -1;
#pragma unroll
                        for (int k = R - 1; k >= 0; --k)
                            if (k < rpt && V::get(Snap[k], l) == b) kk = k;
                        const int32_t j = j0 + kk + 1;
                        if (better(b, bi[l], j, cs[l], ci[l], cj[l])) { cs[l] = b; ci[l] = bi[l]; cj[l] = j; }
                    }
                }
            }
            __syncwarp(gmask);
        }

        // group reduction of the candidates
#pragma unroll
        for (int l = 0; l < NL; ++l) {
            for (int off = G >> 1; off >= 1; off >>= 1) {
                const int32_t os = __shfl_xor_sync(gmask, cs[l], off, G);
                const int32_t oi = __shfl_xor_sync(gmask, ci[l], off, G);
                const int32_t oj = __shfl_xor_sync(gmask, cj[l], off, G);
                if (better(os, oi, oj, cs[l], ci[l], cj[l])) { cs[l] = os; ci[l] = oi; cj[l] = oj; }
            }
        }
        if (t == 0) {
#pragma unroll
            for (int l = 0; l < NL; ++l) {
                if (l == 1 && !has_b) continue;
                if (MODE == M_GLOBAL_FREE) {
                    if (P.last_column_free) {            // H(0, n)
                        const int32_t x = border(P, P.first_row_free, n[l]);
                        if (better(x, 0, n[l], cs[l], ci[l], cj[l])) { cs[l] = x; ci[l] = 0; cj[l] = n[l]; }
                    }
                    if (P.last_row_free) {               // H(m, 0)
                        const int32_t x = border(P, P.first_column_free, m[l]);
                        if (better(x, m[l], 0, cs[l], ci[l], cj[l])) { cs[l] = x; ci[l] = m[l]; cj[l] = 0; }
                    }
                }
                pa_result r;
                r.score = cs[l];
                r.end1 = ci[l];
                r.end2 = cj[l];
                r.width = V::WIDTH;
                r.flags = L.rerun ? PA_RESULT_RERUN : 0;
                r.band_rounds = 0;
                if (MODE == M_LOCAL && cs[l] <= 0) { r.end1 = 0; r.end2 = 0; }
                if (clamp16 && (int64_t)cs[l] <= (int64_t)P.floor16 + (int64_t)P.smax * min(m[l], n[l])) {
                    // a clamp may have reached this result: recompute the pair in s32
                    const uint32_t slot = atomicAdd(L.rerun_count, 1u);
                    L.rerun_list[slot] = id[l];
                    continue;
                }
                L.out[id[l]] = r;
            }
        }
        __syncwarp(gmask);
    }
}

}  // namespace pa
