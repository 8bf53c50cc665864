// pa_dp.cuh -- the affine-gap (Gotoh) score DP kernel for sm_103a.
//
// One "group" of G consecutive lanes of a warp (G = 1, 2, ..., 32) computes the
// DP matrix of two pairs at once in s16x2 lanes (pair A in the low halfword,
// pair B in the high halfword of every register) or of one pair in s32 lanes.
// The recurrence is the reference's compute_cell
// (include/pairwise_aligner/affine/affine_dp_algorithm.hpp:149-155):
//     best = max(diag + s(a,b), vgap, hgap)          [local: max(diag + s, 0) first,
//                                                     dp_matrix_local.hpp:39-47]
//     vgap' = max(vgap + ext, best + open + ext);  hgap' = max(hgap + ext, best + open + ext)
// with the border cells of affine_initialisation_strategy.hpp:38-51.
//
// Layout of the work: sequence2 ("held") runs down the rows, sequence1
// ("streamed") along the columns.  Thread t of a group holds RA consecutive rows
// of the current pass in registers (H and the rightward gap per row, plus a
// byte-permute selector that encodes the row's base); the group sweeps the
// columns as an anti-diagonal wavefront: at step s thread t computes column
// s - t + 1 and hands the bottom H and the downward gap of its strip to thread
// t+1 with __shfl_up_sync.  Rows beyond G*R are covered by further passes; the
// last thread spills its bottom row per column to the pass-boundary scratch
// (8 bytes per column), where thread 0 of the next pass reads it.
//
// Instruction budget (sm_103: PRMT, LOP3 and the 3-operand DPX forms take two
// ALU issue slots, the 2-operand __vmaxs2 one, integer adds go to another pipe);
// per register (two cells of s16x2 lanes):
//     s  = PRMT(table_a, table_b, selector)            score of both lanes
//     t  = VIADDMAX(diag, s, hgap)                      max(diag + s, hgap)
//     H  = VIMAX3(t, vgap, clamp)                       local 0 / global floor
//     Ho = H - |open+ext|                               IADD, borrow free
//     hgap = VMAX(hgap - |ext|, Ho);  vgap = VMAX(vgap - |ext|, Ho)
// s16x2 values are stored with a per-group offset K so that every halfword
// stays in [0, 32767]: subtracting a constant never borrows across halfwords and
// signed DPX comparisons stay valid.  Local: true 0 == K.  Global: the clamp at
// 2048 is a floor; a result above floor + smax * min(m, n) cannot have been
// influenced by a clamp and is exact, anything else is recomputed in s32.
//
// Tracking (the reference trackers, tracker/*.hpp):
//   local  -- running column maximum per strip; on a strict improvement the
//             strip's H column is stored to shared memory, so the end is the
//             smallest column i, then the smallest row j of the maximum.
//   global -- H(m, n) is read where it is computed; free trailing gaps also
//             scan the last row (i = m) and the last column (j = n).
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
        const uint32_t h = (uint16_t)(int16_t)x;
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
    static __device__ __forceinline__ uint32_t hmax(uint32_t t, uint32_t e, uint32_t clamp)
    {
        return __vimax3_s16x2(t, e, clamp);
    }
    static __device__ __forceinline__ uint32_t max2(uint32_t a, uint32_t b) { return __vmaxs2(a, b); }
    static __device__ __forceinline__ uint32_t max3(uint32_t a, uint32_t b, uint32_t c)
    {
        return __vimax3_s16x2(a, b, c);
    }
    // x - c in both halfwords; cabs2 = |c| * 0x10001; halfwords of x are >= |c|.
    static __device__ __forceinline__ uint32_t subc(uint32_t x, uint32_t cabs2) { return x - cabs2; }
    static __device__ __forceinline__ uint32_t cabs(int32_t c) { return (uint32_t)(c < 0 ? -c : c) * 0x10001u; }
    static __device__ __forceinline__ bool improved(uint32_t x, int l) { return (l ? (x >> 16) : (x & 0xffffu)) != 0; }
    // Byte-permute selector of a held row.  Low halfword <- table byte `ca` of lane A
    // (bytes 0-3) sign-extended, high halfword <- byte 4+cb of lane B.  A padded row
    // (code < 0) replicates the sign of a table byte: its score is 0 or -1.
    static __device__ __forceinline__ uint32_t selector(int ca, int cb)
    {
        const uint32_t lo = ca < 0 ? 0x88u : ((uint32_t)ca | (((uint32_t)ca | 8u) << 4));
        const uint32_t hi = cb < 0 ? 0xCCu : ((4u + (uint32_t)cb) | (((4u + (uint32_t)cb) | 8u) << 4));
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
        return (uint32_t)max((int)(a + b), (int)c);
    }
    static __device__ __forceinline__ uint32_t hmax(uint32_t t, uint32_t e, uint32_t clamp)
    {
        return (uint32_t)__vimax3_s32((int)t, (int)e, (int)clamp);
    }
    static __device__ __forceinline__ uint32_t max2(uint32_t a, uint32_t b) { return (uint32_t)max((int)a, (int)b); }
    static __device__ __forceinline__ uint32_t max3(uint32_t a, uint32_t b, uint32_t c)
    {
        return (uint32_t)__vimax3_s32((int)a, (int)b, (int)c);
    }
    static __device__ __forceinline__ uint32_t subc(uint32_t x, uint32_t cabs) { return x - cabs; }
    static __device__ __forceinline__ uint32_t cabs(int32_t c) { return (uint32_t)(c < 0 ? -c : c); }
    static __device__ __forceinline__ bool improved(uint32_t x, int) { return x != 0; }
    static __device__ __forceinline__ uint32_t selector(int ca, int)
    {
        if (ca < 0) return 0x8888u;
        const uint32_t c = (uint32_t)ca, s = c | 8u;
        return c | (s << 4) | (s << 8) | (s << 12);
    }
};

// (score, end1, end2) candidate order: higher score, then smaller end1, then smaller end2.
__device__ __forceinline__ bool better(int32_t s, int32_t i, int32_t j, int32_t bs, int32_t bi, int32_t bj)
{
    return s > bs || (s == bs && (i < bi || (i == bi && j < bj)));
}

constexpr int kChunk = 4;      // granularity of the rows a thread holds in a short last pass
constexpr int kBlock = 256;    // threads per block of every DP launch

// Everything one group needs to know about its current work unit.
struct GroupWork {
    uint32_t id[2];
    uint64_t qoff[2], toff[2];
    int32_t m[2], n[2];
    int32_t ms, nh, passes, rows_full;
    bool has_b;
    uint32_t K, CLAMP;         // offset and clamp of the stored values
    int32_t Kt, clampt;        // the same as true-score integers
    int32_t floor_true;        // global s16 lanes: true value of the clamp
    const uint32_t *qt[2];
    Cell *buf;
    int32_t cs[2], ci[2], cj[2];   // candidate (score, end1, end2) per lane
};

template <class V>
__device__ __forceinline__ uint32_t stored(const GroupWork &w, int32_t true_value)
{
    int32_t x = true_value + w.Kt;
    if (V::LANES == 2) x = max(x, w.clampt);
    return V::splat(x);
}

// VAR bit 0: short-chain form of the vertical gap; bit 2: branch-free top input for
// thread 0 and an L1 prefetch of the score tables eight columns ahead.
template <class V, int R, int RA, int MODE, bool GEN, int VAR>
__device__ __forceinline__ void run_pass(const DpLaunch &L, const DpParams &P, GroupWork &w, int p, int t, int G,
                                         unsigned gmask, uint4 *snap)
{
    constexpr int NL = V::LANES;
    const int32_t j0 = p * w.rows_full + t * RA;   // rows j0+1 .. j0+RA (1-based)
    const uint32_t GOEA = V::cabs(P.gap_open + P.gap_ext);
    const uint32_t EXTA = V::cabs(P.gap_ext);
    const uint32_t CLAMP = w.CLAMP;
    const uint32_t CLAMPG = V::LANES == 2 ? V::subc(CLAMP, GOEA) : (uint32_t)max((int)CLAMP, INT32_MIN + 65536) - GOEA;

    uint32_t H[RA], Fr[RA], Sel[RA];
#pragma unroll
    for (int k = 0; k < RA; ++k) {
        const int32_t j = j0 + k;                     // 0-based index into sequence2
        int c[2];
#pragma unroll
        for (int l = 0; l < 2; ++l) {
            if (GEN) c[l] = (j < w.n[l]) ? (int)L.seq2[w.toff[l] + j] : 0x100;
            else c[l] = (j < w.n[l]) ? (int)dna_code(L.seq2[w.toff[l] + j]) : -1;
        }
        Sel[k] = GEN ? (uint32_t)c[0] : V::selector(c[0], c[1]);
        H[k] = stored<V>(w, border(P, P.first_row_free, (int64_t)j + 1));
        Fr[k] = V::subc(H[k], GOEA);
    }
    uint32_t prevH = stored<V>(w, border(P, P.first_row_free, j0));
    uint32_t topH = prevH;                              // thread 0, pass 0: H(i-1, 0)
    const uint32_t step1 = P.first_column_free ? 0u : V::cabs(P.gap_open + P.gap_ext);
    const uint32_t stepn = P.first_column_free ? 0u : EXTA;
    uint32_t outH = 0, outE = 0, best = w.K;
    int32_t bi[2] = {0, 0};
    int32_t own_k[2], own_t[2];
    bool own_p[2];
#pragma unroll
    for (int l = 0; l < 2; ++l) {                     // where row n[l] lives
        const int32_t pl = (w.n[l] - 1) / w.rows_full;
        own_p[l] = (pl == p);
        const int32_t r = (w.n[l] - 1) - pl * w.rows_full;
        own_t[l] = r / RA;
        own_k[l] = r - own_t[l] * RA;
    }
    const int32_t ms = w.ms;
    const bool last_pass = p + 1 == w.passes;
    // next column's score tables, loaded one step ahead
    uint32_t nta = 0, ntb = 0;
    auto load_tables = [&](int32_t col, uint32_t &a, uint32_t &b) {
        if (GEN) {
            a = (col <= w.m[0]) ? (uint32_t)L.seq1[w.qoff[0] + col - 1] : 0x200u;
            b = a;
        } else {
            a = __ldg(w.qt[0] + min(col - 1, w.m[0]));
            b = NL == 2 ? __ldg(w.qt[1] + min(col - 1, w.m[1])) : a;
        }
    };
    Cell nbuf = Cell{0u, 0u};                        // thread 0, pass > 0: next boundary cell
    if (t == 0 && p > 0) nbuf = w.buf[1];
    constexpr bool TUNED = (VAR & 4) != 0;
    const bool first_thread = t == 0;
    const bool top_border = first_thread && p == 0;
    const bool top_buffer = first_thread && p > 0;
    auto step = [&](int32_t i, bool active) {
        uint32_t upH = __shfl_up_sync(gmask, outH, 1, G);
        uint32_t upE = __shfl_up_sync(gmask, outE, 1, G);
        if (!active) return;
        if (TUNED) {
            // every lane computes the border candidate; thread 0 selects it (no divergence)
            const uint32_t nt = V::max2(V::subc(topH, i == 1 ? step1 : stepn), CLAMP);
            topH = top_border ? nt : topH;
            const Cell c = nbuf;
            if (top_buffer && i < ms) nbuf = w.buf[i + 1];
            upH = top_border ? nt : (top_buffer ? c.h : upH);
            upE = top_border ? V::subc(nt, GOEA) : (top_buffer ? c.e : upE);
            if (!GEN && i + 8 <= ms) {
                asm volatile("prefetch.global.L1 [%0];" ::"l"(w.qt[0] + min(i + 7, w.m[0])));
                if (NL == 2) asm volatile("prefetch.global.L1 [%0];" ::"l"(w.qt[1] + min(i + 7, w.m[1])));
            }
        } else if (t == 0) {
            if (p == 0) {
                topH = V::max2(V::subc(topH, i == 1 ? step1 : stepn), CLAMP);
                upH = topH;
                upE = V::subc(topH, GOEA);
            } else {
                upH = nbuf.h;
                upE = nbuf.e;
                if (i < ms) nbuf = w.buf[i + 1];
            }
        }
        const uint32_t ta = nta, tb = ntb;
        if (i < ms) load_tables(i + 1, nta, ntb);
        uint32_t diag = prevH, Ed = upE;
#pragma unroll
        for (int k = 0; k < RA; ++k) {
            uint32_t sc;
            if (GEN) {
                const uint32_t x = Sel[k];
                sc = (x == ta) ? (uint32_t)P.match : (((x | ta) >> 8) ? (uint32_t)P.spad : (uint32_t)P.mismatch);
            } else {
                sc = prmt(ta, tb, Sel[k]);
            }
            const uint32_t tt = V::addmax(diag, sc, Fr[k]);
            diag = H[k];
            if ((VAR & 8) != 0) {
                // vgap' = max(vgap + ext, t + open + ext, clamp + open + ext): the H term of the
                // vertical gap is dominated, so the serial chain is one IADD and one VIMAX3
                const uint32_t h = V::hmax(tt, Ed, CLAMP);
                H[k] = h;
                Fr[k] = V::max2(V::subc(Fr[k], EXTA), V::subc(h, GOEA));
                Ed = V::max3(V::subc(Ed, EXTA), V::subc(tt, GOEA), CLAMPG);
            } else if ((VAR & 1) == 0) {
                const uint32_t h = V::hmax(tt, Ed, CLAMP);
                H[k] = h;
                const uint32_t hoe = V::subc(h, GOEA);
                Fr[k] = V::max2(V::subc(Fr[k], EXTA), hoe);
                Ed = V::max2(V::subc(Ed, EXTA), hoe);
            } else {
                // vgap' = max(vgap + ext, max(t, clamp) + open + ext): H leaves the serial chain
                const uint32_t x = V::max2(tt, CLAMP);
                const uint32_t h = V::max2(x, Ed);
                H[k] = h;
                Fr[k] = V::max2(V::subc(Fr[k], EXTA), V::subc(h, GOEA));
                Ed = V::max2(V::subc(Ed, EXTA), V::subc(x, GOEA));
            }
        }
        prevH = upH;
        outH = H[RA - 1];
        outE = Ed;
        if (t == G - 1 && !last_pass) w.buf[i] = Cell{outH, outE};

        if (MODE == M_LOCAL) {
            uint32_t cm = H[0];
#pragma unroll
            for (int k = 1; k < RA; k += 2) cm = V::max3(cm, H[k], H[k + 1 < RA ? k + 1 : k]);
            const uint32_t nb = V::max2(best, cm);
            const uint32_t x = nb ^ best;
            best = nb;
#pragma unroll
            for (int l = 0; l < NL; ++l) {
                if (x != 0u && V::improved(x, l)) {
                    bi[l] = i;
#pragma unroll
                    for (int v = 0; v < RA / 4; ++v)
                        snap[(l * (R / 4) + v) * kBlock + threadIdx.x] =
                            make_uint4(H[4 * v], H[4 * v + 1], H[4 * v + 2], H[4 * v + 3]);
                }
            }
        } else {
#pragma unroll
            for (int l = 0; l < NL; ++l) {
                if (l == 1 && !w.has_b) continue;
                if (MODE == M_GLOBAL_FREE && P.last_column_free && own_p[l] && t == own_t[l] && i <= w.m[l]) {
                    uint32_t v = H[0];
#pragma unroll
                    for (int k = 1; k < RA; ++k)
                        if (own_k[l] == k) v = H[k];
                    const int32_t xs = V::get(v, l) - w.Kt;
                    if (better(xs, i, w.n[l], w.cs[l], w.ci[l], w.cj[l])) { w.cs[l] = xs; w.ci[l] = i; w.cj[l] = w.n[l]; }
                }
                if (i == w.m[l]) {
                    if (MODE == M_GLOBAL_FREE && P.last_row_free) {
#pragma unroll
                        for (int k = 0; k < RA; ++k) {
                            const int32_t j = j0 + k + 1;
                            if (j <= w.n[l]) {
                                const int32_t xs = V::get(H[k], l) - w.Kt;
                                if (better(xs, i, j, w.cs[l], w.ci[l], w.cj[l])) { w.cs[l] = xs; w.ci[l] = i; w.cj[l] = j; }
                            }
                        }
                    } else if (own_p[l] && t == own_t[l]) {
                        uint32_t v = H[0];
#pragma unroll
                        for (int k = 1; k < RA; ++k)
                            if (own_k[l] == k) v = H[k];
                        const int32_t xs = V::get(v, l) - w.Kt;
                        if (better(xs, i, w.n[l], w.cs[l], w.ci[l], w.cj[l])) { w.cs[l] = xs; w.ci[l] = i; w.cj[l] = w.n[l]; }
                    }
                }
            }
        }
    };
    // fill: thread t starts at step t (steps 0..G-1); steady: every thread active; drain
    if (t == 0) load_tables(1, nta, ntb);
    const int32_t fill_end = min(G, ms + G - 1);
    int s = 0;
    for (; s < fill_end; ++s) {
        const int32_t i = s - t + 1;
        if (i == 1 && t > 0) load_tables(1, nta, ntb);
        step(i, i >= 1 && i <= ms);
    }
    for (; s < ms; ++s) step(s - t + 1, true);
    for (; s < ms + G - 1; ++s) {
        const int32_t i = s - t + 1;
        step(i, i >= 1 && i <= ms);
    }
    if (MODE == M_LOCAL) {
#pragma unroll
        for (int l = 0; l < NL; ++l) {
            const int32_t b = V::get(best, l);
            if (b > w.Kt) {
                int32_t kk = 0;
                for (int v = RA / 4 - 1; v >= 0; --v) {
                    const uint4 q = snap[(l * (R / 4) + v) * kBlock + threadIdx.x];
                    if (V::get(q.w, l) == b) kk = 4 * v + 3;
                    if (V::get(q.z, l) == b) kk = 4 * v + 2;
                    if (V::get(q.y, l) == b) kk = 4 * v + 1;
                    if (V::get(q.x, l) == b) kk = 4 * v;
                }
                const int32_t xs = b - w.Kt, j = j0 + kk + 1;
                if (better(xs, bi[l], j, w.cs[l], w.ci[l], w.cj[l])) { w.cs[l] = xs; w.ci[l] = bi[l]; w.cj[l] = j; }
            }
        }
    }
}

// GEN = byte-compare scoring (any bytes, any int32 scores), always with L32 lanes.
template <class V, int R, int MODE, bool GEN, int VAR, int MINB = 2>
__global__ void __launch_bounds__(kBlock, MINB) dp_kernel(DpLaunch L, DpParams P)
{
    static_assert(R % kChunk == 0 && R <= 32, "R must be a multiple of the chunk");
    constexpr int NL = V::LANES;
    __shared__ uint4 snap_store[MODE == M_LOCAL ? NL * (R / 4) * kBlock : 1];
    const int lane = threadIdx.x & 31;
    const int G = L.G;
    const int t = lane & (G - 1);
    const int g = lane / G;
    const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (g * G));
    const uint32_t count = *L.count_ptr;
    const uint32_t *order = L.order + *L.begin_ptr;
    const uint32_t ppw = (uint32_t)(32 / G) * NL;   // pairs per warp unit
    const uint32_t n_units = (count + ppw - 1) / ppw;

    for (;;) {
        uint32_t u = 0;
        if (lane == 0) u = atomicAdd(L.unit_counter, 1u);
        u = __shfl_sync(0xffffffffu, u, 0);
        if (u >= n_units) break;
        u = n_units - 1 - u;                         // largest shapes first
        const uint32_t first = u * ppw + (uint32_t)g * NL;
        if (first >= count) continue;                // idle group in the last unit

        GroupWork w;
        w.id[0] = order[first];
        w.has_b = NL == 2 && first + 1 < count;
        w.id[1] = w.has_b ? order[first + 1] : w.id[0];
#pragma unroll
        for (int l = 0; l < 2; ++l) {
            w.qoff[l] = L.off1[w.id[l]];
            w.m[l] = (int32_t)(L.off1[w.id[l] + 1] - w.qoff[l]);
            w.toff[l] = L.off2[w.id[l]];
            w.n[l] = (int32_t)(L.off2[w.id[l] + 1] - w.toff[l]);
            w.qt[l] = L.qtab + w.qoff[l] + w.id[l];
            w.cs[l] = MODE == M_LOCAL ? 0 : INT32_MIN;
            w.ci[l] = 0;
            w.cj[l] = 0;
        }
        w.ms = NL == 2 ? max(w.m[0], w.m[1]) : w.m[0];
        w.nh = NL == 2 ? max(w.n[0], w.n[1]) : w.n[0];
        w.rows_full = G * R;
        w.passes = (w.nh + w.rows_full - 1) / w.rows_full;
        const uint32_t owner = (NL == 2 && w.m[1] > w.m[0]) ? w.id[1] : w.id[0];
        w.buf = L.boundary + (L.off1[owner] + owner);
        if (NL == 2) {
            if (MODE == M_LOCAL) {
                w.Kt = 2048;
                w.clampt = 2048;
                w.floor_true = 0;
            } else {
                const int32_t ub = P.smax * max(min(w.m[0], w.n[0]), min(w.m[1], w.n[1]));
                w.Kt = 32767 - 512 - ub;
                w.clampt = 2048;
                w.floor_true = 2048 - w.Kt;
            }
            w.K = V::splat(w.Kt);
            w.CLAMP = V::splat(w.clampt);
        } else {
            w.Kt = 0;
            w.clampt = MODE == M_LOCAL ? 0 : INT32_MIN;
            w.floor_true = INT32_MIN;
            w.K = 0;
            w.CLAMP = (uint32_t)w.clampt;
        }

        for (int p = 0; p < w.passes; ++p) {
            const int32_t rem = w.nh - p * w.rows_full;
            const int32_t rpt = rem >= w.rows_full ? R : ((rem + G * kChunk - 1) / (G * kChunk)) * kChunk;
            switch (rpt / kChunk) {
            case 1: run_pass<V, R, 4, MODE, GEN, VAR>(L, P, w, p, t, G, gmask, snap_store); break;
            case 2: run_pass<V, R, 8, MODE, GEN, VAR>(L, P, w, p, t, G, gmask, snap_store); break;
            case 3: run_pass<V, R, 12, MODE, GEN, VAR>(L, P, w, p, t, G, gmask, snap_store); break;
            default: run_pass<V, R, R, MODE, GEN, VAR>(L, P, w, p, t, G, gmask, snap_store); break;
            }
            __syncwarp(gmask);
        }

        // group reduction of the candidates
#pragma unroll
        for (int l = 0; l < NL; ++l) {
            for (int off = G >> 1; off >= 1; off >>= 1) {
                const int32_t os = __shfl_xor_sync(gmask, w.cs[l], off, G);
                const int32_t oi = __shfl_xor_sync(gmask, w.ci[l], off, G);
                const int32_t oj = __shfl_xor_sync(gmask, w.cj[l], off, G);
                if (better(os, oi, oj, w.cs[l], w.ci[l], w.cj[l])) { w.cs[l] = os; w.ci[l] = oi; w.cj[l] = oj; }
            }
        }
        if (t == 0) {
#pragma unroll
            for (int l = 0; l < NL; ++l) {
                if (l == 1 && !w.has_b) continue;
                if (MODE == M_GLOBAL_FREE) {
                    if (P.last_column_free) {            // H(0, n)
                        const int32_t x = border(P, P.first_row_free, w.n[l]);
                        if (better(x, 0, w.n[l], w.cs[l], w.ci[l], w.cj[l])) { w.cs[l] = x; w.ci[l] = 0; w.cj[l] = w.n[l]; }
                    }
                    if (P.last_row_free) {               // H(m, 0)
                        const int32_t x = border(P, P.first_column_free, w.m[l]);
                        if (better(x, w.m[l], 0, w.cs[l], w.ci[l], w.cj[l])) { w.cs[l] = x; w.ci[l] = w.m[l]; w.cj[l] = 0; }
                    }
                }
                pa_result r;
                r.score = w.cs[l];
                r.end1 = w.ci[l];
                r.end2 = w.cj[l];
                r.width = V::WIDTH;
                r.flags = L.rerun ? PA_RESULT_RERUN : 0;
                r.band_rounds = 0;
                if (MODE == M_LOCAL && w.cs[l] <= 0) { r.end1 = 0; r.end2 = 0; }
                if (NL == 2 && MODE != M_LOCAL &&
                    (int64_t)w.cs[l] <= (int64_t)w.floor_true + (int64_t)P.smax * min(w.m[l], w.n[l])) {
                    // a clamp may have reached this result: recompute the pair in s32
                    const uint32_t slot = atomicAdd(L.rerun_count, 1u);
                    L.rerun_list[slot] = w.id[l];
                    continue;
                }
                L.out[w.id[l]] = r;
            }
        }
        __syncwarp(gmask);
    }
}

}  // namespace pa
