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
// signed DPX comparisons stay valid.  Local: true 0 == K.  Global modes store the
// column-shifted H'(i, j) = H(i, j) - smax * i, which no step increases, and clamp it
// at a floor (stored 2048): a cell that met the clamp stays at or below the floor, so a
// result whose H' is above the floor is exact; anything else is recomputed in s32.
//
// Tracking (the reference trackers, tracker/*.hpp):
//   local  -- running column maximum per strip; on a strict improvement the
//             strip's H column is stored to shared memory, so the end is the
//             smallest column i, then the smallest row j of the maximum.
//   global -- H(m, n) is read where it is computed; free trailing gaps also
//             scan the last row (i = m) and the last column (j = n).
#pragma once
#include <cooperative_groups.h>
#include <cuda/atomic>

#include "pa_common.cuh"

namespace pa {

enum Mode : int { M_LOCAL = 0, M_GLOBAL = 1, M_GLOBAL_FREE = 2, M_LABEL_FWD = 3, M_LABEL_REV = 4, M_BAND = 5 };

// "Minus infinity" of band mode: cells outside the band.  s16x2 lanes use the
// clamp floor (its exactness check covers it), s32 lanes a value far below any
// score that gaps can still be subtracted from without wrapping.
constexpr int32_t kNeg32 = -(1 << 30);

// Checkpoint columns of the band labels: i_c = c * m / 9, c = 1..8.
__device__ __forceinline__ int32_t checkpoint_col(int c, int32_t m) { return (int32_t)(((int64_t)(c + 1) * m) / 9); }

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
    Cell *buf;                     // single-group passes read and write this boundary row
    Cell *bin, *bout;              // the boundary row a pass reads (from the pass above) and writes
    int *prog_in, *prog_out;       // CTA mode: progress of the pass above / of this pass
    int32_t base_in, base_out;     // progress value of column 0 of those passes
    int32_t seen;                  // last progress value thread 0 observed
    bool wait_failed;              // a progress wait of this unit ran out (thread 0 of a group)
    int32_t cs[2], ci[2], cj[2];   // candidate (score, end1, end2) per lane
    int32_t lb_v[8], lb_j[8];      // label mode: best forward + reverse score per checkpoint and its row
    // band mode: columns ibase+1 .. iend of the current pass; thread 0's first diagonal
    int32_t ibase, iend;
    uint32_t diag0;
    int32_t ub[2];                 // largest bound on a path that leaves the band, per lane
    unsigned long long cells;      // band cells computed (statistics)
};

// CTA mode: the groups of a block work on consecutive passes of one pair; the
// group of pass p waits (thread 0, before reading boundary column c) until the
// pass above has published column c.  Waits are bounded (DpLaunch::spin_limit polls
// after the first look, default kSpinLimit); a wait that runs out sets an error bit,
// the pair's result is written as an error (PA_RESULT_ERROR) and the kernel carries on.
constexpr uint32_t kSpinLimit = 1u << 24;
constexpr uint32_t kErrWaitTimeout = 1u;

// SYNC scope of a kernel: 0 none (one group per pair), 1 the block (CTA mode), 2 the
// thread-block cluster (cluster mode: flags may live in another block's shared memory).
__device__ __forceinline__ int load_acquire_cluster(const int *p)
{
    int v;
    asm volatile("ld.acquire.cluster.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void store_release_cluster(int *p, int v)
{
    asm volatile("st.release.cluster.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

template <int SCOPE>
__device__ __forceinline__ int32_t wait_progress(int *flag, int32_t need, uint32_t *err, uint32_t limit)
{
    for (uint32_t it = 0;; ++it) {
        const int v = SCOPE == 2 ? load_acquire_cluster(flag)
                                 : cuda::atomic_ref<int, cuda::thread_scope_block>(*flag).load(cuda::memory_order_acquire);
        if (v >= need) return v;
        if (it >= limit) break;
        if (it >= 64) __nanosleep(64);
    }
    if (err) atomicOr(err, kErrWaitTimeout);
    return INT32_MAX;
}

template <int SCOPE>
__device__ __forceinline__ void publish_progress(int *flag, int32_t v)
{
    if (SCOPE == 2) store_release_cluster(flag, v);
    else cuda::atomic_ref<int, cuda::thread_scope_block>(*flag).store(v, cuda::memory_order_release);
}

// A boundary cell written by another pass: in cluster mode the writer may sit on another SM,
// so the read goes to L2 (no stale L1 line of an earlier pass that used the same ring row).
template <int SCOPE>
__device__ __forceinline__ Cell load_cell(const Cell *p)
{
    if (SCOPE == 2) {
        const uint2 v = __ldcg(reinterpret_cast<const uint2 *>(p));
        return Cell{v.x, v.y};
    }
    return *p;
}

// Upper bound on the score of a path that enters cell (i, j) from inside the band
// and then runs to (m, n): `gapv` is the score of entering in a gap state, `diagv`
// by a diagonal step.  From (i, j) at most min(m - i, n - j) diagonal steps gain
// smax each, and the diagonal changes by d = |(n - j) - (m - i)|, which costs at
// least d gap extensions (the gap may continue the entering one) or, after a
// diagonal step, one gap open and d extensions.
__device__ __forceinline__ int32_t exit_bound(const DpParams &P, int32_t gapv, int32_t diagv, int32_t i, int32_t j,
                                              int32_t m, int32_t n)
{
    const int64_t ri = m - i, rj = n - j;
    const int64_t d = ri > rj ? ri - rj : rj - ri;
    const int64_t gain = (int64_t)P.smax * (ri < rj ? ri : rj);
    const int64_t g = gapv + gain + (int64_t)P.gap_ext * d;
    const int64_t h = diagv + gain + (d ? (int64_t)P.gap_open + (int64_t)P.gap_ext * d : 0);
    const int64_t b = g > h ? g : h;
    return b > INT32_MAX ? INT32_MAX : (b < INT32_MIN ? INT32_MIN : (int32_t)b);
}

template <class V>
__device__ __forceinline__ uint32_t stored(const GroupWork &w, int32_t true_value)
{
    int32_t x = true_value + w.Kt;
    if (V::LANES == 2) x = max(x, w.clampt);
    return V::splat(x);
}

// Maximum of x[0..N) as a tree of three-operand maxima (depth log3 N, not N/2).
template <class V, int N>
__device__ __forceinline__ uint32_t tree_max(const uint32_t *x)
{
    if constexpr (N == 1) {
        return x[0];
    } else if constexpr (N == 2) {
        return V::max2(x[0], x[1]);
    } else if constexpr (N == 3) {
        return V::max3(x[0], x[1], x[2]);
    } else {
        constexpr int M = (N + 2) / 3;
        uint32_t y[M];
#pragma unroll
        for (int k = 0; k < M; ++k) {
            const int a = 3 * k, left = N - a;
            y[k] = left >= 3 ? V::max3(x[a], x[a + 1], x[a + 2]) : (left == 2 ? V::max2(x[a], x[a + 1]) : x[a]);
        }
        return tree_max<V, M>(y);
    }
}

// VAR bit 0: short-chain form of the vertical gap; bit 2: branch-free top input for
// thread 0 and an L1 prefetch of the score tables eight columns ahead.
template <class V, int R, int RA, int MODE, bool GEN, int VAR, int SYNC = 0>
__device__ __forceinline__ void run_pass(const DpLaunch &L, const DpParams &P, GroupWork &w, int p, int t, int G,
                                         unsigned gmask, uint4 *snap)
{
    constexpr int NL = V::LANES;
    const int32_t j0 = p * w.rows_full + t * RA;   // rows j0+1 .. j0+RA (1-based)
    // vertical steps (along sequence2) cost the gap scores; horizontal steps (to the next
    // column) also subtract the column shift of global modes (P.shift = smax, local 0)
    const uint32_t GOEA = V::cabs(P.gap_open + P.gap_ext);
    const uint32_t EXTA = V::cabs(P.gap_ext);
    const uint32_t GOEH = V::cabs(P.gap_open + P.gap_ext - P.shift);
    const uint32_t EXTH = V::cabs(P.gap_ext - P.shift);
    const uint32_t CLAMP = w.CLAMP;
    const uint32_t CLAMPG = V::LANES == 2 ? V::subc(CLAMP, GOEA) : (uint32_t)max((int)CLAMP, INT32_MIN + 65536) - GOEA;

    constexpr bool BAND = MODE == M_BAND;
    constexpr bool SHIFTED = MODE != M_LOCAL;       // H is stored as H - shift * column
    const int32_t ibase = BAND ? w.ibase : 0;      // the pass sweeps columns ibase+1 .. iend
    const int32_t iend = BAND ? w.iend : w.ms;
    const int32_t msw = iend - ibase;
    const bool left_out = BAND && ibase > 0;        // column ibase lies outside the band
    const uint32_t NEGV = V::LANES == 2 ? CLAMP : (uint32_t)kNeg32;

    // byte-compare kernels with a substitution matrix: held rows carry the symbol's rank,
    // streamed columns rank * dim (both below 0x400 for dim <= 32); 0x400 / 0x800 mark
    // padding (and an invalid symbol, which the classifier reports as an error)
    const bool MAT = GEN && L.matrix != nullptr;
    auto rank_of = [&](uint8_t b) -> int { return (int)__ldg(L.rank_map + b); };

    uint32_t H[RA], Fr[RA], Sel[RA];
#pragma unroll
    for (int k = 0; k < RA; ++k) {
        const int32_t j = j0 + k;                     // 0-based index into sequence2
        int c[2];
#pragma unroll
        for (int l = 0; l < 2; ++l) {
            if (GEN) {
                c[l] = (j < w.n[l]) ? (int)L.seq2[w.toff[l] + j] : 0x100;
                if (MAT) {
                    const int r = c[l] < 0x100 ? rank_of((uint8_t)c[l]) : -1;
                    c[l] = r < 0 ? 0x400 : r;
                }
            } else {
                c[l] = (j < w.n[l]) ? (int)dna_code(L.seq2[w.toff[l] + j]) : -1;
            }
        }
        Sel[k] = GEN ? (uint32_t)c[0] : V::selector(c[0], c[1]);
        H[k] = left_out ? NEGV : stored<V>(w, border(P, P.first_row_free, (int64_t)j + 1));
        Fr[k] = V::subc(H[k], GOEH);
    }
    uint32_t prevH = left_out ? (t == 0 ? w.diag0 : NEGV) : stored<V>(w, border(P, P.first_row_free, j0));
    uint32_t topH = prevH;                              // thread 0, pass 0: H(i-1, 0)
    uint32_t top_last = NEGV;                           // band: thread 0's top input at column iend
    const uint32_t step1 = V::cabs((P.first_column_free ? 0 : P.gap_open + P.gap_ext) - P.shift);
    const uint32_t stepn = V::cabs((P.first_column_free ? 0 : P.gap_ext) - P.shift);
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
    const bool last_pass = p + 1 == w.passes;
    // next column's score tables, loaded one step ahead
    uint32_t nta = 0, ntb = 0;
    auto load_tables = [&](int32_t col, uint32_t &a, uint32_t &b) {
        if (GEN) {
            a = (col <= w.m[0]) ? (uint32_t)L.seq1[w.qoff[0] + col - 1] : 0x200u;
            if (MAT) {
                const int r = a < 0x200u ? rank_of((uint8_t)a) : -1;
                a = r < 0 ? 0x800u : (uint32_t)(r * L.mdim);
            }
            b = a;
        } else {
            a = __ldg(w.qt[0] + min(col - 1, w.m[0]));
            b = NL == 2 ? __ldg(w.qt[1] + min(col - 1, w.m[1])) : a;
        }
    };
    // thread 0, pass > 0: the next boundary cell (and in cluster mode, where the cell comes
    // from L2, the one after it as well)
    constexpr bool PF2 = SYNC == 2;
    Cell nbuf = Cell{0u, 0u}, nbuf2 = Cell{0u, 0u};
    // thread 0 of a pass below the first reads the boundary row; in CTA mode it first
    // waits until the pass above has published the column
    auto ready = [&](int32_t col) {
        if (SYNC && w.seen < w.base_in + col) {
            w.seen = wait_progress<SYNC>(w.prog_in, w.base_in + col, L.error, L.spin_limit);
            if (w.seen == INT32_MAX) w.wait_failed = true;
        }
    };
    auto advance = [&](int32_t i) {                  // at column i < iend: fetch what column i + 1 needs
        if (PF2) {
            nbuf = nbuf2;
            if (i + 2 <= iend) {
                ready(i + 2);
                nbuf2 = load_cell<SYNC>(w.bin + i + 2);
            }
        } else {
            ready(i + 1);
            nbuf = load_cell<SYNC>(w.bin + i + 1);
        }
    };
    if (t == 0 && p > 0) {
        ready(ibase + 1);
        nbuf = load_cell<SYNC>(w.bin + ibase + 1);
        if (PF2 && ibase + 2 <= iend) {
            ready(ibase + 2);
            nbuf2 = load_cell<SYNC>(w.bin + ibase + 2);
        }
    }
    constexpr bool TUNED = (VAR & 4) != 0;
    constexpr bool SPARSE = (VAR & 16) != 0;        // prefetches once per 8 columns, boundary included
    constexpr bool TABLE_PF = (VAR & 32) == 0;      // L1 prefetch of the score tables 7 columns ahead
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
            if (top_buffer && i < iend) advance(i);
            upH = top_border ? nt : (top_buffer ? c.h : upH);
            upE = top_border ? V::subc(nt, GOEA) : (top_buffer ? c.e : upE);
            if (SPARSE) {
                // one prefetch per 8 columns: the score-table line 24 columns ahead, and for
                // thread 0 the boundary row 32 columns ahead (written by the pass above, it is
                // in L2 but not in this SM's L1)
                if ((i & 7) == 0) {
                    if (!GEN && i + 24 <= iend) {
                        asm volatile("prefetch.global.L1 [%0];" ::"l"(w.qt[0] + min(i + 24, w.m[0])));
                        if (NL == 2) asm volatile("prefetch.global.L1 [%0];" ::"l"(w.qt[1] + min(i + 24, w.m[1])));
                    }
                    if (!SYNC && top_buffer && i + 32 <= iend) asm volatile("prefetch.global.L1 [%0];" ::"l"(w.bin + i + 32));
                }
            } else if (TABLE_PF && !GEN && i + 8 <= iend) {
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
                if (i < iend) advance(i);
            }
        }
        if (BAND && i == iend) top_last = upH;
        const uint32_t ta = nta, tb = ntb;
        if (i < iend) load_tables(i + 1, nta, ntb);
        uint32_t diag = prevH, Ed = upE;
#pragma unroll
        for (int k = 0; k < RA; ++k) {
            uint32_t sc;
            if (GEN) {
                const uint32_t x = Sel[k];
                if (MAT)
                    sc = ((x | ta) >> 10) ? (uint32_t)(P.spad - P.shift) : (uint32_t)(__ldg(L.matrix + ta + x) - P.shift);
                else
                    sc = (x == ta) ? (uint32_t)(P.match - P.shift)
                                   : (((x | ta) >> 8) ? (uint32_t)(P.spad - P.shift) : (uint32_t)(P.mismatch - P.shift));
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
                Fr[k] = V::max2(V::subc(Fr[k], EXTH), V::subc(h, GOEH));
                Ed = V::max3(V::subc(Ed, EXTA), V::subc(tt, GOEA), CLAMPG);
            } else if ((VAR & 1) == 0) {
                const uint32_t h = V::hmax(tt, Ed, CLAMP);
                H[k] = h;
                const uint32_t hoe = V::subc(h, GOEA);
                Fr[k] = V::max2(V::subc(Fr[k], EXTH), SHIFTED ? V::subc(h, GOEH) : hoe);
                Ed = V::max2(V::subc(Ed, EXTA), hoe);
            } else {
                // vgap' = max(vgap + ext, max(t, clamp) + open + ext): H leaves the serial chain
                const uint32_t x = V::max2(tt, CLAMP);
                const uint32_t h = V::max2(x, Ed);
                H[k] = h;
                Fr[k] = V::max2(V::subc(Fr[k], EXTH), V::subc(h, GOEH));
                Ed = V::max2(V::subc(Ed, EXTA), V::subc(x, GOEA));
            }
        }
        prevH = upH;
        outH = H[RA - 1];
        outE = Ed;
        if (t == G - 1 && !last_pass) {
            w.bout[i] = Cell{outH, outE};
            if (SYNC && ((i & 7) == 0 || i == iend)) publish_progress<SYNC>(w.prog_out, w.base_out + i);
        }

        if (MODE == M_LABEL_FWD || MODE == M_LABEL_REV) {
            // forward: keep the checkpoint columns; reverse (sequences reversed): column i is
            // the forward column m - i, row j the forward row n - j
            const int32_t m0 = w.m[0], n0 = w.n[0];
            for (int c = 0; c < 8; ++c) {
                const int32_t col = MODE == M_LABEL_FWD ? checkpoint_col(c, m0) : m0 - checkpoint_col(c, m0);
                if (col != i) continue;
                int32_t *dc = L.dump + L.dump_off[w.id[0]] + (uint64_t)c * (n0 + 1);
                if (MODE == M_LABEL_FWD) {
                    if (t == 0 && p == 0) dc[0] = border(P, P.first_column_free, i);
#pragma unroll
                    for (int k = 0; k < RA; ++k)
                        if (j0 + k + 1 <= n0) dc[j0 + k + 1] = V::get(H[k], 0) - w.Kt + P.shift * i;
                } else {
#pragma unroll
                    for (int k = 0; k < RA; ++k) {
                        const int32_t jf = n0 - (j0 + k + 1);            // forward row
                        if (jf >= 0) {
                            const int32_t v = dc[jf] + V::get(H[k], 0) - w.Kt + P.shift * i;
                            if (v > w.lb_v[c] || (v == w.lb_v[c] && jf < w.lb_j[c])) { w.lb_v[c] = v; w.lb_j[c] = jf; }
                        }
                    }
                }
            }
        }
        if (MODE == M_LOCAL) {
            const uint32_t cm = tree_max<V, RA>(H);
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
                    const int32_t xs = V::get(v, l) - w.Kt + P.shift * i;
                    if (better(xs, i, w.n[l], w.cs[l], w.ci[l], w.cj[l])) { w.cs[l] = xs; w.ci[l] = i; w.cj[l] = w.n[l]; }
                }
                if (i == w.m[l]) {
                    if (MODE == M_GLOBAL_FREE && P.last_row_free) {
#pragma unroll
                        for (int k = 0; k < RA; ++k) {
                            const int32_t j = j0 + k + 1;
                            if (j <= w.n[l]) {
                                const int32_t xs = V::get(H[k], l) - w.Kt + P.shift * i;
                                if (better(xs, i, j, w.cs[l], w.ci[l], w.cj[l])) { w.cs[l] = xs; w.ci[l] = i; w.cj[l] = j; }
                            }
                        }
                    } else if (own_p[l] && t == own_t[l]) {
                        uint32_t v = H[0];
#pragma unroll
                        for (int k = 1; k < RA; ++k)
                            if (own_k[l] == k) v = H[k];
                        const int32_t xs = V::get(v, l) - w.Kt + P.shift * i;
                        if (better(xs, i, w.n[l], w.cs[l], w.ci[l], w.cj[l])) { w.cs[l] = xs; w.ci[l] = i; w.cj[l] = w.n[l]; }
                    }
                }
            }
        }
    };
    // fill: thread t starts at step t (steps 0..G-1); steady: every thread active; drain
    if (t == 0) load_tables(ibase + 1, nta, ntb);
    const int32_t fill_end = min(G, msw + G - 1);
    int s = 0;
    for (; s < fill_end; ++s) {
        const int32_t li = s - t + 1;
        if (li == 1 && t > 0) load_tables(ibase + 1, nta, ntb);
        step(ibase + li, li >= 1 && li <= msw);
    }
    for (; s < msw; ++s) step(ibase + s - t + 1, true);
    for (; s < msw + G - 1; ++s) {
        const int32_t li = s - t + 1;
        step(ibase + li, li >= 1 && li <= msw);
    }
    if (BAND) {
        // exits through the right edge: cells (iend + 1, j) of this pass's rows, entered
        // by a horizontal gap from (iend, j) or diagonally from (iend, j - 1)
        const uint32_t above = __shfl_up_sync(gmask, H[RA - 1], 1, G);
        const uint32_t hup0 = t == 0 ? top_last : above;
#pragma unroll
        for (int l = 0; l < NL; ++l) {
            if ((l == 1 && !w.has_b) || iend >= w.m[l]) continue;
#pragma unroll
            for (int k = 0; k < RA; ++k) {
                const int32_t j = j0 + k + 1;
                if (j > w.n[l]) continue;
                const int32_t gv = V::get(Fr[k], l) - w.Kt + P.shift * (iend + 1);
                const int32_t dv = V::get(k == 0 ? hup0 : H[k - 1], l) - w.Kt + P.shift * iend + P.smax;
                w.ub[l] = max(w.ub[l], exit_bound(P, gv, dv, iend + 1, j, w.m[l], w.n[l]));
            }
        }
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

// ---- pieces shared by the single-group and the CTA kernels ---------------------------

// The work of pair order[first] (and order[first + 1] in s16x2 lanes).
template <class V, int MODE>
__device__ __forceinline__ void init_work(const DpLaunch &L, const DpParams &P, const uint32_t *order, uint32_t first,
                                          uint32_t count, int G, int R, GroupWork &w)
{
    constexpr int NL = V::LANES;
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
    for (int c = 0; c < 8; ++c) { w.lb_v[c] = INT32_MIN; w.lb_j[c] = 0; }
    w.ub[0] = w.ub[1] = INT32_MIN;
    w.cells = 0;
    w.ms = NL == 2 ? max(w.m[0], w.m[1]) : w.m[0];
    w.nh = NL == 2 ? max(w.n[0], w.n[1]) : w.n[0];
    w.rows_full = G * R;
    w.passes = (w.nh + w.rows_full - 1) / w.rows_full;
    const uint32_t owner = (NL == 2 && w.m[1] > w.m[0]) ? w.id[1] : w.id[0];
    w.buf = L.boundary + (L.off1[owner] + owner);
    w.bin = w.bout = w.buf;
    w.seen = INT32_MIN;
    w.wait_failed = false;
    if (NL == 2) {
        if (MODE == M_LOCAL) {
            w.Kt = 2048;
            w.clampt = 2048;
            w.floor_true = 0;
        } else {
            // stored H - smax * column never exceeds 0 (no step gains more than the shift)
            w.Kt = 32767 - 512;
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
}

// Band mode: the column window of pass p, the union of the lanes' windows from the
// window table (monotone and overlapping per lane; a lane past its last pass keeps
// its last window, which ends at its column m, so the union is too).
template <int NL>
__device__ __forceinline__ int2 band_window(const DpLaunch &L, const GroupWork &w, int p)
{
    int32_t a = INT32_MAX, b = 0;
#pragma unroll
    for (int l = 0; l < NL; ++l) {
        if (l == 1 && !w.has_b) continue;
        const int32_t pl = (w.n[l] + w.rows_full - 1) / w.rows_full;
        const uint64_t slot = (L.off2[w.id[l]] - L.off2[0]) / (uint64_t)L.band_rows + w.id[l];
        const int2 x = L.band_win[slot + min(p, pl - 1)];
        a = min(a, x.x);
        b = max(b, x.y);
    }
    if (a == INT32_MAX) { a = 1; b = w.ms; }
    a = p == 0 ? 1 : max(a, 1);
    b = min(max(b, a), w.ms);
    return make_int2(a, b);
}

// One pass p of the group's pair(s): the band window and its exits (band mode),
// then the wavefront sweep.
template <class V, int R, int MODE, bool GEN, int VAR, int SYNC>
__device__ __forceinline__ void pass_body(const DpLaunch &L, const DpParams &P, GroupWork &w, int p, int t, int G,
                                          unsigned gmask, uint4 *snap)
{
    constexpr int NL = V::LANES;
    const int32_t rem = w.nh - p * w.rows_full;
    const int32_t rpt = rem >= w.rows_full ? R : ((rem + G * kChunk - 1) / (G * kChunk)) * kChunk;
    const uint32_t NEGV = NL == 2 ? w.CLAMP : (uint32_t)kNeg32;
    int2 bprev = make_int2(1, w.ms), bcur = bprev, bnext = bprev;
    const bool more = p + 1 < w.passes;
    if (MODE == M_BAND) {
        bcur = band_window<NL>(L, w, p);
        if (p > 0) bprev = band_window<NL>(L, w, p - 1);
        if (more) bnext = band_window<NL>(L, w, p + 1);
        // the exits below assume monotone, overlapping windows: refuse to certify otherwise
        if (p > 0 && (bcur.x < bprev.x || bcur.y < bprev.y || bcur.x > bprev.y)) w.ub[0] = w.ub[1] = INT32_MAX;
        w.ibase = bcur.x - 1;
        w.iend = bcur.y;
        const int32_t c0 = bcur.x - 1;
        w.diag0 = NEGV;
        if (t == 0 && p > 0 && c0 >= bprev.x && c0 <= bprev.y) {
            if (SYNC && w.seen < w.base_in + c0) {
                w.seen = wait_progress<SYNC>(w.prog_in, w.base_in + c0, L.error, L.spin_limit);
                if (w.seen == INT32_MAX) w.wait_failed = true;
            }
            w.diag0 = load_cell<SYNC>(w.bin + c0).h;
        }
    }
    switch (rpt / kChunk) {
    case 1: run_pass<V, R, 4, MODE, GEN, VAR, SYNC>(L, P, w, p, t, G, gmask, snap); break;
    case 2: run_pass<V, R, 8, MODE, GEN, VAR, SYNC>(L, P, w, p, t, G, gmask, snap); break;
    case 3: run_pass<V, R, 12, MODE, GEN, VAR, SYNC>(L, P, w, p, t, G, gmask, snap); break;
    default: run_pass<V, R, R, MODE, GEN, VAR, SYNC>(L, P, w, p, t, G, gmask, snap); break;
    }
    __syncwarp(gmask);
    if (MODE == M_BAND) {
        const int32_t jlo = p * w.rows_full + 1, jhi = p * w.rows_full + G * rpt;
        const int32_t goe = P.gap_open + P.gap_ext;
#pragma unroll
        for (int l = 0; l < NL; ++l) {
            if (l == 1 && !w.has_b) continue;
            const int32_t ml = w.m[l], nl = w.n[l];
            if (jlo > nl) continue;
            if (t == 0) w.cells += (unsigned long long)(bcur.y - bcur.x + 1) * (min(jhi, nl) - jlo + 1);
            if (p == 0)       // along the top border past the window, then down into row 1
                for (int32_t i = bcur.y + 1 + t; i <= ml; i += G)
                    w.ub[l] = max(w.ub[l], exit_bound(P, border(P, 0, i) + goe, border(P, 0, i - 1) + P.smax,
                                                      i, 1, ml, nl));
            if (bcur.x > 1)   // down the left border, then into column 1 of this pass
                for (int32_t j = jlo + t; j <= min(jhi, nl); j += G)
                    w.ub[l] = max(w.ub[l], exit_bound(P, border(P, 0, j) + goe, border(P, 0, j - 1) + P.smax,
                                                      1, j, ml, nl));
            if (more && jhi < nl) {   // through the bottom edge left of the next window
                const int32_t last = min(min(bcur.y, bnext.x - 1), ml);
                for (int32_t i = bcur.x + t; i <= last; i += G) {
                    const Cell c = w.bout[i];
                    const int32_t cv = P.shift * i - w.Kt;
                    w.ub[l] = max(w.ub[l], exit_bound(P, V::get(c.e, l) + cv, kNeg32, i, jhi + 1, ml, nl));
                    if (i + 1 < bnext.x)
                        w.ub[l] = max(w.ub[l], exit_bound(P, kNeg32, V::get(c.h, l) + cv + P.smax, i + 1,
                                                          jhi + 1, ml, nl));
                }
            }
        }
        if (more)             // columns the next pass reads beyond this window: outside
            for (int32_t i = bcur.y + 1 + t; i <= bnext.y; i += G) w.bout[i] = Cell{NEGV, NEGV};
        __syncwarp(gmask);
    }
}

// Reduction over the threads of a group (results in every thread).
template <class V, int MODE>
__device__ __forceinline__ void reduce_group(GroupWork &w, unsigned gmask, int G)
{
    constexpr int NL = V::LANES;
    if (MODE == M_LABEL_REV)
        for (int c = 0; c < 8; ++c)
            for (int off = G >> 1; off >= 1; off >>= 1) {
                const int32_t ov = __shfl_xor_sync(gmask, w.lb_v[c], off, G);
                const int32_t oj = __shfl_xor_sync(gmask, w.lb_j[c], off, G);
                if (ov > w.lb_v[c] || (ov == w.lb_v[c] && oj < w.lb_j[c])) { w.lb_v[c] = ov; w.lb_j[c] = oj; }
            }
#pragma unroll
    for (int l = 0; l < NL; ++l) {
        if (MODE == M_BAND)
            for (int off = G >> 1; off >= 1; off >>= 1) w.ub[l] = max(w.ub[l], __shfl_xor_sync(gmask, w.ub[l], off, G));
        for (int off = G >> 1; off >= 1; off >>= 1) {
            const int32_t os = __shfl_xor_sync(gmask, w.cs[l], off, G);
            const int32_t oi = __shfl_xor_sync(gmask, w.ci[l], off, G);
            const int32_t oj = __shfl_xor_sync(gmask, w.cj[l], off, G);
            if (better(os, oi, oj, w.cs[l], w.ci[l], w.cj[l])) { w.cs[l] = os; w.ci[l] = oi; w.cj[l] = oj; }
        }
    }
}

// Results of the unit (one thread): labels, free-end borders, the s16 exactness
// check, the band outcome.
template <class V, int MODE>
__device__ __forceinline__ void emit(const DpLaunch &L, const DpParams &P, GroupWork &w, uint32_t first)
{
    constexpr int NL = V::LANES;
    if (MODE == M_LABEL_REV)
        for (int c = 0; c < 8; ++c) L.labels[(uint64_t)w.id[0] * 8 + c] = w.lb_j[c] - checkpoint_col(c, w.m[0]);
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
        if (w.wait_failed) {
            // a boundary row was read before it was published: the score is not valid
            r.score = INT32_MIN;
            r.end1 = r.end2 = 0;
            r.flags = PA_RESULT_ERROR;
            L.out[w.id[l]] = r;
            if (MODE == M_BAND) {
                L.band_code[first + l] = 0;
                if (L.band_ub) L.band_ub[w.id[l]] = INT32_MAX;
            }
            continue;
        }
        if (MODE == M_BAND) {
            uint8_t code;
            if (NL == 2 && (int64_t)w.cs[l] - (int64_t)P.shift * w.ci[l] <= (int64_t)w.floor_true) {
                code = 3;                           // a clamp may have reached it: redo in s32
            } else if (w.cs[l] != INT32_MIN && w.ub[l] <= w.cs[l]) {   // no path leaving the band scores more
                r.flags |= PA_RESULT_BANDED;
                r.band_rounds = (uint16_t)L.band_round;
                L.out[w.id[l]] = r;
                code = 0;
            } else {
                code = 1;
            }
            L.band_code[first + l] = code;
            if (L.band_ub) L.band_ub[w.id[l]] = w.ub[l];
            continue;
        }
        if (NL == 2 && MODE != M_LOCAL && (int64_t)w.cs[l] - (int64_t)P.shift * w.ci[l] <= (int64_t)w.floor_true) {
            // every step adds at most 0 to H - shift * column, so a clamped cell stays at or
            // below the floor: a result above it never met a clamp.  Otherwise recompute in s32
            const uint32_t slot = atomicAdd(L.rerun_count, 1u);
            L.rerun_list[slot] = w.id[l];
            continue;
        }
        L.out[w.id[l]] = r;
    }
    if (MODE == M_BAND && L.dp_cells && w.cells) atomicAdd(L.dp_cells, w.cells);
}

// GEN = byte-compare scoring (any bytes, any int32 scores), always with L32 lanes.
// One group of G lanes per pair (two pairs in s16x2 lanes); the group runs all
// passes of its pair(s) one after the other.
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
        init_work<V, MODE>(L, P, order, first, count, G, R, w);
        for (int p = 0; p < w.passes; ++p) pass_body<V, R, MODE, GEN, VAR, 0>(L, P, w, p, t, G, gmask, snap_store);
        reduce_group<V, MODE>(w, gmask, G);
        if (t == 0) emit<V, MODE>(L, P, w, first);
        __syncwarp(gmask);
    }
}

// CTA mode for long pairs: the NG = 8 warps of a block are groups of 32 lanes that
// take the passes of one unit (one pair, two in s16x2 lanes) round robin: pass p
// runs on warp p % NG, reads the boundary row of pass p - 1 from ring row
// (p - 1) % NG and writes its own to ring row p % NG, column by column, behind
// published progress.  Ring row k is reused by pass p + NG only after pass p + 1
// has read it: pass p + NG reaches column c only after every pass between did.
template <class V, int R, int MODE, bool GEN, int VAR>
__global__ void __launch_bounds__(kBlock, 2) dp_kernel_cta(DpLaunch L, DpParams P)
{
    static_assert(R % kChunk == 0 && R <= 32, "R must be a multiple of the chunk");
    constexpr int NL = V::LANES;
    constexpr int NG = kBlock / 32;
    constexpr int G = 32;
    __shared__ uint4 snap_store[MODE == M_LOCAL ? NL * (R / 4) * kBlock : 1];
    __shared__ int prog[NG];
    __shared__ uint32_t s_unit;
    __shared__ int32_t s_cand[NG][2][4];
    __shared__ int32_t s_lb[MODE == M_LABEL_REV ? NG : 1][8][2];
    __shared__ unsigned long long s_cells[NG];
    __shared__ bool s_fail[NG];
    const int t = threadIdx.x & 31, g = threadIdx.x >> 5;
    const unsigned gmask = 0xffffffffu;
    const uint32_t count_main = *L.count_ptr;
    const uint32_t *order_main = L.order + *L.begin_ptr;
    const uint32_t count_lead = L.lead_count_ptr ? *L.lead_count_ptr : 0u;
    const uint32_t *order_lead = L.lead_count_ptr ? L.lead_order + *L.lead_begin_ptr : nullptr;
    const uint32_t units_lead = (count_lead + NL - 1) / NL;
    const uint32_t n_units = units_lead + (count_main + NL - 1) / NL;
    Cell *ring = L.ring + (uint64_t)blockIdx.x * NG * L.ring_stride;

    for (;;) {
        if (threadIdx.x < NG) prog[threadIdx.x] = -1;
        if (threadIdx.x == 0) s_unit = atomicAdd(L.unit_counter, 1u);
        __syncthreads();
        uint32_t u = s_unit;
        __syncthreads();
        if (u >= n_units) break;
        // the lead list first, then the main list, each largest shapes first
        const bool lead = u < units_lead;
        const uint32_t count = lead ? count_lead : count_main;
        const uint32_t *order = lead ? order_lead : order_main;
        u = lead ? units_lead - 1 - u : n_units - 1 - u;
        const uint32_t first = u * NL;
        GroupWork w;
        init_work<V, MODE>(L, P, order, first, count, G, R, w);
        const int32_t span = w.ms + 2;               // progress values of consecutive passes never overlap
        for (int p = g; p < w.passes; p += NG) {
            w.bin = ring + (uint64_t)((p + NG - 1) % NG) * L.ring_stride;
            w.bout = ring + (uint64_t)(p % NG) * L.ring_stride;
            w.prog_in = &prog[(p + NG - 1) % NG];
            w.prog_out = &prog[p % NG];
            w.base_in = (p - 1) * span;
            w.base_out = p * span;
            w.seen = INT32_MIN;
            pass_body<V, R, MODE, GEN, VAR, 1>(L, P, w, p, t, G, gmask, snap_store);
            if (t == G - 1 && p + 1 < w.passes) publish_progress<1>(w.prog_out, w.base_out + w.ms + 1);
        }
        reduce_group<V, MODE>(w, gmask, G);
        if (t == 0) {
            for (int l = 0; l < 2; ++l) {
                s_cand[g][l][0] = w.cs[l];
                s_cand[g][l][1] = w.ci[l];
                s_cand[g][l][2] = w.cj[l];
                s_cand[g][l][3] = w.ub[l];
            }
            if (MODE == M_LABEL_REV)
                for (int c = 0; c < 8; ++c) { s_lb[g][c][0] = w.lb_v[c]; s_lb[g][c][1] = w.lb_j[c]; }
            s_cells[g] = w.cells;
            s_fail[g] = w.wait_failed;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int k = 1; k < NG; ++k) {
                w.wait_failed |= s_fail[k];
                for (int l = 0; l < 2; ++l) {
                    const int32_t *c = s_cand[k][l];
                    if (better(c[0], c[1], c[2], w.cs[l], w.ci[l], w.cj[l])) { w.cs[l] = c[0]; w.ci[l] = c[1]; w.cj[l] = c[2]; }
                    w.ub[l] = max(w.ub[l], c[3]);
                }
                if (MODE == M_LABEL_REV)
                    for (int c = 0; c < 8; ++c) {
                        const int32_t ov = s_lb[k][c][0], oj = s_lb[k][c][1];
                        if (ov > w.lb_v[c] || (ov == w.lb_v[c] && oj < w.lb_j[c])) { w.lb_v[c] = ov; w.lb_j[c] = oj; }
                    }
                w.cells += s_cells[k];
            }
            emit<V, MODE>(L, P, w, first);
        }
        __syncthreads();
    }
}

// Teams mode (band mode on long pairs): the warps of a block form teams of T warps
// (1, 2, 4 or 8); each team takes one unit (one pair, two in s16x2 lanes) at a time and its warps
// take the unit's passes round robin: pass p runs on team warp p % T, reads the boundary
// row of pass p - 1 from that warp's ring row and writes its own, column by column, behind
// published progress.  A team's ring row k is reused by pass p + T only after pass p + 1
// has read it: pass p + T reaches column c only after every pass between did.  Teams
// smaller than the block suit banded pairs, whose narrow windows keep only a few passes in
// flight at once.
template <class V, int R, int MODE, bool GEN, int VAR, int T>
__global__ void __launch_bounds__(kBlock, 2) dp_kernel_team(DpLaunch L, DpParams P)
{
    static_assert(R % kChunk == 0 && R <= 32, "R must be a multiple of the chunk");
    constexpr int NL = V::LANES;
    constexpr int NW = kBlock / 32;
    constexpr int G = 32;
    __shared__ uint4 snap_store[MODE == M_LOCAL ? NL * (R / 4) * kBlock : 1];
    __shared__ int prog[NW];
    __shared__ uint32_t s_unit[NW];
    __shared__ int32_t s_cand[NW][2][4];
    __shared__ int32_t s_lb[MODE == M_LABEL_REV ? NW : 1][8][2];
    __shared__ unsigned long long s_cells[NW];
    __shared__ bool s_fail[NW];
    // the unit lists, in shared memory so that they hold no registers during the passes
    __shared__ const uint32_t *s_order[2];
    __shared__ uint32_t s_count[2], s_units_lead, s_units;
    if (threadIdx.x == 0) {
        const uint32_t cm = *L.count_ptr, cl = L.lead_count_ptr ? *L.lead_count_ptr : 0u;
        s_order[0] = L.order + *L.begin_ptr;
        s_order[1] = L.lead_count_ptr ? L.lead_order + *L.lead_begin_ptr : nullptr;
        s_count[0] = cm;
        s_count[1] = cl;
        s_units_lead = (cl + NL - 1) / NL;
        s_units = s_units_lead + (cm + NL - 1) / NL;
    }
    __syncthreads();
    static_assert(T == 1 || T == 2 || T == 4 || T == kBlock / 32, "team of 1, 2, 4 or all warps");
    const int t = threadIdx.x & 31, g = threadIdx.x >> 5;
    const unsigned gmask = 0xffffffffu;
    auto team_sync = [&]() {
        if (T == 1) __syncwarp();
        else asm volatile("bar.sync %0, %1;" ::"r"(1 + g / T), "r"(T * 32) : "memory");
    };

    for (;;) {
        if (t == 0) prog[g] = -1;
        if (g % T == 0 && t == 0) s_unit[g / T] = atomicAdd(L.unit_counter, 1u);
        team_sync();
        uint32_t u = s_unit[g / T];
        team_sync();
        const uint32_t units_lead = *(volatile uint32_t *)&s_units_lead, n_units = *(volatile uint32_t *)&s_units;
        if (u >= n_units) break;
        // the lead list first, then the main list, each largest shapes first
        const int which = u < units_lead ? 1 : 0;
        u = which ? units_lead - 1 - u : n_units - 1 - u;
        const uint32_t first = u * NL;
        GroupWork w;
        init_work<V, MODE>(L, P, *(const uint32_t *volatile *)&s_order[which], first,
                           *(volatile uint32_t *)&s_count[which], G, R, w);
        const int32_t span = w.ms + 2;           // progress values of consecutive passes never overlap
        for (int p = g % T; p < w.passes; p += T) {
            const int lead = g - g % T, pw = (p + T - 1) % T;   // team's first warp; warp of pass p - 1
            Cell *ring = L.ring + ((uint64_t)blockIdx.x * NW + lead) * L.ring_stride;
            w.bin = ring + (uint64_t)pw * L.ring_stride;
            w.bout = ring + (uint64_t)(p % T) * L.ring_stride;
            w.prog_in = &prog[lead + pw];
            w.prog_out = &prog[g];
            w.base_in = (p - 1) * span;
            w.base_out = p * span;
            w.seen = INT32_MIN;
            pass_body<V, R, MODE, GEN, VAR, 1>(L, P, w, p, t, G, gmask, snap_store);
            if (t == G - 1 && p + 1 < w.passes) publish_progress<1>(w.prog_out, w.base_out + w.ms + 1);
        }
        reduce_group<V, MODE>(w, gmask, G);
        if (t == 0) {
            for (int l = 0; l < 2; ++l) {
                s_cand[g][l][0] = w.cs[l];
                s_cand[g][l][1] = w.ci[l];
                s_cand[g][l][2] = w.cj[l];
                s_cand[g][l][3] = w.ub[l];
            }
            if (MODE == M_LABEL_REV)
                for (int c = 0; c < 8; ++c) { s_lb[g][c][0] = w.lb_v[c]; s_lb[g][c][1] = w.lb_j[c]; }
            s_cells[g] = w.cells;
            s_fail[g] = w.wait_failed;
        }
        team_sync();
        if (g % T == 0 && t == 0) {
            for (int k = g + 1; k < g + T; ++k) {
                w.wait_failed |= s_fail[k];
                for (int l = 0; l < 2; ++l) {
                    const int32_t *c = s_cand[k][l];
                    if (better(c[0], c[1], c[2], w.cs[l], w.ci[l], w.cj[l])) { w.cs[l] = c[0]; w.ci[l] = c[1]; w.cj[l] = c[2]; }
                    w.ub[l] = max(w.ub[l], c[3]);
                }
                if (MODE == M_LABEL_REV)
                    for (int c = 0; c < 8; ++c) {
                        const int32_t ov = s_lb[k][c][0], oj = s_lb[k][c][1];
                        if (ov > w.lb_v[c] || (ov == w.lb_v[c] && oj < w.lb_j[c])) { w.lb_v[c] = ov; w.lb_j[c] = oj; }
                    }
                w.cells += s_cells[k];
            }
            emit<V, MODE>(L, P, w, first);
        }
        team_sync();
    }
}

// Cluster mode for the largest pairs: a cluster of CL blocks (co-scheduled by the
// hardware) works on one unit with all its 8*CL warps, pass p on group p % (8*CL)
// (block (p % (8*CL)) / 8, warp p % 8).  Progress flags stay in the shared memory
// of the producing block and are read through distributed shared memory with
// cluster-scope acquire; ring rows are the 8*CL rows of the cluster's blocks.
template <class V, int R, int MODE, bool GEN, int VAR, int CL>
__global__ void __launch_bounds__(kBlock, 2) dp_kernel_cluster(DpLaunch L, DpParams P)
{
    static_assert(R % kChunk == 0 && R <= 32, "R must be a multiple of the chunk");
    constexpr int NL = V::LANES;
    constexpr int NW = kBlock / 32;              // warps (groups) per block
    constexpr int NG = NW * CL;                  // groups per cluster
    constexpr int G = 32;
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    __shared__ uint4 snap_store[MODE == M_LOCAL ? NL * (R / 4) * kBlock : 1];
    __shared__ int prog[NW];
    __shared__ uint32_t s_unit;
    __shared__ int32_t s_cand[NW][2][4];
    __shared__ int32_t s_lb[NW][8][2];
    __shared__ unsigned long long s_cells[NW];
    __shared__ int32_t s_part[2][4];             // this block's merged result, read by rank 0
    __shared__ int32_t s_plb[8][2];
    __shared__ unsigned long long s_pcells;
    __shared__ bool s_fail[NW], s_pfail;
    const int t = threadIdx.x & 31, g = threadIdx.x >> 5;
    const unsigned gmask = 0xffffffffu;
    const uint32_t count = *L.count_ptr;
    const uint32_t *order = L.order + *L.begin_ptr;
    const uint32_t n_units = (count + NL - 1) / NL;
    Cell *ring = L.ring + (uint64_t)(blockIdx.x - rank) * NW * L.ring_stride;   // the cluster's rows
    const int gg = rank * NW + g;                // this warp's group in the cluster

    for (;;) {
        if (threadIdx.x < NW) prog[threadIdx.x] = -1;
        if (rank == 0 && threadIdx.x == 0) s_unit = atomicAdd(L.unit_counter, 1u);
        cluster.sync();
        uint32_t u = *cluster.map_shared_rank(&s_unit, 0);
        cluster.sync();
        if (u >= n_units) break;
        u = n_units - 1 - u;                     // largest shapes first
        const uint32_t first = u * NL;
        GroupWork w;
        init_work<V, MODE>(L, P, order, first, count, G, R, w);
        const int32_t span = w.ms + 2;
        for (int p = gg; p < w.passes; p += NG) {
            const int pg = (p + NG - 1) % NG;    // the group of pass p - 1
            w.bin = ring + (uint64_t)pg * L.ring_stride;
            w.bout = ring + (uint64_t)(p % NG) * L.ring_stride;
            w.prog_in = cluster.map_shared_rank(prog, pg / NW) + (pg % NW);
            w.prog_out = &prog[g];
            w.base_in = (p - 1) * span;
            w.base_out = p * span;
            w.seen = INT32_MIN;
            pass_body<V, R, MODE, GEN, VAR, 2>(L, P, w, p, t, G, gmask, snap_store);
            if (t == G - 1 && p + 1 < w.passes) publish_progress<2>(w.prog_out, w.base_out + w.ms + 1);
        }
        reduce_group<V, MODE>(w, gmask, G);
        if (t == 0) {
            for (int l = 0; l < 2; ++l) {
                s_cand[g][l][0] = w.cs[l];
                s_cand[g][l][1] = w.ci[l];
                s_cand[g][l][2] = w.cj[l];
                s_cand[g][l][3] = w.ub[l];
            }
            for (int c = 0; c < 8; ++c) { s_lb[g][c][0] = w.lb_v[c]; s_lb[g][c][1] = w.lb_j[c]; }
            s_cells[g] = w.cells;
            s_fail[g] = w.wait_failed;
        }
        __syncthreads();
        // merge the block's groups, then rank 0 merges the blocks
        auto merge = [&](const int32_t (*cand)[4], const int32_t (*lb)[2], unsigned long long cells, bool failed) {
            w.wait_failed |= failed;
            for (int l = 0; l < 2; ++l) {
                const int32_t *c = cand[l];
                if (better(c[0], c[1], c[2], w.cs[l], w.ci[l], w.cj[l])) { w.cs[l] = c[0]; w.ci[l] = c[1]; w.cj[l] = c[2]; }
                w.ub[l] = max(w.ub[l], c[3]);
            }
            for (int c = 0; c < 8; ++c) {
                const int32_t ov = lb[c][0], oj = lb[c][1];
                if (ov > w.lb_v[c] || (ov == w.lb_v[c] && oj < w.lb_j[c])) { w.lb_v[c] = ov; w.lb_j[c] = oj; }
            }
            w.cells += cells;
        };
        if (threadIdx.x == 0) {
            for (int k = 1; k < NW; ++k) merge(s_cand[k], s_lb[k], s_cells[k], s_fail[k]);
            for (int l = 0; l < 2; ++l) {
                s_part[l][0] = w.cs[l];
                s_part[l][1] = w.ci[l];
                s_part[l][2] = w.cj[l];
                s_part[l][3] = w.ub[l];
            }
            for (int c = 0; c < 8; ++c) { s_plb[c][0] = w.lb_v[c]; s_plb[c][1] = w.lb_j[c]; }
            s_pcells = w.cells;
            s_pfail = w.wait_failed;
        }
        cluster.sync();
        if (rank == 0 && threadIdx.x == 0) {
            for (int r = 1; r < CL; ++r)
                merge(cluster.map_shared_rank(s_part, r), cluster.map_shared_rank(s_plb, r),
                      *cluster.map_shared_rank(&s_pcells, r), *cluster.map_shared_rank(&s_pfail, r));
            emit<V, MODE>(L, P, w, first);
        }
        cluster.sync();
    }
}

}  // namespace pa

