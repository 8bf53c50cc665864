// pa_short.cuh -- the short-pair DP kernel in s16x2 lanes (unitary DNA scores).
//
// The same recurrence, borders, trackers and wavefront as dp_kernel<L16> (pa_dp.cuh):
// a group of G lanes holds two pairs in the halves of s16x2 registers, thread t holds
// R rows of sequence2, and the group sweeps sequence1 as an anti-diagonal wavefront.
// The reference's hot loop it replaces is compute_block / compute_cell
// (dp_algorithm_template/dp_algorithm_template_base.hpp:82-129,
// affine/affine_dp_algorithm.hpp:133-156).  What differs is how little each column step
// costs besides the recurrence:
//  * every streamed column has one 16-byte slot {table of lane A, table of lane B, top H,
//    top vertical gap}.  The group writes the slots of its unit once (tables from the
//    sequence1 bytes, the top border of the first pass); thread 0 then reads one slot per
//    column with a single vector load, one column ahead, and the last thread writes the
//    pass's bottom row back into the .h/.e halves for the next pass;
//  * the score tables travel down the group with the H and gap values by shuffle, so no
//    other thread loads anything per column;
//  * no border arithmetic in the column loop: thread 0 selects the slot values;
//  * the rows are written so that the diagonal term of row k + 1 is formed before row k's
//    new H replaces the old one (no register copies between column steps).
#pragma once
#include "pa_dp.cuh"

namespace pa {

// State of the unit a group works on (two pairs in s16x2 lanes; lane B may be absent).
struct ShortUnit {
    uint32_t id[2];
    uint64_t qoff[2], toff[2];
    int32_t m[2], n[2];
    int32_t ms, nh, passes;
    bool has_b;
    Slot *slot;                    // slots 1..ms of the unit (slot 0 unused)
    int32_t cs[2], ci[2], cj[2];   // candidate (score, end1, end2) per lane
};

template <int MODE>
struct ShortConst {
    static constexpr int32_t Kt = MODE == M_LOCAL ? 2048 : 32767 - 512;   // stored = true + Kt (+ shift)
    static constexpr int32_t clampt = 2048;
    static constexpr int32_t floor_true = MODE == M_LOCAL ? 0 : 2048 - Kt;
};

// One pass p of the unit: rows p*G*R + t*RA + 1 .. + RA (1-based) on thread t.
template <int MODE, int G, int R, int RA>
__device__ __forceinline__ void short_pass(const DpLaunch &L, const DpParams &P, ShortUnit &u, int p, int t,
                                           unsigned gmask, uint4 *snap)
{
    using V = L16;
    using KC = ShortConst<MODE>;
    constexpr bool SHIFTED = MODE != M_LOCAL;
    const int32_t rows_full = G * R;
    const int32_t j0 = p * rows_full + t * RA;
    const uint32_t GOEA = V::cabs(P.gap_open + P.gap_ext);
    const uint32_t EXTA = V::cabs(P.gap_ext);
    const uint32_t GOEH = V::cabs(P.gap_open + P.gap_ext - P.shift);
    const uint32_t EXTH = V::cabs(P.gap_ext - P.shift);
    const uint32_t CLAMP = V::splat(KC::clampt);
    const uint32_t K = V::splat(KC::Kt);
    auto stored = [&](int32_t true_value) { return V::splat(max(true_value + KC::Kt, KC::clampt)); };

    uint32_t H[RA], Fr[RA], Sel[RA];
#pragma unroll
    for (int k = 0; k < RA; ++k) {
        const int32_t j = j0 + k;                 // 0-based row of sequence2
        const int ca = j < u.n[0] ? (int)dna_code(L.seq2[u.toff[0] + j]) : -1;
        const int cb = j < u.n[1] ? (int)dna_code(L.seq2[u.toff[1] + j]) : -1;
        Sel[k] = V::selector(ca, cb);
        H[k] = stored(border(P, P.first_row_free, (int64_t)j + 1));
        Fr[k] = V::subc(H[k], GOEH);
    }
    uint32_t prevH = stored(border(P, P.first_row_free, j0));
    // where row n[l] lives (global modes read the result there)
    int32_t own_k[2];
    bool own[2];
#pragma unroll
    for (int l = 0; l < 2; ++l) {
        const int32_t r = (u.n[l] - 1) - p * rows_full - t * RA;
        own[l] = r >= 0 && r < RA && (u.n[l] - 1) / rows_full == p;
        own_k[l] = r;
    }
    const bool last_pass = p + 1 == u.passes;
    const bool writer = t == G - 1 && !last_pass;
    const bool t0 = t == 0;
    const int32_t ms = u.ms;

    uint32_t outH = 0, outE = 0, ta = 0, tb = 0, best = K;
    int32_t bi[2] = {0, 0};
    Slot nx = Slot{0u, 0u, 0u, 0u};
    if (t0) nx = u.slot[1];
    Slot *cur = u.slot + 1;                       // the slot of the thread's current column

    auto step = [&](int32_t i, bool active) {
        const uint32_t xH = __shfl_up_sync(gmask, outH, 1, G);
        const uint32_t xE = __shfl_up_sync(gmask, outE, 1, G);
        const uint32_t xA = __shfl_up_sync(gmask, ta, 1, G);
        const uint32_t xB = __shfl_up_sync(gmask, tb, 1, G);
        if (!active) return;
        const uint32_t upH = t0 ? nx.h : xH;
        uint32_t Ed = t0 ? nx.e : xE;
        ta = t0 ? nx.ta : xA;
        tb = t0 ? nx.tb : xB;
        if (t0 && i < ms) nx = cur[1];            // thread 0: the next column's slot
        uint32_t tt = V::addmax(prevH, prmt(ta, tb, Sel[0]), Fr[0]);
#pragma unroll
        for (int k = 0; k < RA; ++k) {
            // the next row's diagonal term uses this row's H before it is replaced
            const uint32_t tn = k + 1 < RA ? V::addmax(H[k], prmt(ta, tb, Sel[k + 1]), Fr[k + 1]) : 0u;
            const uint32_t h = V::hmax(tt, Ed, CLAMP);
            H[k] = h;
            const uint32_t hoe = V::subc(h, GOEA);
            Fr[k] = V::max2(V::subc(Fr[k], EXTH), SHIFTED ? V::subc(h, GOEH) : hoe);
            Ed = V::max2(V::subc(Ed, EXTA), hoe);
            tt = tn;
        }
        prevH = upH;
        outH = H[RA - 1];
        outE = Ed;
        if (writer) *reinterpret_cast<uint2 *>(&cur->h) = make_uint2(outH, outE);
        ++cur;
        if (MODE == M_LOCAL) {
            const uint32_t cm = tree_max<V, RA>(H);
            const uint32_t nb = V::max2(best, cm);
            const uint32_t x = nb ^ best;
            best = nb;
            if (x != 0u) {
#pragma unroll
                for (int l = 0; l < 2; ++l) {
                    if (V::improved(x, l)) {
                        bi[l] = i;
#pragma unroll
                        for (int v = 0; v < RA / 4; ++v)
                            snap[(l * (R / 4) + v) * kBlock] = make_uint4(H[4 * v], H[4 * v + 1], H[4 * v + 2], H[4 * v + 3]);
                    }
                }
            }
        } else {
#pragma unroll
            for (int l = 0; l < 2; ++l) {
                if (l == 1 && !u.has_b) continue;
                if (MODE == M_GLOBAL_FREE && P.last_column_free && own[l] && i <= u.m[l]) {
                    uint32_t v = H[0];
#pragma unroll
                    for (int k = 1; k < RA; ++k)
                        if (own_k[l] == k) v = H[k];
                    const int32_t xs = V::get(v, l) - KC::Kt + P.shift * i;
                    if (better(xs, i, u.n[l], u.cs[l], u.ci[l], u.cj[l])) { u.cs[l] = xs; u.ci[l] = i; u.cj[l] = u.n[l]; }
                }
                if (i == u.m[l]) {
                    if (MODE == M_GLOBAL_FREE && P.last_row_free) {
#pragma unroll
                        for (int k = 0; k < RA; ++k) {
                            const int32_t j = j0 + k + 1;
                            if (j <= u.n[l]) {
                                const int32_t xs = V::get(H[k], l) - KC::Kt + P.shift * i;
                                if (better(xs, i, j, u.cs[l], u.ci[l], u.cj[l])) { u.cs[l] = xs; u.ci[l] = i; u.cj[l] = j; }
                            }
                        }
                    } else if (own[l]) {
                        uint32_t v = H[0];
#pragma unroll
                        for (int k = 1; k < RA; ++k)
                            if (own_k[l] == k) v = H[k];
                        const int32_t xs = V::get(v, l) - KC::Kt + P.shift * i;
                        if (better(xs, i, u.n[l], u.cs[l], u.ci[l], u.cj[l])) { u.cs[l] = xs; u.ci[l] = i; u.cj[l] = u.n[l]; }
                    }
                }
            }
        }
    };
    // fill: thread t starts at step t; steady: every thread active; drain
    const int32_t fill_end = min(G, ms + G - 1);
    int32_t s = 0;
    for (; s < fill_end; ++s) {
        const int32_t i = s - t + 1;
        step(i, i >= 1 && i <= ms);          // the slot pointers advance on active steps only
    }
    for (; s < ms; ++s) step(s - t + 1, true);
    for (; s < ms + G - 1; ++s) {
        const int32_t i = s - t + 1;
        step(i, i >= 1 && i <= ms);
    }
    if (MODE == M_LOCAL) {
#pragma unroll
        for (int l = 0; l < 2; ++l) {
            const int32_t b = V::get(best, l);
            if (b > KC::Kt) {
                int32_t kk = 0;
                for (int v = RA / 4 - 1; v >= 0; --v) {
                    const uint4 q = snap[(l * (R / 4) + v) * kBlock];
                    if (V::get(q.w, l) == b) kk = 4 * v + 3;
                    if (V::get(q.z, l) == b) kk = 4 * v + 2;
                    if (V::get(q.y, l) == b) kk = 4 * v + 1;
                    if (V::get(q.x, l) == b) kk = 4 * v;
                }
                const int32_t xs = b - KC::Kt, j = j0 + kk + 1;
                if (better(xs, bi[l], j, u.cs[l], u.ci[l], u.cj[l])) { u.cs[l] = xs; u.ci[l] = bi[l]; u.cj[l] = j; }
            }
        }
    }
}

// The short-pair kernel: a persistent grid whose warps take units of 32/G groups x two
// pairs from the class queue, largest shapes first.  MINB: resident blocks per SM the
// register allocation is held to (2: 128 registers, 3: 80).
template <int MODE, int G, int MINB>
__global__ void __launch_bounds__(kBlock, MINB) dp_short(DpLaunch L, DpParams P)
{
    constexpr int R = 16;
    using V = L16;
    using KC = ShortConst<MODE>;
    __shared__ uint4 snap_store[MODE == M_LOCAL ? 2 * (R / 4) * kBlock : 1];
    uint4 *snap = snap_store + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const int t = lane & (G - 1);
    const int g = lane / G;
    const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (g * G));
    const uint32_t count = *L.count_ptr;
    const uint32_t *order = L.order + *L.begin_ptr;
    constexpr uint32_t ppw = (uint32_t)(32 / G) * 2;   // pairs per warp unit
    const uint32_t n_units = (count + ppw - 1) / ppw;
    const uint32_t match4 = (uint8_t)(P.match - P.shift) * 0x01010101u;
    const uint32_t mis4 = (uint8_t)(P.mismatch - P.shift) * 0x01010101u;
    const uint32_t GOEA = V::cabs(P.gap_open + P.gap_ext);

    for (;;) {
        uint32_t uu = 0;
        if (lane == 0) uu = atomicAdd(L.unit_counter, 1u);
        uu = __shfl_sync(0xffffffffu, uu, 0);
        if (uu >= n_units) break;
        uu = n_units - 1 - uu;                       // largest shapes first
        const uint32_t first = uu * ppw + (uint32_t)g * 2;
        if (first >= count) continue;                // idle group in the last unit
        ShortUnit u;
        u.id[0] = order[first];
        u.has_b = first + 1 < count;
        u.id[1] = u.has_b ? order[first + 1] : u.id[0];
#pragma unroll
        for (int l = 0; l < 2; ++l) {
            u.qoff[l] = L.off1[u.id[l]];
            u.m[l] = (int32_t)(L.off1[u.id[l] + 1] - u.qoff[l]);
            u.toff[l] = L.off2[u.id[l]];
            u.n[l] = (int32_t)(L.off2[u.id[l] + 1] - u.toff[l]);
            u.cs[l] = MODE == M_LOCAL ? 0 : INT32_MIN;
            u.ci[l] = 0;
            u.cj[l] = 0;
        }
        u.ms = max(u.m[0], u.m[1]);
        u.nh = max(u.n[0], u.n[1]);
        u.passes = (u.nh + G * R - 1) / (G * R);
        const uint32_t owner = u.m[1] > u.m[0] ? u.id[1] : u.id[0];
        u.slot = L.slots + (L.off1[owner] + owner);   // slots 0..m(owner) = 0..ms
        // the unit's slots: both lanes' score tables (a padding table past a lane's end) and
        // the top border of the first pass, H(i, 0) - shift * i
        for (int32_t i = 1 + t; i <= u.ms; i += G) {
            const uint32_t a = i <= u.m[0] ? score_table(L.seq1[u.qoff[0] + i - 1], match4, mis4) : 0x80808080u;
            const uint32_t b = i <= u.m[1] ? score_table(L.seq1[u.qoff[1] + i - 1], match4, mis4) : 0x80808080u;
            const int64_t top = (int64_t)border(P, P.first_column_free, i) - (int64_t)P.shift * i + KC::Kt;
            const uint32_t h = V::splat((int32_t)max(top, (int64_t)KC::clampt));
            *reinterpret_cast<uint4 *>(u.slot + i) = make_uint4(a, b, h, V::subc(h, GOEA));
        }
        __syncwarp(gmask);
        for (int p = 0; p < u.passes; ++p) {
            const int32_t rem = u.nh - p * G * R;
            const int32_t rpt = rem >= G * R ? R : ((rem + G * kChunk - 1) / (G * kChunk)) * kChunk;
            switch (rpt / kChunk) {
            case 1: short_pass<MODE, G, R, 4>(L, P, u, p, t, gmask, snap); break;
            case 2: short_pass<MODE, G, R, 8>(L, P, u, p, t, gmask, snap); break;
            case 3: short_pass<MODE, G, R, 12>(L, P, u, p, t, gmask, snap); break;
            default: short_pass<MODE, G, R, R>(L, P, u, p, t, gmask, snap); break;
            }
            __syncwarp(gmask);
        }
        // reduce over the group, then thread 0 writes the results
#pragma unroll
        for (int l = 0; l < 2; ++l)
            for (int off = G >> 1; off >= 1; off >>= 1) {
                const int32_t os = __shfl_xor_sync(gmask, u.cs[l], off, G);
                const int32_t oi = __shfl_xor_sync(gmask, u.ci[l], off, G);
                const int32_t oj = __shfl_xor_sync(gmask, u.cj[l], off, G);
                if (better(os, oi, oj, u.cs[l], u.ci[l], u.cj[l])) { u.cs[l] = os; u.ci[l] = oi; u.cj[l] = oj; }
            }
        if (t == 0) {
#pragma unroll
            for (int l = 0; l < 2; ++l) {
                if (l == 1 && !u.has_b) continue;
                if (MODE == M_GLOBAL_FREE) {
                    if (P.last_column_free) {            // H(0, n)
                        const int32_t x = border(P, P.first_row_free, u.n[l]);
                        if (better(x, 0, u.n[l], u.cs[l], u.ci[l], u.cj[l])) { u.cs[l] = x; u.ci[l] = 0; u.cj[l] = u.n[l]; }
                    }
                    if (P.last_row_free) {               // H(m, 0)
                        const int32_t x = border(P, P.first_column_free, u.m[l]);
                        if (better(x, u.m[l], 0, u.cs[l], u.ci[l], u.cj[l])) { u.cs[l] = x; u.ci[l] = u.m[l]; u.cj[l] = 0; }
                    }
                }
                if (MODE != M_LOCAL &&
                    (int64_t)u.cs[l] - (int64_t)P.shift * u.ci[l] <= (int64_t)KC::floor_true) {
                    // a clamp may have reached this result: recompute it in s32
                    const uint32_t slot = atomicAdd(L.rerun_count, 1u);
                    L.rerun_list[slot] = u.id[l];
                    continue;
                }
                pa_result r;
                r.score = u.cs[l];
                r.end1 = u.ci[l];
                r.end2 = u.cj[l];
                r.width = 16;
                r.flags = 0;
                r.band_rounds = 0;
                if (MODE == M_LOCAL && u.cs[l] <= 0) { r.end1 = 0; r.end2 = 0; }
                L.out[u.id[l]] = r;
            }
        }
        __syncwarp(gmask);
    }
}

}  // namespace pa
