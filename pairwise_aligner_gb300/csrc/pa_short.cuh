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
//    sequence1 bytes, the top border of the first pass); the last thread writes the
//    pass's bottom row back into the .h/.e halves for the next pass;
//  * thread 0 reads one slot per column with a single vector load, one column ahead, and
//    the score tables travel down the group with the H and gap values by shuffle, so no
//    other thread loads anything per column (thread 0 selects the slot's values);
//  * the rows are written so that the diagonal term of row k + 1 is formed before row k's
//    new H replaces the old one (no register copies between column steps);
//  * the unit's description, the per-thread candidates and the column of the last local
//    improvement live in shared memory, so the registers hold the R rows (R = 32 halves
//    the column steps of R = 16).
#pragma once
#include "pa_dp.cuh"

namespace pa {

// The unit a group works on: two pairs in s16x2 lanes (lane B may be absent).
struct ShortUnit {
    uint32_t id[2];
    uint64_t toff[2];
    int32_t m[2], n[2];
    int32_t ms, nh, passes, has_b;
    Slot *slot;                    // slots 1..ms of the unit (slot 0 unused)
};

template <int MODE>
struct ShortConst {
    static constexpr int32_t Kt = MODE == M_LOCAL ? 2048 : 32767 - 512;   // stored = true + Kt (+ shift)
    static constexpr int32_t clampt = 2048;
    static constexpr int32_t floor_true = MODE == M_LOCAL ? 0 : 2048 - Kt;
};

// Per-thread shared-memory state: result candidates (score, end1, end2) of both lanes and,
// in local mode, the column of each lane's last improvement in the current pass.
struct ShortShared {
    int32_t (*c)[3][kBlock];       // [lane][field][thread]
    int32_t (*bi)[kBlock];         // [lane][thread]
    __device__ __forceinline__ int32_t &s(int l) { return c[l][0][threadIdx.x]; }
    __device__ __forceinline__ int32_t &i(int l) { return c[l][1][threadIdx.x]; }
    __device__ __forceinline__ int32_t &j(int l) { return c[l][2][threadIdx.x]; }
    __device__ __forceinline__ void offer(int l, int32_t xs, int32_t xi, int32_t xj)
    {
        if (better(xs, xi, xj, s(l), i(l), j(l))) { s(l) = xs; i(l) = xi; j(l) = xj; }
    }
};

// One pass p of the unit: rows p*G*R + t*RA + 1 .. + RA (1-based) on thread t.
template <int MODE, int G, int R, int RA>
__device__ __forceinline__ void short_pass(const DpLaunch &L, const DpParams &P, const ShortUnit &u, int p, int t,
                                           unsigned gmask, uint4 *snap, ShortShared sh)
{
    using V = L16;
    using KC = ShortConst<MODE>;
    constexpr bool SHIFTED = MODE != M_LOCAL;      // local mode has no column shift (P.shift == 0)
    const int32_t rows_full = G * R;
    const int32_t j0 = p * rows_full + t * RA;
    const uint32_t GOEA = V::cabs(P.gap_open + P.gap_ext);
    const uint32_t EXTA = V::cabs(P.gap_ext);
    const uint32_t GOEH = SHIFTED ? V::cabs(P.gap_open + P.gap_ext - P.shift) : GOEA;
    const uint32_t EXTH = SHIFTED ? V::cabs(P.gap_ext - P.shift) : EXTA;
    const uint32_t CLAMP = V::splat(KC::clampt);
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
    const bool writer = t == G - 1 && p + 1 < u.passes;
    const bool t0 = t == 0;
    const int32_t ms = u.ms;
    Slot *const slot = u.slot;
    const int32_t um[2] = {u.m[0], u.m[1]}, un[2] = {u.n[0], u.n[1]};
    const bool has_b = u.has_b != 0;

    // the registers a thread hands on: bottom H and gap of its strip and the column's tables
    uint32_t sH = 0, sE = 0, sA = 0, sB = 0;
    uint4 nx = make_uint4(0u, 0u, 0u, 0u);        // thread 0: the slot of its next column
    if (t0) nx = *reinterpret_cast<const uint4 *>(slot + 1);
    uint32_t best = V::splat(KC::Kt);
    // global modes: where rows n[0], n[1] live
    int32_t own_k[2] = {0, 0};
    bool own[2] = {false, false};
    if (MODE != M_LOCAL) {
#pragma unroll
        for (int l = 0; l < 2; ++l) {
            const int32_t r = (un[l] - 1) - j0;
            own[l] = r >= 0 && r < RA && (un[l] - 1) / rows_full == p;
            own_k[l] = r;
        }
    }

    // step s of the pass: thread t computes column i = s - t + 1 when 1 <= i <= ms
    auto step = [&](int32_t s, bool active) {
        const int32_t i = s - t + 1;
        const uint32_t xH = __shfl_up_sync(gmask, sH, 1, G);
        const uint32_t xE = __shfl_up_sync(gmask, sE, 1, G);
        const uint32_t xA = __shfl_up_sync(gmask, sA, 1, G);
        const uint32_t xB = __shfl_up_sync(gmask, sB, 1, G);
        if (active) {
            const uint32_t upH = t0 ? nx.z : xH;
            uint32_t Ed = t0 ? nx.w : xE;
            const uint32_t ta = t0 ? nx.x : xA;
            const uint32_t tb = t0 ? nx.y : xB;
            if (t0 && i < ms) nx = *reinterpret_cast<const uint4 *>(slot + i + 1);
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
            sH = H[RA - 1];
            sE = Ed;
            sA = ta;
            sB = tb;
            if (writer) *reinterpret_cast<uint2 *>(&slot[i].h) = make_uint2(sH, sE);
            if (MODE == M_LOCAL) {
                const uint32_t cm = tree_max<V, RA>(H);
                const uint32_t nb = V::max2(best, cm);
                const uint32_t x = nb ^ best;
                best = nb;
                if (x != 0u) {
#pragma unroll
                    for (int l = 0; l < 2; ++l) {
                        if (V::improved(x, l)) {
                            sh.bi[l][threadIdx.x] = i;
#pragma unroll
                            for (int v = 0; v < RA / 4; ++v)
                                snap[(l * (R / 4) + v) * kBlock] =
                                    make_uint4(H[4 * v], H[4 * v + 1], H[4 * v + 2], H[4 * v + 3]);
                        }
                    }
                }
            } else {
#pragma unroll
                for (int l = 0; l < 2; ++l) {
                    if (l == 1 && !has_b) continue;
                    if (MODE == M_GLOBAL_FREE && P.last_column_free && own[l] && i <= um[l]) {
                        uint32_t v = H[0];
#pragma unroll
                        for (int k = 1; k < RA; ++k)
                            if (own_k[l] == k) v = H[k];
                        sh.offer(l, V::get(v, l) - KC::Kt + P.shift * i, i, un[l]);
                    }
                    if (i == um[l]) {
                        if (MODE == M_GLOBAL_FREE && P.last_row_free) {
#pragma unroll
                            for (int k = 0; k < RA; ++k)
                                if (j0 + k + 1 <= un[l])
                                    sh.offer(l, V::get(H[k], l) - KC::Kt + P.shift * i, i, j0 + k + 1);
                        } else if (own[l]) {
                            uint32_t v = H[0];
#pragma unroll
                            for (int k = 1; k < RA; ++k)
                                if (own_k[l] == k) v = H[k];
                            sh.offer(l, V::get(v, l) - KC::Kt + P.shift * i, i, un[l]);
                        }
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
        step(s, i >= 1 && i <= ms);
    }
    for (; s < ms; ++s) step(s, true);
    for (; s < ms + G - 1; ++s) {
        const int32_t i = s - t + 1;
        step(s, i >= 1 && i <= ms);
    }
    if (MODE == M_LOCAL) {
#pragma unroll
        for (int l = 0; l < 2; ++l) {
            const int32_t b = V::get(best, l);
            if (b > KC::Kt) {                     // improved in this pass: snapshot and column are set
                int32_t kk = 0;
                for (int v = RA / 4 - 1; v >= 0; --v) {
                    const uint4 q = snap[(l * (R / 4) + v) * kBlock];
                    if (V::get(q.w, l) == b) kk = 4 * v + 3;
                    if (V::get(q.z, l) == b) kk = 4 * v + 2;
                    if (V::get(q.y, l) == b) kk = 4 * v + 1;
                    if (V::get(q.x, l) == b) kk = 4 * v;
                }
                sh.offer(l, b - KC::Kt, sh.bi[l][threadIdx.x], j0 + kk + 1);
            }
        }
    }
}

// The short-pair kernel: a persistent grid whose warps take units of 32/G groups x two
// pairs from the class queue, largest shapes first; R rows of sequence2 per thread.
template <int MODE, int G, int R>
__global__ void __launch_bounds__(kBlock, 2) dp_short(DpLaunch L, DpParams P)
{
    static_assert(R % kChunk == 0 && R <= 32, "R must be a multiple of the chunk");
    using V = L16;
    using KC = ShortConst<MODE>;
    constexpr int NGROUPS = kBlock / G;
    __shared__ uint4 snap_store[MODE == M_LOCAL ? 2 * (R / 4) * kBlock : 1];
    __shared__ ShortUnit s_unit[NGROUPS];
    __shared__ int32_t s_cand[2][3][kBlock];
    __shared__ int32_t s_bi[MODE == M_LOCAL ? 2 : 1][kBlock];
    uint4 *snap = snap_store + threadIdx.x;
    ShortShared sh{s_cand, s_bi};
    const int lane = threadIdx.x & 31;
    const int t = lane & (G - 1);
    const int g = lane / G;
    ShortUnit &su = s_unit[threadIdx.x / G];
    const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (g * G));
    const uint32_t count = *L.count_ptr;
    const uint32_t *order = L.order + *L.begin_ptr;
    constexpr uint32_t ppw = (uint32_t)(32 / G) * 2;   // pairs per warp unit
    const uint32_t n_units = (count + ppw - 1) / ppw;
    const uint32_t match4 = (uint8_t)(P.match - P.shift) * 0x01010101u;
    const uint32_t mis4 = (uint8_t)(P.mismatch - P.shift) * 0x01010101u;

    for (;;) {
        uint32_t uu = 0;
        if (lane == 0) uu = atomicAdd(L.unit_counter, 1u);
        uu = __shfl_sync(0xffffffffu, uu, 0);
        if (uu >= n_units) break;
        uu = n_units - 1 - uu;                       // largest shapes first
        const uint32_t first = uu * ppw + (uint32_t)g * 2;
        if (first >= count) continue;                // idle group in the last unit
        if (t == 0) {
            ShortUnit u;
            u.id[0] = order[first];
            u.has_b = first + 1 < count;
            u.id[1] = u.has_b ? order[first + 1] : u.id[0];
            for (int l = 0; l < 2; ++l) {
                const uint64_t q0 = L.off1[u.id[l]];
                u.m[l] = (int32_t)(L.off1[u.id[l] + 1] - q0);
                u.toff[l] = L.off2[u.id[l]];
                u.n[l] = (int32_t)(L.off2[u.id[l] + 1] - u.toff[l]);
            }
            u.ms = max(u.m[0], u.m[1]);
            u.nh = max(u.n[0], u.n[1]);
            u.passes = (u.nh + G * R - 1) / (G * R);
            const uint32_t owner = u.m[1] > u.m[0] ? u.id[1] : u.id[0];
            u.slot = L.slots + (L.off1[owner] + owner);   // slots 0..m(owner) = 0..ms
            su = u;
        }
        for (int l = 0; l < 2; ++l) {
            sh.s(l) = MODE == M_LOCAL ? 0 : INT32_MIN;
            sh.i(l) = 0;
            sh.j(l) = 0;
        }
        __syncwarp(gmask);
        // the unit's slots: both lanes' score tables (a padding table past a lane's end) and
        // the top border of the first pass, H(i, 0) - shift * i
        {
            const uint64_t qa = L.off1[su.id[0]], qb = L.off1[su.id[1]];
            const int32_t ma = su.m[0], mb = su.m[1];
            const uint32_t GOEA = V::cabs(P.gap_open + P.gap_ext);
            for (int32_t i = 1 + t; i <= su.ms; i += G) {
                const uint32_t a = i <= ma ? score_table(L.seq1[qa + i - 1], match4, mis4) : 0x80808080u;
                const uint32_t b = i <= mb ? score_table(L.seq1[qb + i - 1], match4, mis4) : 0x80808080u;
                const int64_t top = (int64_t)border(P, P.first_column_free, i) - (int64_t)P.shift * i + KC::Kt;
                const uint32_t h = V::splat((int32_t)max(top, (int64_t)KC::clampt));
                *reinterpret_cast<uint4 *>(su.slot + i) = make_uint4(a, b, h, V::subc(h, GOEA));
            }
        }
        __syncwarp(gmask);
        const int32_t passes = su.passes;
        for (int p = 0; p < passes; ++p) {
            const ShortUnit u = su;
            const int32_t rem = u.nh - p * G * R;
            const int32_t rpt = rem >= G * R ? R : ((rem + G * kChunk - 1) / (G * kChunk)) * kChunk;
            switch (rpt / kChunk) {
            case 1: short_pass<MODE, G, R, 4>(L, P, u, p, t, gmask, snap, sh); break;
            case 2: short_pass<MODE, G, R, (R >= 8 ? 8 : R)>(L, P, u, p, t, gmask, snap, sh); break;
            case 3: short_pass<MODE, G, R, (R >= 12 ? 12 : R)>(L, P, u, p, t, gmask, snap, sh); break;
            case 4: short_pass<MODE, G, R, (R >= 16 ? 16 : R)>(L, P, u, p, t, gmask, snap, sh); break;
            case 5: short_pass<MODE, G, R, (R >= 20 ? 20 : R)>(L, P, u, p, t, gmask, snap, sh); break;
            case 6: short_pass<MODE, G, R, (R >= 24 ? 24 : R)>(L, P, u, p, t, gmask, snap, sh); break;
            case 7: short_pass<MODE, G, R, (R >= 28 ? 28 : R)>(L, P, u, p, t, gmask, snap, sh); break;
            default: short_pass<MODE, G, R, R>(L, P, u, p, t, gmask, snap, sh); break;
            }
            __syncwarp(gmask);
        }
        // reduce over the group, then thread 0 writes the results
        int32_t cs[2], ci[2], cj[2];
#pragma unroll
        for (int l = 0; l < 2; ++l) {
            cs[l] = sh.s(l);
            ci[l] = sh.i(l);
            cj[l] = sh.j(l);
            for (int off = G >> 1; off >= 1; off >>= 1) {
                const int32_t os = __shfl_xor_sync(gmask, cs[l], off, G);
                const int32_t oi = __shfl_xor_sync(gmask, ci[l], off, G);
                const int32_t oj = __shfl_xor_sync(gmask, cj[l], off, G);
                if (better(os, oi, oj, cs[l], ci[l], cj[l])) { cs[l] = os; ci[l] = oi; cj[l] = oj; }
            }
        }
        if (t == 0) {
            const ShortUnit u = su;
#pragma unroll
            for (int l = 0; l < 2; ++l) {
                if (l == 1 && !u.has_b) continue;
                if (MODE == M_GLOBAL_FREE) {
                    if (P.last_column_free) {            // H(0, n)
                        const int32_t x = border(P, P.first_row_free, u.n[l]);
                        if (better(x, 0, u.n[l], cs[l], ci[l], cj[l])) { cs[l] = x; ci[l] = 0; cj[l] = u.n[l]; }
                    }
                    if (P.last_row_free) {               // H(m, 0)
                        const int32_t x = border(P, P.first_column_free, u.m[l]);
                        if (better(x, u.m[l], 0, cs[l], ci[l], cj[l])) { cs[l] = x; ci[l] = u.m[l]; cj[l] = 0; }
                    }
                }
                if (MODE != M_LOCAL && (int64_t)cs[l] - (int64_t)P.shift * ci[l] <= (int64_t)KC::floor_true) {
                    // a clamp may have reached this result: recompute it in s32
                    const uint32_t slot = atomicAdd(L.rerun_count, 1u);
                    L.rerun_list[slot] = u.id[l];
                    continue;
                }
                pa_result r;
                r.score = cs[l];
                r.end1 = ci[l];
                r.end2 = cj[l];
                r.width = 16;
                r.flags = 0;
                r.band_rounds = 0;
                if (MODE == M_LOCAL && cs[l] <= 0) { r.end1 = 0; r.end2 = 0; }
                L.out[u.id[l]] = r;
            }
        }
        __syncwarp(gmask);
    }
}

}  // namespace pa
