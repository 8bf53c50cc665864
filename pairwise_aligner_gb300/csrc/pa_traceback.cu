// pa_traceback.cu -- the optimal alignment itself (begin cell and SAM-style ops), on the GPU.
//
// The reference computes scores only (every tracker carries "TODO: optimal_coordinate()",
// tracker/tracker_global_scalar.hpp, tracker/tracker_local_scalar.hpp).  This kernel runs the
// same recurrence with the same borders and end-cell rule as the score kernels
// (affine/affine_dp_algorithm.hpp:133-156, affine/affine_initialisation_strategy.hpp:38-51,
// matrix/dp_matrix_local.hpp:39-47) in int32 lanes, and keeps 4 direction bits per cell:
//   bits 0-1  where H(i,j) came from: 0 the diagonal, 1 P (a gap along sequence1), 2 Q (a gap
//             along sequence2), 3 local start (H == 0)
//   bit 2     P(i+1,j) extends P(i,j) (else it opens from H(i,j))
//   bit 3     Q(i,j+1) extends Q(i,j)
// Ties: the diagonal, then P, then Q; a gap opens unless extending is strictly better.
//
// Layout: one warp per pair, passes of 256 rows of sequence2, 8 rows per lane (the last pass
// ra = ceil(rows left / 32) rows per lane); lane t works on column s - t + 1 at step s, so the 32
// direction words of a step (ra rows x 4 bits each) are contiguous: word (p * (m + 31) + s) * 32
// + t.  The walk back reads cell (i, j) at p = (j-1) / 256, t = ((j-1) % 256) / ra_p,
// s = i + t - 1, nibble ((j-1) % 256) % ra_p.
#include <cuda_runtime.h>

#include <algorithm>

#include "pa_launch.h"

namespace pa {

constexpr int kTbRows = 8;
constexpr int kTbPassRows = 32 * kTbRows;
static_assert(kTbPassRows == kTracebackPassRows, "pass height shared with the host");

__device__ __forceinline__ bool tb_better(int32_t v, int32_t i, int32_t j, int32_t bv, int32_t bi, int32_t bj)
{
    return v > bv || (v == bv && (i < bi || (i == bi && j < bj)));
}

// One pair, as a warp sees it.
struct TbPair {
    int32_t m, n, S, passes, ra_last;
    const uint8_t *a_seq, *b_seq;
    uint32_t *D;
    Cell *bnd;
};

// Rows per lane of pass p: 8, and in the last pass just enough for its rows (1..8), so that
// at most 31 computed rows lie past the end of sequence2.
__device__ __forceinline__ int32_t tb_rows(const TbPair &w, int32_t p) { return p + 1 < w.passes ? kTbRows : w.ra_last; }

// One pass of RA rows per lane: rows p * 256 + lane * RA + 1 .. + RA of sequence2, streamed
// over the columns of sequence1.  Candidates of the end cell go to (bv, bi, bj).
template <bool LOCAL, bool MAT, int RA>
__device__ __forceinline__ void tb_pass(const TbLaunch &L, const DpParams &P, const TbPair &w, int32_t p, int lane,
                                        int32_t &bv, int32_t &bi, int32_t &bj)
{
    const int32_t goe = P.gap_open + P.gap_ext, ext = P.gap_ext;
    const int fcf = P.first_column_free, frf = P.first_row_free;
    const bool lcf = P.last_column_free, lrf = P.last_row_free;
    const int32_t m = w.m, n = w.n;
    const int32_t j0 = p * kTbPassRows + lane * RA;                   // rows j0+1 .. j0+RA
    const int32_t nvalid = min(max(n - j0, 0), RA);                   // rows of this lane within n
    const bool holds_n = n > j0 && n <= j0 + RA;
    int32_t H[RA], Pg[RA], bsym[RA];
#pragma unroll
    for (int r = 0; r < RA; ++r) {
        const int32_t j = j0 + r + 1;
        const uint32_t b = r < nvalid ? w.b_seq[j - 1] : 0u;
        bsym[r] = MAT ? (r < nvalid ? (int32_t)L.rank[b] : 0) : (int32_t)b;   // rows past n: any rank
        H[r] = border(P, frf, j);                                          // H(0, j)
        Pg[r] = H[r] + goe;                                                // P(1, j)
    }
    int32_t prevH = border(P, frf, j0);                                   // H(0, j0)
    int32_t outH = 0, outQ = 0;
    // local: a lane meets its cells of one pass in (i, j) order, so only a strictly larger column
    // maximum can be a better candidate
    int32_t pv = INT32_MIN, pi = 0, pj = 0;
    for (int32_t s = 0; s < w.S; ++s) {
        int32_t upH = __shfl_up_sync(0xffffffffu, outH, 1);
        int32_t upQ = __shfl_up_sync(0xffffffffu, outQ, 1);
        const int32_t i = s - lane + 1;
        if (i < 1 || i > m) continue;
        if (lane == 0) {
            if (p == 0) {
                upH = border(P, fcf, i);                                   // H(i, 0)
                upQ = upH + goe;                                           // Q(i, 1)
            } else {
                const Cell c = w.bnd[i];
                upH = (int32_t)c.h;
                upQ = (int32_t)c.e;
            }
        }
        const uint32_t a = w.a_seq[i - 1];
        const int32_t arow = MAT ? (int32_t)L.rank[a] * L.dim : 0;
        int32_t diag = prevH, qg = upQ;
        uint32_t word = 0;
#pragma unroll
        for (int r = 0; r < RA; ++r) {
            const int32_t sc = MAT ? __ldg(L.matrix + arow + bsym[r]) : ((int32_t)a == bsym[r] ? P.match : P.mismatch);
            int32_t d = diag + sc;
            if (LOCAL) d = max(d, 0);
            const int32_t pc = Pg[r];
            const int32_t h = __vimax3_s32(d, pc, qg);
            const uint32_t src = (LOCAL && h == 0) ? 3u : (h == d ? 0u : (h == pc ? 1u : 2u));
            const int32_t pe = pc + ext, po = h + goe;
            const int32_t qe = qg + ext;
            word |= (src | ((uint32_t)(pe > po) << 2) | ((uint32_t)(qe > po) << 3)) << (4 * r);
            Pg[r] = max(pe, po);
            qg = max(qe, po);
            diag = H[r];
            H[r] = h;
        }
        if (LOCAL) {
            int32_t cm = INT32_MIN;
#pragma unroll
            for (int r = 0; r < RA; ++r) cm = max(cm, r < nvalid ? H[r] : INT32_MIN);
            if (cm > pv) {
                int32_t first = RA - 1;
#pragma unroll
                for (int r = RA - 1; r >= 0; --r)
                    if (r < nvalid && H[r] == cm) first = r;
                pv = cm;
                pi = i;
                pj = j0 + first + 1;
            }
        } else {
            if (lcf && holds_n) {                                          // H(i, n)
#pragma unroll
                for (int r = 0; r < RA; ++r)
                    if (j0 + r + 1 == n && tb_better(H[r], i, n, bv, bi, bj)) { bv = H[r]; bi = i; bj = n; }
            }
            if (i == m) {
#pragma unroll
                for (int r = 0; r < RA; ++r) {
                    const int32_t j = j0 + r + 1;
                    if (r < nvalid && (lrf || j == n) && tb_better(H[r], m, j, bv, bi, bj)) {
                        bv = H[r]; bi = m; bj = j;
                    }
                }
            }
        }
        prevH = upH;
        outH = H[RA - 1];
        outQ = qg;
        w.D[((int64_t)p * w.S + s) * 32 + lane] = word;
        if (lane == 31 && p + 1 < w.passes) w.bnd[i] = Cell{(uint32_t)H[RA - 1], (uint32_t)qg};
    }
    if (LOCAL && tb_better(pv, pi, pj, bv, bi, bj)) { bv = pv; bi = pi; bj = pj; }
    __syncwarp();                                 // the boundary row, for lane 0 of the next pass
}

template <bool LOCAL, bool MAT>
__device__ __forceinline__ void tb_last_pass(const TbLaunch &L, const DpParams &P, const TbPair &w, int32_t p,
                                             int lane, int32_t &bv, int32_t &bi, int32_t &bj)
{
    switch (w.ra_last) {
    case 1: tb_pass<LOCAL, MAT, 1>(L, P, w, p, lane, bv, bi, bj); break;
    case 2: tb_pass<LOCAL, MAT, 2>(L, P, w, p, lane, bv, bi, bj); break;
    case 3: tb_pass<LOCAL, MAT, 3>(L, P, w, p, lane, bv, bi, bj); break;
    case 4: tb_pass<LOCAL, MAT, 4>(L, P, w, p, lane, bv, bi, bj); break;
    case 5: tb_pass<LOCAL, MAT, 5>(L, P, w, p, lane, bv, bi, bj); break;
    case 6: tb_pass<LOCAL, MAT, 6>(L, P, w, p, lane, bv, bi, bj); break;
    case 7: tb_pass<LOCAL, MAT, 7>(L, P, w, p, lane, bv, bi, bj); break;
    default: tb_pass<LOCAL, MAT, 8>(L, P, w, p, lane, bv, bi, bj); break;
    }
}

// LOCAL: method_local; MAT: substitution-matrix scores (else match / mismatch on raw bytes).
template <bool LOCAL, bool MAT>
__global__ void __launch_bounds__(128) k_traceback(TbLaunch L, DpParams P)
{
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const int fcf = P.first_column_free, frf = P.first_row_free;
    const bool lcf = P.last_column_free, lrf = P.last_row_free;

    for (uint32_t q = warp; q < L.count; q += nwarps) {
        const uint32_t k = L.first + q;
        const uint64_t q0 = L.off1[k], t0 = L.off2[k];
        TbPair w;
        w.m = (int32_t)(L.off1[k + 1] - q0);
        w.n = (int32_t)(L.off2[k + 1] - t0);
        w.a_seq = L.seq1 + q0;
        w.b_seq = L.seq2 + t0;
        w.D = L.dir + L.dir_off[q];
        w.bnd = L.bnd + (q0 - L.off1[0]) + k;
        w.S = w.m + 31;
        w.passes = (w.n + kTbPassRows - 1) / kTbPassRows;
        w.ra_last = w.passes ? (w.n - (w.passes - 1) * kTbPassRows + 31) / 32 : kTbRows;
        const int32_t m = w.m, n = w.n;

        // end-cell candidates of this lane (value, i, j); lane 0 adds the border ones
        int32_t bv = INT32_MIN, bi = INT32_MAX, bj = INT32_MAX;
        if (!LOCAL && lane == 0) {
            auto cand = [&](int32_t v, int32_t i, int32_t j) {
                if (tb_better(v, i, j, bv, bi, bj)) { bv = v; bi = i; bj = j; }
            };
            if (m == 0 || n == 0) cand(m == 0 ? border(P, frf, n) : border(P, fcf, m), m, n);
            if (lcf) {
                cand(border(P, frf, n), 0, n);
                if (n == 0)
                    for (int32_t i = 1; i <= m; ++i) cand(border(P, fcf, i), i, 0);
            }
            if (lrf) {
                cand(border(P, fcf, m), m, 0);
                if (m == 0)
                    for (int32_t j = 1; j <= n; ++j) cand(border(P, frf, j), 0, j);
            }
        }
        if (m > 0 && n > 0) {
            for (int32_t p = 0; p + 1 < w.passes; ++p) tb_pass<LOCAL, MAT, kTbRows>(L, P, w, p, lane, bv, bi, bj);
            tb_last_pass<LOCAL, MAT>(L, P, w, w.passes - 1, lane, bv, bi, bj);
        }
        // the end cell: the best candidate over the warp
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const int32_t ov = __shfl_xor_sync(0xffffffffu, bv, o);
            const int32_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
            const int32_t oj = __shfl_xor_sync(0xffffffffu, bj, o);
            if (tb_better(ov, oi, oj, bv, bi, bj)) { bv = ov; bi = oi; bj = oj; }
        }
        __syncwarp();                             // every direction word is visible to lane 0
        const uint64_t obase = (q0 - L.off1[0]) + (t0 - L.off2[0]);
        uint8_t *ops = L.ops + obase;
        int32_t score = bv, e1 = bi, e2 = bj;
        if (LOCAL) {
            if (m == 0 || n == 0) { score = INT32_MIN; e1 = e2 = 0; }
            else if (bv <= 0) { score = max(bv, 0); e1 = e2 = 0; }
        }
        int32_t nops = 0, b1 = 0, b2 = 0;
        if (lane == 0 && !(LOCAL && (m == 0 || n == 0 || score <= 0))) {
            int32_t i = e1, j = e2, state = 0;
            auto nib = [&](int32_t ci, int32_t cj) -> uint32_t {
                const int32_t pp = (cj - 1) / kTbPassRows, r = (cj - 1) % kTbPassRows;
                const int32_t ra = tb_rows(w, pp);
                const int32_t tt = r / ra, kk = r % ra;
                const uint32_t word = w.D[((int64_t)pp * w.S + (ci + tt - 1)) * 32 + tt];
                return (word >> (4 * kk)) & 15u;
            };
            for (;;) {
                if (state == 0) {
                    if (i == 0 || j == 0) {
                        if (i == 0 && j > 0 && !frf) { while (j > 0) { ops[nops++] = 'I'; --j; } }
                        else if (j == 0 && i > 0 && !fcf) { while (i > 0) { ops[nops++] = 'D'; --i; } }
                        break;
                    }
                    const uint32_t src = nib(i, j) & 3u;
                    if (src == 3u) break;
                    if (src == 0u) {
                        ops[nops++] = w.a_seq[i - 1] == w.b_seq[j - 1] ? '=' : 'X';
                        --i;
                        --j;
                    } else {
                        state = (int32_t)src;
                    }
                } else if (state == 1) {
                    ops[nops++] = 'D';
                    --i;
                    state = (i >= 1 && j >= 1 && (nib(i, j) & 4u)) ? 1 : 0;
                } else {
                    ops[nops++] = 'I';
                    --j;
                    state = (j >= 1 && i >= 1 && (nib(i, j) & 8u)) ? 2 : 0;
                }
            }
            b1 = i;
            b2 = j;
        }
        nops = __shfl_sync(0xffffffffu, nops, 0);
        b1 = __shfl_sync(0xffffffffu, b1, 0);
        b2 = __shfl_sync(0xffffffffu, b2, 0);
        __syncwarp();
        for (int32_t x = lane; x < nops / 2; x += 32) {             // path order
            const uint8_t u = ops[x];
            ops[x] = ops[nops - 1 - x];
            ops[nops - 1 - x] = u;
        }
        if (lane == 0) {
            pa_result res;
            res.score = score;
            res.end1 = e1;
            res.end2 = e2;
            res.width = 32;
            res.flags = (m == 0 || n == 0) ? PA_RESULT_TRIVIAL : 0;
            res.band_rounds = 0;
            L.out[k] = res;
            pa_alignment al;
            al.begin1 = b1;
            al.begin2 = b2;
            al.n_ops = (uint32_t)nops;
            al.reserved = 0;
            L.aln[k] = al;
        }
        __syncwarp();
    }
}

int traceback_grid(int sm_count)
{
    int per_sm = 0, v = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_traceback<false, false>, 128, 0);
    per_sm = v;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_traceback<true, false>, 128, 0);
    per_sm = std::min(per_sm, v);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_traceback<false, true>, 128, 0);
    per_sm = std::min(per_sm, v);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_traceback<true, true>, 128, 0);
    per_sm = std::min(per_sm, v);
    return std::max(1, per_sm) * sm_count;
}

void traceback_launch(int grid, cudaStream_t st, const TbLaunch &L, const DpParams &P)
{
    const bool mat = L.matrix != nullptr;
    if (P.local) {
        if (mat) k_traceback<true, true><<<grid, 128, 0, st>>>(L, P);
        else k_traceback<true, false><<<grid, 128, 0, st>>>(L, P);
    } else {
        if (mat) k_traceback<false, true><<<grid, 128, 0, st>>>(L, P);
        else k_traceback<false, false><<<grid, 128, 0, st>>>(L, P);
    }
}

}  // namespace pa
