// pa_band_dp.cu -- banded global alignment with an admissible certificate.
//
// The reference has no banded mode; this is the accelerated form of its global
// score DP (affine_dp_algorithm.hpp:133-156 under method_global, all end gaps
// penalised) and must return exactly the same scores.  Per pair:
//
//   band      centre line through (0, 0), 8 checkpoints and (m, n) (BandSpec),
//             widened to also cover the end diagonal n - m, half-width tapering
//             from w_start at column 0 to w_min at column m (doubling per round);
//   windows   k_band_windows turns the band into one column window per pass of
//             G*R rows (the DP kernel computes whole rectangles of a pass);
//   DP        dp_kernel in M_BAND mode (pa_dp.cuh) computes the best score S of
//             paths that stay inside the windows, and the largest upper bound U
//             of any path that leaves them: the exact score on reaching the
//             last cell inside, plus the best the rest of the path could gain;
//   accept    U <= S proves that no path outside scores more, so S is the score.
//             Otherwise the band doubles; once its windows would cover more than
//             a set fraction of the matrix, the pair goes to the full DP.
#include <cuda_bf16.h>

#include <algorithm>

#include "pa_dp.cuh"

namespace pa {

// ---- band geometry -----------------------------------------------------------
struct Centre {
    int32_t x[10], y[10];
    int32_t m, n;
    __device__ void init(const BandSpec &B, int32_t m_, int32_t n_)
    {
        m = m_;
        n = n_;
        x[0] = 0;
        y[0] = 0;
        for (int c = 0; c < 8; ++c) {
            const int32_t xc = (int32_t)(((int64_t)(c + 1) * m) / 9);
            int64_t yc = (int64_t)xc + B.diag[c];
            yc = yc < y[c] ? y[c] : (yc > n ? n : yc);        // non-decreasing, inside [0, n]
            x[c + 1] = xc;
            y[c + 1] = (int32_t)yc;
        }
        x[9] = m;
        y[9] = n;
    }
    // centre row at column i, with k the segment cursor (moved forward or back)
    __device__ int32_t at(int32_t i, int &k) const
    {
        while (k < 8 && i > x[k + 1]) ++k;
        while (k > 0 && i < x[k]) --k;
        const int64_t dx = x[k + 1] - x[k];
        if (dx <= 0) return y[k + 1];
        return y[k] + (int32_t)(((int64_t)(y[k + 1] - y[k]) * (i - x[k])) / dx);
    }
};

__device__ __forceinline__ int32_t half_width(const BandSpec &B, int32_t i, int32_t m, int shift)
{
    const int64_t ws = (int64_t)B.w_start << shift, wm = (int64_t)B.w_min << shift;
    const int64_t w = wm + ((ws - wm) * (m - i)) / (m > 0 ? m : 1);
    return (int32_t)(w > (1 << 30) ? (1 << 30) : w);
}

// One warp per listed pair: per-pass windows {first, last column} of the band at width
// multiplier 2^shift, made monotone and overlapping like the DP kernel does; code[k] = 2 when
// the windows cover more than full_frac of the matrix (team_frac for pairs of at most
// team_max_n rows).  The lanes take 32 columns at a time:
// a warp scan gives the running maximum of the band's top (the first column that reaches a
// pass) and, going back from column m, the running minimum of its bottom (the last column
// that still reaches a pass); each pass boundary is written by the one lane that crosses it.
__global__ void k_band_windows(const uint64_t *__restrict__ off1, const uint64_t *__restrict__ off2,
                               const uint32_t *__restrict__ list, uint32_t count, const BandSpec *__restrict__ spec,
                               int32_t rows, int shift, float full_frac, float team_frac, int32_t team_max_n,
                               int2 *__restrict__ win, uint8_t *__restrict__ code,
                               unsigned long long *__restrict__ width_stats)
{
    const uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (k >= count) return;                       // whole warps: count is per warp
    const uint32_t id = list[k];
    const int32_t m = (int32_t)(off1[id + 1] - off1[id]), n = (int32_t)(off2[id + 1] - off2[id]);
    const BandSpec B = spec[id];
    int2 *wv = win + (off2[id] - off2[0]) / (uint64_t)rows + id;
    const int32_t P = (n + rows - 1) / rows;
    const int32_t dend = n - m;
    Centre C;
    C.init(B, m, n);
    // passes p with p * rows + 1 <= v (the top v reaches them)
    auto reached = [&](int64_t v) -> int32_t {
        if (v < 1) return 0;
        const int64_t q = (v - 1) / rows + 1;
        return q < P ? (int32_t)q : P;
    };
    // the first pass p with min((p + 1) * rows, n) >= v (a bottom v reaches it and every later one)
    auto first_reached = [&](int64_t v) -> int32_t {
        if (v > n) return P;
        if (v <= 0) return 0;
        const int64_t q = (v + rows - 1) / rows - 1;
        return q < P ? (int32_t)q : P;
    };
    int seg = 0;
    int64_t top = INT64_MIN;                      // running maximum before this chunk
    for (int32_t base = 1; base <= m && reached(top) < P; base += 32) {
        const int32_t i = base + lane;
        int64_t hi = INT64_MIN;
        if (i <= m) hi = (int64_t)max(C.at(i, seg), i + dend) + half_width(B, i, m, shift);
        int64_t run = max(hi, top);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, run, o);
            if (lane >= o) run = max(run, y);
        }
        int64_t before = __shfl_up_sync(0xffffffffu, run, 1);
        if (lane == 0) before = top;
        for (int32_t p = reached(before); p < reached(run); ++p) wv[p].x = i;
        top = __shfl_sync(0xffffffffu, run, 31);
    }
    for (int32_t p = reached(top) + lane; p < P; p += 32) wv[p].x = m;
    seg = 8;
    int64_t bot = INT64_MAX;                      // running minimum after this chunk
    for (int32_t base = m; base >= 1 && first_reached(bot) > 0; base -= 32) {
        const int32_t i = base - lane;
        int64_t lo = INT64_MAX;
        if (i >= 1) lo = (int64_t)min(C.at(i, seg), i + dend) - half_width(B, i, m, shift);
        int64_t run = min(lo, bot);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, run, o);
            if (lane >= o) run = min(run, y);
        }
        int64_t before = __shfl_up_sync(0xffffffffu, run, 1);
        if (lane == 0) before = bot;
        for (int32_t p = first_reached(run); p < first_reached(before); ++p) wv[p].y = i;
        bot = __shfl_sync(0xffffffffu, run, 31);
    }
    for (int32_t p = lane; p < first_reached(bot); p += 32) wv[p].y = 1;
    __syncwarp();
    if (lane != 0) return;
    // the same monotone, overlapping fix-up as the DP kernel; cells of the result
    int64_t cells = 0;
    int32_t pa = 1, pb = 1;
    for (int32_t p = 0; p < P; ++p) {
        int2 x = wv[p];
        if (p == 0) x.x = 1;
        else x.x = max(min(x.x, pb), pa);
        x.y = min(max(max(x.y, x.x), pb), m);
        if (p == P - 1) x.y = m;
        wv[p] = x;
        cells += (int64_t)(x.y - x.x + 1) * min(rows, n - p * rows);
        pa = x.x;
        pb = x.y;
    }
    const float frac = (n <= team_max_n && team_frac > 0.f) ? team_frac : full_frac;
    const bool full = (double)cells > (double)frac * (double)m * (double)n;
    code[k] = full ? 2 : 0;
    if (!full && width_stats) {          // mean window width of the banded pairs (team size)
        atomicAdd(width_stats, (unsigned long long)(cells / rows));
        atomicAdd(width_stats + 1, (unsigned long long)P);
    }
}

// The full DP's work kind of each listed pair, as the plain path's classifier routes long
// pairs: 2 clusters (m * n >= huge_cells and n >= huge_min_n), 0 teams of 4 warps (at most
// team_max_n rows), 1 whole blocks.
__global__ void k_size_code(const uint64_t *__restrict__ off1, const uint64_t *__restrict__ off2,
                            const uint32_t *__restrict__ list, uint32_t count, int32_t team_max_n, int64_t huge_cells,
                            int32_t huge_min_n, uint8_t *__restrict__ code)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const uint32_t id = list[k];
    const int64_t m = (int64_t)(off1[id + 1] - off1[id]), n = (int64_t)(off2[id + 1] - off2[id]);
    code[k] = (m * n >= huge_cells && n >= huge_min_n) ? 2 : (n <= team_max_n ? 0 : 1);
}

// Network outputs (16 floats per pair, 9 used) -> band: checkpoint diagonals
// out[c] * (m + n) / 4 and, from the predicted deficit c2 = 2^(16 out[8]) - 1
// (= smax (m + n) - 2 S), the starting half-width.  A path that leaves the band
// by d diagonals and comes back pays two gap opens and at least d extensions
// while the diagonal steps it gives up could gain at most smax each; the band
// proves itself once that cost exceeds the deficit D = c2 / 2 of the rest of the
// alignment: d >= (D - 2 |open|) / (|ext| + smax).
__global__ void k_band_decode(const float *__restrict__ out, const uint64_t *__restrict__ off1,
                              const uint64_t *__restrict__ off2, uint64_t n_pairs, DpParams P, float margin,
                              int32_t w_min, BandSpec *__restrict__ spec)
{
    const uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (k >= n_pairs) return;
    const int32_t m = (int32_t)(off1[k + 1] - off1[k]), n = (int32_t)(off2[k + 1] - off2[k]);
    const float *o = out + k * 16;
    BandSpec B;
    const float scale = (float)(m + n) * 0.25f;
    for (int c = 0; c < 8; ++c) B.diag[c] = __float2int_rn(o[c] * scale);
    const float c2 = exp2f(fminf(o[8], 1.5f) * 16.f) - 1.f;
    const float per = (float)(-P.gap_ext + P.smax);
    float ws = (0.5f * c2 + 2.f * (float)P.gap_open) / (per > 0.f ? per : 1.f);
    ws = margin * fmaxf(ws, 0.f) + (float)w_min;
    const float cap = (float)max(m, n) + 1.f;
    B.w_start = (int32_t)fminf(ws, cap);
    B.w_min = w_min;
    B.pad[0] = B.pad[1] = 0;
    spec[k] = B;
}

// The band without the network: the straight line from (0, 0) to (m, n) and a
// fixed starting half-width.
__global__ void k_band_straight(const uint64_t *__restrict__ off1, const uint64_t *__restrict__ off2,
                                uint64_t n_pairs, int32_t w_start, int32_t w_min, BandSpec *__restrict__ spec)
{
    const uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (k >= n_pairs) return;
    const int64_t m = (int64_t)(off1[k + 1] - off1[k]), n = (int64_t)(off2[k + 1] - off2[k]);
    BandSpec B;
    for (int c = 0; c < 8; ++c) {
        const int64_t xc = ((c + 1) * m) / 9;
        B.diag[c] = (int32_t)((m > 0 ? (xc * n) / m : 0) - xc);
    }
    B.w_start = w_start;
    B.w_min = w_min;
    B.pad[0] = B.pad[1] = 0;
    spec[k] = B;
}

// Host-given bands: 10 int32 per pair (diag[8], w_start, w_min).
__global__ void k_band_from_ints(const int32_t *__restrict__ in, uint64_t n_pairs, BandSpec *__restrict__ spec)
{
    const uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (k >= n_pairs) return;
    BandSpec B;
    for (int c = 0; c < 8; ++c) B.diag[c] = in[k * 10 + c];
    B.w_start = max(in[k * 10 + 8], 1);
    B.w_min = max(min(in[k * 10 + 9], B.w_start), 1);
    B.pad[0] = B.pad[1] = 0;
    spec[k] = B;
}

// ---- order-preserving compaction of a list by an outcome code -----------------
__device__ __forceinline__ uint32_t scan1024(uint32_t v, uint32_t *sh, uint32_t &total)
{
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[wp] = x;
    __syncthreads();
    if (wp == 0) {
        uint32_t s = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        sh[lane] = s;
    }
    __syncthreads();
    total = sh[(blockDim.x >> 5) - 1];
    const uint32_t before = wp > 0 ? sh[wp - 1] : 0u;
    __syncthreads();
    return before + x - v;
}

__global__ void __launch_bounds__(1024) k_compact_count(const uint8_t *__restrict__ code, uint32_t count, uint8_t sel,
                                                        uint32_t *__restrict__ block_sum)
{
    __shared__ uint32_t sh[32];
    const uint32_t k = blockIdx.x * 1024u + threadIdx.x;
    uint32_t total;
    scan1024(k < count && code[k] == sel, sh, total);
    if (threadIdx.x == 0) block_sum[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) k_compact_scan(uint32_t *__restrict__ block_sum, uint32_t nblocks,
                                                       uint32_t *__restrict__ total_out)
{
    __shared__ uint32_t sh[32];
    uint32_t carry = 0;
    for (uint32_t b0 = 0; b0 < nblocks; b0 += 1024) {
        const uint32_t b = b0 + threadIdx.x;
        uint32_t total;
        const uint32_t v = b < nblocks ? block_sum[b] : 0u;
        const uint32_t ex = scan1024(v, sh, total);
        if (b < nblocks) block_sum[b] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) *total_out = carry;
}

__global__ void __launch_bounds__(1024) k_compact_write(const uint32_t *__restrict__ list, const uint8_t *__restrict__ code,
                                                        uint32_t count, uint8_t sel,
                                                        const uint32_t *__restrict__ block_sum,
                                                        uint32_t *__restrict__ out)
{
    __shared__ uint32_t sh[32];
    const uint32_t k = blockIdx.x * 1024u + threadIdx.x;
    const bool take = k < count && code[k] == sel;
    uint32_t total;
    const uint32_t pos = scan1024(take, sh, total) + block_sum[blockIdx.x];
    if (take) out[pos] = list[k];
}

// Results that no certificate accepted were computed by the full DP.
__global__ void k_mark_full(pa_result *__restrict__ out, uint64_t n_pairs)
{
    const uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (k >= n_pairs) return;
    if (!(out[k].flags & (PA_RESULT_BANDED | PA_RESULT_TRIVIAL))) out[k].flags |= PA_RESULT_FULL_DP;
}

// ---- host-side launchers ---------------------------------------------------------
namespace {
constexpr int kBandVar = 36;     // branch-free top input, one-op vertical-gap chain, no table prefetch

template <class V, bool CTA>
int band_occ()
{
    static int per_sm = -1;
    if (per_sm < 0) {
        int v = 0;
        if (CTA)
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, dp_kernel_team<V, 16, M_BAND, false, kBandVar, 1>, kBlock, 0);
        else
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, dp_kernel<V, 16, M_BAND, false, kBandVar, 2>, kBlock, 0);
        per_sm = v < 1 ? 1 : v;
    }
    return per_sm;
}
inline unsigned blocks(uint64_t n, unsigned per) { return (unsigned)((n + per - 1) / per); }
}  // namespace

int band_dp_occupancy(bool lanes16, bool cta)
{
    if (cta) return lanes16 ? band_occ<L16, true>() : band_occ<L32, true>();
    return lanes16 ? band_occ<L16, false>() : band_occ<L32, false>();
}

int band_cta_occupancy() { return std::max(band_dp_occupancy(true, true), band_dp_occupancy(false, true)); }

// CTA launches use the ring rows of L (grid blocks of 8 rows each).
void band_dp_launch(bool lanes16, bool cta, int grid, cudaStream_t st, const DpLaunch &L, const DpParams &P)
{
    if (cta) {
        // teams of L.team warps per pair (narrow bands keep few passes in flight)
        if (lanes16) {
            if (L.team == 1) dp_kernel_team<L16, 16, M_BAND, false, kBandVar, 1><<<grid, kBlock, 0, st>>>(L, P);
            else if (L.team == 2) dp_kernel_team<L16, 16, M_BAND, false, kBandVar, 2><<<grid, kBlock, 0, st>>>(L, P);
            else if (L.team == 4) dp_kernel_team<L16, 16, M_BAND, false, kBandVar, 4><<<grid, kBlock, 0, st>>>(L, P);
            else dp_kernel_cta<L16, 16, M_BAND, false, kBandVar><<<grid, kBlock, 0, st>>>(L, P);
        } else {
            if (L.team == 1) dp_kernel_team<L32, 16, M_BAND, false, kBandVar, 1><<<grid, kBlock, 0, st>>>(L, P);
            else if (L.team == 2) dp_kernel_team<L32, 16, M_BAND, false, kBandVar, 2><<<grid, kBlock, 0, st>>>(L, P);
            else if (L.team == 4) dp_kernel_team<L32, 16, M_BAND, false, kBandVar, 4><<<grid, kBlock, 0, st>>>(L, P);
            else dp_kernel_cta<L32, 16, M_BAND, false, kBandVar><<<grid, kBlock, 0, st>>>(L, P);
        }
    } else if (lanes16) {
        dp_kernel<L16, 16, M_BAND, false, kBandVar, 2><<<grid, kBlock, 0, st>>>(L, P);
    } else {
        dp_kernel<L32, 16, M_BAND, false, kBandVar, 2><<<grid, kBlock, 0, st>>>(L, P);
    }
}

// width_stats (2 device words, may be null) accumulates the window widths and passes of
// the pairs that stay banded.
void band_windows_launch(cudaStream_t st, const uint64_t *off1, const uint64_t *off2, const uint32_t *list,
                         uint32_t count, const BandSpec *spec, int32_t rows, int shift, float full_frac,
                         float team_frac, int32_t team_max_n, int2 *win, uint8_t *code,
                         unsigned long long *width_stats)
{
    // one warp per pair
    if (count)
        k_band_windows<<<blocks((uint64_t)count * 32, 128), 128, 0, st>>>(
            off1, off2, list, count, spec, rows, shift, full_frac, team_frac, team_max_n, win, code, width_stats);
}

void size_code_launch(cudaStream_t st, const uint64_t *off1, const uint64_t *off2, const uint32_t *list,
                      uint32_t count, int32_t team_max_n, int64_t huge_cells, int32_t huge_min_n, uint8_t *code)
{
    if (count)
        k_size_code<<<blocks(count, 256), 256, 0, st>>>(off1, off2, list, count, team_max_n, huge_cells, huge_min_n,
                                                         code);
}

void band_decode_launch(cudaStream_t st, const float *out, const uint64_t *off1, const uint64_t *off2,
                        uint64_t n_pairs, const DpParams &P, float margin, int32_t w_min, BandSpec *spec)
{
    if (n_pairs) k_band_decode<<<blocks(n_pairs, 256), 256, 0, st>>>(out, off1, off2, n_pairs, P, margin, w_min, spec);
}

void band_straight_launch(cudaStream_t st, const uint64_t *off1, const uint64_t *off2, uint64_t n_pairs,
                          int32_t w_start, int32_t w_min, BandSpec *spec)
{
    if (n_pairs) k_band_straight<<<blocks(n_pairs, 256), 256, 0, st>>>(off1, off2, n_pairs, w_start, w_min, spec);
}

void band_from_ints_launch(cudaStream_t st, const int32_t *in, uint64_t n_pairs, BandSpec *spec)
{
    if (n_pairs) k_band_from_ints<<<blocks(n_pairs, 256), 256, 0, st>>>(in, n_pairs, spec);
}

// out[0 .. *total) = the entries of list[0 .. count) whose code is sel, in list order.
// block_sum needs ceil(count / 1024) + 1 words; total is a device word.
void compact_launch(cudaStream_t st, const uint32_t *list, const uint8_t *code, uint32_t count, uint8_t sel,
                    uint32_t *block_sum, uint32_t *out, uint32_t *total)
{
    const unsigned nb = count ? blocks(count, 1024) : 0;
    if (nb) k_compact_count<<<nb, 1024, 0, st>>>(code, count, sel, block_sum);
    k_compact_scan<<<1, 1024, 0, st>>>(block_sum, nb, total);
    if (nb) k_compact_write<<<nb, 1024, 0, st>>>(list, code, count, sel, block_sum, out);
}

void mark_full_launch(cudaStream_t st, pa_result *out, uint64_t n_pairs)
{
    if (n_pairs) k_mark_full<<<blocks(n_pairs, 256), 256, 0, st>>>(out, n_pairs);
}

}  // namespace pa
