// pa_band.cu -- the learned band for global alignment: features, the BF16 MLP
// (forward, backward, Adam), and the banded DP with its certificate.
//
// None of this has a counterpart in the reference (it has no banded or
// heuristic mode); the full DP of pa_dp.cuh stays the exact fallback and arbiter.
//
// Features (k_kmer_hist): a 128-bin histogram of the diagonal offsets j - i of
// 12-mers shared by sequence1 (position i) and sequence2 (position j), bins
// spanning [-m, n], normalised by the number of sequence1 12-mers, plus m/1024
// and n/1024: 130 inputs.
//
// Network: 130 -> 256 -> 256 -> 9 (8 band-centre checkpoints as diagonals /
// (m + n), and log2 of the half-width), ReLU, BF16 weights and activations,
// FP32 accumulate (mma.sync m16n8k16), FP32 master weights, loss and Adam.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/pairwise_aligner_gb300.h"

namespace pa {

constexpr int kFeat = 130, kFeatPad = 144, kHidden = 256, kOut = 9, kOutPad = 16;
constexpr int kHashSlots = 8192;            // shared-memory 12-mer table per block
constexpr uint32_t kEmpty = 0xffffffffu;

__device__ __forceinline__ int base_code(uint8_t b)
{
    switch (b) {
    case 'A': return 0;
    case 'C': return 1;
    case 'G': return 2;
    case 'T': return 3;
    default: return -1;
    }
}

// 2-bit packed 12-mer starting at s[x], or kEmpty if it holds a byte outside A/C/G/T.
__device__ __forceinline__ uint32_t kmer12(const uint8_t *s, int64_t x)
{
    uint32_t key = 0;
#pragma unroll
    for (int u = 0; u < 12; ++u) {
        const int c = base_code(s[x + u]);
        if (c < 0) return kEmpty;
        key = (key << 2) | (uint32_t)c;
    }
    return key;
}

__device__ __forceinline__ uint32_t slot_of(uint32_t key) { return (key * 2654435761u) >> 19; }   // 13 bits

// One block per pair.  Sequence2 12-mers go into an open-addressing table (first
// position kept; long sequences are subsampled to fit); every sequence1 12-mer
// probes it and adds its diagonal to the histogram.
__global__ void __launch_bounds__(256) k_kmer_hist(const uint8_t *__restrict__ seq1, const uint64_t *__restrict__ off1,
                                                   const uint8_t *__restrict__ seq2, const uint64_t *__restrict__ off2,
                                                   uint64_t n_pairs, float *__restrict__ feat)
{
    __shared__ uint32_t keys[kHashSlots];
    __shared__ int32_t pos[kHashSlots];
    __shared__ uint32_t hist[128];
    __shared__ uint32_t n_query;
    for (uint64_t p = blockIdx.x; p < n_pairs; p += gridDim.x) {
        const uint64_t q0 = off1[p], t0 = off2[p];
        const int64_t m = (int64_t)(off1[p + 1] - q0), n = (int64_t)(off2[p + 1] - t0);
        for (int x = threadIdx.x; x < kHashSlots; x += blockDim.x) { keys[x] = kEmpty; pos[x] = INT32_MAX; }
        if (threadIdx.x < 128) hist[threadIdx.x] = 0;
        if (threadIdx.x == 0) n_query = 0;
        __syncthreads();
        const int64_t stride = n > 6000 ? (n + 5999) / 6000 : 1;
        for (int64_t j = threadIdx.x * stride; j + 12 <= n; j += (int64_t)blockDim.x * stride) {
            const uint32_t key = kmer12(seq2 + t0, j);
            if (key == kEmpty) continue;
            uint32_t sl = slot_of(key);
            for (int probe = 0; probe < kHashSlots; ++probe) {
                const uint32_t prev = atomicCAS(&keys[sl], kEmpty, key);
                if (prev == kEmpty || prev == key) { atomicMin(&pos[sl], (int32_t)j); break; }
                sl = (sl + 1) & (kHashSlots - 1);
            }
        }
        __syncthreads();
        for (int64_t i = threadIdx.x; i + 12 <= m; i += blockDim.x) {
            const uint32_t key = kmer12(seq1 + q0, i);
            if (key == kEmpty) continue;
            atomicAdd(&n_query, 1u);
            uint32_t sl = slot_of(key);
            for (int probe = 0; probe < kHashSlots; ++probe) {
                const uint32_t k = keys[sl];
                if (k == kEmpty) break;
                if (k == key) {
                    const int64_t d = (int64_t)pos[sl] - i;                        // diagonal j - i
                    int64_t b = ((d + m) * 128) / (m + n + 1);
                    b = b < 0 ? 0 : (b > 127 ? 127 : b);
                    atomicAdd(&hist[b], 1u);
                    break;
                }
                sl = (sl + 1) & (kHashSlots - 1);
            }
        }
        __syncthreads();
        float *f = feat + p * kFeat;
        const float norm = 1.0f / (float)(n_query > 0 ? n_query : 1);
        if (threadIdx.x < 128) f[threadIdx.x] = (float)hist[threadIdx.x] * norm;
        if (threadIdx.x == 0) { f[128] = (float)m / 1024.0f; f[129] = (float)n / 1024.0f; }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// BF16 GEMM on the tensor cores (mma.sync m16n8k16, FP32 accumulate).
// C[M x N] = op(A)[M x K] * op(B)[K x N]; A is MxK row-major (ta = 0) or KxM
// row-major read transposed (ta = 1); B is KxN row-major (tb = 0) or NxK
// row-major read transposed (tb = 1).  M, N multiples of 64, K of 16 (padded).
// Epilogue: +bias, ReLU, store FP32 and/or BF16.
// ---------------------------------------------------------------------------
struct GemmArgs {
    const __nv_bfloat16 *A, *B;
    float *C32;                   // optional fp32 output
    __nv_bfloat16 *C16;           // optional bf16 output
    const float *bias;            // optional, length N
    int M, N, K, lda, ldb, ldc;
    int ta, tb, relu;
    float beta;                   // C32 = acc + beta * C32 (gradient accumulation)
};

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi)
{
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

__global__ void __launch_bounds__(128) k_gemm_bf16(GemmArgs g)
{
    constexpr int BM = 64, BN = 64, BK = 32;
    __shared__ __nv_bfloat16 As[BM][BK + 8];
    __shared__ __nv_bfloat16 Bs[BK][BN + 8];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;     // 2x2 warps of 32x32
    float acc[2][4][4];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b)
#pragma unroll
            for (int c = 0; c < 4; ++c) acc[a][b][c] = 0.f;
    const __nv_bfloat16 zero = __float2bfloat16(0.f);
    for (int k0 = 0; k0 < g.K; k0 += BK) {
        for (int x = tid; x < BM * BK; x += blockDim.x) {
            const int r = x / BK, c = x % BK, gm = m0 + r, gk = k0 + c;
            __nv_bfloat16 v = zero;
            if (gm < g.M && gk < g.K) v = g.ta ? g.A[(size_t)gk * g.lda + gm] : g.A[(size_t)gm * g.lda + gk];
            As[r][c] = v;
        }
        for (int x = tid; x < BK * BN; x += blockDim.x) {
            const int r = x / BN, c = x % BN, gk = k0 + r, gn = n0 + c;
            __nv_bfloat16 v = zero;
            if (gk < g.K && gn < g.N) v = g.tb ? g.B[(size_t)gn * g.ldb + gk] : g.B[(size_t)gk * g.ldb + gn];
            Bs[r][c] = v;
        }
        __syncthreads();
        const int gid = lane >> 2, tig = lane & 3;
#pragma unroll
        for (int kk = 0; kk < BK; kk += 16) {
            uint32_t af[2][4], bf[4][2];
#pragma unroll
            for (int a = 0; a < 2; ++a) {
                const int r = wm + a * 16 + gid, c = kk + tig * 2;
                af[a][0] = pack2(As[r][c], As[r][c + 1]);
                af[a][1] = pack2(As[r + 8][c], As[r + 8][c + 1]);
                af[a][2] = pack2(As[r][c + 8], As[r][c + 9]);
                af[a][3] = pack2(As[r + 8][c + 8], As[r + 8][c + 9]);
            }
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const int c = wn + b * 8 + gid, r = kk + tig * 2;
                bf[b][0] = pack2(Bs[r][c], Bs[r + 1][c]);
                bf[b][1] = pack2(Bs[r + 8][c], Bs[r + 9][c]);
            }
#pragma unroll
            for (int a = 0; a < 2; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b)
                    asm volatile(
                        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                        "{%0,%1,%2,%3};"
                        : "+f"(acc[a][b][0]), "+f"(acc[a][b][1]), "+f"(acc[a][b][2]), "+f"(acc[a][b][3])
                        : "r"(af[a][0]), "r"(af[a][1]), "r"(af[a][2]), "r"(af[a][3]), "r"(bf[b][0]), "r"(bf[b][1]));
        }
        __syncthreads();
    }
    const int gid = lane >> 2, tig = lane & 3;
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b)
#pragma unroll
            for (int h = 0; h < 2; ++h)
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    const int r = m0 + wm + a * 16 + gid + h * 8, c = n0 + wn + b * 8 + tig * 2 + e;
                    if (r >= g.M || c >= g.N) continue;
                    float v = acc[a][b][h * 2 + e];
                    if (g.bias) v += g.bias[c];
                    if (g.relu) v = v > 0.f ? v : 0.f;
                    const size_t idx = (size_t)r * g.ldc + c;
                    if (g.C32) g.C32[idx] = v + (g.beta != 0.f ? g.beta * g.C32[idx] : 0.f);
                    if (g.C16) g.C16[idx] = __float2bfloat16(v);
                }
}

// Loss and its gradient.  out: B x 16 (first 9 used), target: B x 9, mask: B (1 = labelled).
// loss_sum += sum of squared errors; dout (bf16, B x 16) = 2 (out - target) / (B * 9).
__global__ void k_mse(const float *__restrict__ out, const float *__restrict__ target, const float *__restrict__ mask,
                      int B, __nv_bfloat16 *__restrict__ dout, float *__restrict__ loss_sum)
{
    __shared__ float sh[256];
    float acc = 0.f;
    const float scale = 2.0f / ((float)B * kOut);
    for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < B * kOutPad; x += gridDim.x * blockDim.x) {
        const int r = x / kOutPad, c = x % kOutPad;
        float d = 0.f;
        if (c < kOut && mask[r] != 0.f) {
            d = out[(size_t)r * kOutPad + c] - target[(size_t)r * kOut + c];
            acc += d * d;
        }
        dout[x] = __float2bfloat16(d * scale);
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss_sum, sh[0]);
}

// dH (bf16, in place) *= (H > 0): the ReLU derivative of a hidden layer.
__global__ void k_relu_grad(__nv_bfloat16 *__restrict__ dh, const __nv_bfloat16 *__restrict__ h, int n)
{
    for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < n; x += gridDim.x * blockDim.x)
        if (!(__bfloat162float(h[x]) > 0.f)) dh[x] = __float2bfloat16(0.f);
}

// Column sums (bias gradient): db[c] = sum_r d[r, c] over a B x N bf16 matrix.
__global__ void k_colsum(const __nv_bfloat16 *__restrict__ d, int B, int N, float *__restrict__ db)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    float s = 0.f;
    for (int r = 0; r < B; ++r) s += __bfloat162float(d[(size_t)r * N + c]);
    db[c] = s;
}

// Adam on FP32 master weights; refresh the BF16 copy.
__global__ void k_adam(float *__restrict__ w, __nv_bfloat16 *__restrict__ w16, const float *__restrict__ grad,
                       float *__restrict__ m1, float *__restrict__ m2, int n, float lr, float b1, float b2, float eps,
                       float bc1, float bc2, float wd)
{
    for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < n; x += gridDim.x * blockDim.x) {
        const float g = grad[x] + wd * w[x];
        m1[x] = b1 * m1[x] + (1.f - b1) * g;
        m2[x] = b2 * m2[x] + (1.f - b2) * g * g;
        const float mh = m1[x] / bc1, vh = m2[x] / bc2;
        w[x] -= lr * mh / (sqrtf(vh) + eps);
        if (w16) w16[x] = __float2bfloat16(w[x]);
    }
}

// FP32 -> BF16 copy with row padding (features to the padded input).
__global__ void k_to_bf16_pad(const float *__restrict__ src, int rows, int cols, int ld_dst,
                              __nv_bfloat16 *__restrict__ dst)
{
    for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < rows * ld_dst; x += gridDim.x * blockDim.x) {
        const int r = x / ld_dst, c = x % ld_dst;
        dst[x] = __float2bfloat16(c < cols ? src[(size_t)r * cols + c] : 0.f);
    }
}

}  // namespace pa

using namespace pa;

static int blocks_for(long long n, int per) { return (int)((n + per - 1) / per < 4096 ? (n + per - 1) / per : 4096); }

extern "C" {

pa_status pa_band_features_device(const uint8_t *d_seq1, const uint64_t *d_off1, const uint8_t *d_seq2,
                                  const uint64_t *d_off2, uint64_t n_pairs, float *d_features, void *stream)
{
    if (n_pairs == 0) return PA_OK;
    if (!d_seq1 || !d_off1 || !d_seq2 || !d_off2 || !d_features) return PA_ERR_INVALID_ARGUMENT;
    const int grid = (int)(n_pairs < 65535 ? n_pairs : 65535);
    k_kmer_hist<<<grid, 256, 0, (cudaStream_t)stream>>>(d_seq1, d_off1, d_seq2, d_off2, n_pairs, d_features);
    return cudaGetLastError() == cudaSuccess ? PA_OK : PA_ERR_CUDA;
}

// One GEMM (see GemmArgs); device pointers.
pa_status pa_mlp_gemm(const void *A, const void *B, float *C32, void *C16, const float *bias, int M, int N, int K,
                      int lda, int ldb, int ldc, int ta, int tb, int relu, float beta, void *stream)
{
    if (!A || !B || (!C32 && !C16) || M <= 0 || N <= 0 || K <= 0) return PA_ERR_INVALID_ARGUMENT;
    GemmArgs g{(const __nv_bfloat16 *)A, (const __nv_bfloat16 *)B, C32, (__nv_bfloat16 *)C16, bias, M, N, K,
               lda, ldb, ldc, ta, tb, relu, beta};
    dim3 grid((N + 63) / 64, (M + 63) / 64);
    k_gemm_bf16<<<grid, 128, 0, (cudaStream_t)stream>>>(g);
    return cudaGetLastError() == cudaSuccess ? PA_OK : PA_ERR_CUDA;
}

pa_status pa_mlp_mse(const float *out, const float *target, const float *mask, int B, void *dout, float *loss_sum,
                     void *stream)
{
    k_mse<<<blocks_for((long long)B * kOutPad, 256), 256, 0, (cudaStream_t)stream>>>(
        out, target, mask, B, (__nv_bfloat16 *)dout, loss_sum);
    return cudaGetLastError() == cudaSuccess ? PA_OK : PA_ERR_CUDA;
}

pa_status pa_mlp_relu_grad(void *dh, const void *h, int n, void *stream)
{
    k_relu_grad<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>((__nv_bfloat16 *)dh, (const __nv_bfloat16 *)h, n);
    return cudaGetLastError() == cudaSuccess ? PA_OK : PA_ERR_CUDA;
}

pa_status pa_mlp_colsum(const void *d, int B, int N, float *db, void *stream)
{
    k_colsum<<<(N + 127) / 128, 128, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)d, B, N, db);
    return cudaGetLastError() == cudaSuccess ? PA_OK : PA_ERR_CUDA;
}

pa_status pa_mlp_adam(float *w, void *w16, const float *grad, float *m1, float *m2, int n, float lr, float b1, float b2,
                      float eps, int step, float weight_decay, void *stream)
{
    const float bc1 = 1.f - powf(b1, (float)step), bc2 = 1.f - powf(b2, (float)step);
    k_adam<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(w, (__nv_bfloat16 *)w16, grad, m1, m2, n, lr, b1, b2,
                                                                   eps, bc1, bc2, weight_decay);
    return cudaGetLastError() == cudaSuccess ? PA_OK : PA_ERR_CUDA;
}

pa_status pa_mlp_to_bf16(const float *src, int rows, int cols, int ld_dst, void *dst, void *stream)
{
    k_to_bf16_pad<<<blocks_for((long long)rows * ld_dst, 256), 256, 0, (cudaStream_t)stream>>>(
        src, rows, cols, ld_dst, (__nv_bfloat16 *)dst);
    return cudaGetLastError() == cudaSuccess ? PA_OK : PA_ERR_CUDA;
}

}  // extern "C"
