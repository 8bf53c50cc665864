// pa_static.cu -- pa_align_batch_device_static: the affine-gap DP with no allocation.
//
// Some callers cannot allocate device memory at the moment they align: a host
// runtime that owns every cudaMalloc (an arena or pool allocator that must not
// be bypassed), code running while a CUDA graph is being captured (where
// cudaMalloc is not allowed), or a real-time path that must never stall on an
// allocation.  This entry point serves them.  It takes the caller's device
// inputs and output and creates no context, stream or buffer: the only scratch
// the DP needs, the pass-boundary row of long pairs, lives in the file-scope
// array below.  That array is part of this module's device image, so every GPU
// that loads the library holds its 32 MiB until the process exits.
//
// The kernel is a variant of dp_kernel<L32, byte-compare>: pairs are taken in
// input order (no bucketing, so no keys, histogram or score tables are needed),
// one pair per group of 8 lanes, s32 arithmetic, raw byte equality.
#include <cstring>
#include <mutex>

#include "pa_dp.cuh"

namespace {

// Capacity of the static pass-boundary scratch, in cells (8 bytes each): the call
// needs seq1_bytes + n_pairs cells.
constexpr uint64_t kStaticCells = 4u << 20;                // 4,194,304 cells = 32 MiB
constexpr int kStaticG = 8;
constexpr int kStaticR = 16;

static __device__ __align__(256) pa::Cell g_static_boundary[kStaticCells];
static __device__ __align__(256) uint32_t g_static_counters[64];

// Per device: the device addresses of the two arrays (see static_slot).
struct StaticSlot {
    bool ready = false;
    pa::Cell *boundary = nullptr;
    uint32_t *counters = nullptr;
};
constexpr int kMaxDevices = 64;
StaticSlot g_slots[kMaxDevices];
std::mutex g_slots_mutex;

// Result of a pair with an empty sequence: the candidate rules of the DP applied
// to the border cells alone (local: INT32_MIN at (0,0), tracker_local_scalar.hpp:38).
__device__ void empty_pair_result(const pa::DpParams &P, int32_t m, int32_t n, pa_result &r)
{
    r.width = 32;
    r.flags = PA_RESULT_TRIVIAL;
    r.band_rounds = 0;
    if (P.local) { r.score = INT32_MIN; r.end1 = 0; r.end2 = 0; return; }
    int32_t s, i, j;
    if (m == 0) { s = pa::border(P, P.first_row_free, n); i = 0; j = n; }
    else { s = pa::border(P, P.first_column_free, m); i = m; j = 0; }
    // with a free trailing row (m == 0) or column (n == 0) the corner H(0,0) = 0 is a candidate
    if ((m == 0 && P.last_row_free) || (n == 0 && P.last_column_free))
        if (0 > s || (0 == s && (0 < i || (0 == i && 0 < j)))) { s = 0; i = 0; j = 0; }
    r.score = s; r.end1 = i; r.end2 = j;
}

// A pair whose offsets decrease or run past the byte buffers is not aligned: its scratch
// row (at off1[k] + k) could leave the static array.  It gets INT32_MIN and PA_RESULT_ERROR.
template <int MODE>
__global__ void __launch_bounds__(pa::kBlock, 2) dp_kernel_static(pa::DpLaunch L, pa::DpParams P, uint32_t count,
                                                                  uint64_t seq1_bytes, uint64_t seq2_bytes)
{
    using namespace pa;
    using V = L32;
    constexpr int R = kStaticR;
    __shared__ uint4 snap_store[MODE == M_LOCAL ? (R / 4) * kBlock : 1];
    const int lane = threadIdx.x & 31;
    const int G = L.G;
    const int t = lane & (G - 1);
    const int g = lane / G;
    const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (g * G));
    const uint32_t ppw = (uint32_t)(32 / G);
    const uint32_t n_units = (count + ppw - 1) / ppw;

    for (;;) {
        uint32_t u = 0;
        if (lane == 0) u = atomicAdd(L.unit_counter, 1u);
        u = __shfl_sync(0xffffffffu, u, 0);
        if (u >= n_units) break;
        const uint32_t first = u * ppw + (uint32_t)g;
        if (first >= count) continue;

        {
            const uint64_t q0 = L.off1[first], q1 = L.off1[first + 1], t0 = L.off2[first], t1 = L.off2[first + 1];
            if (q0 > q1 || q1 > seq1_bytes || t0 > t1 || t1 > seq2_bytes) {
                if (t == 0) {
                    pa_result r;
                    r.score = INT32_MIN;
                    r.end1 = r.end2 = 0;
                    r.width = 32;
                    r.flags = PA_RESULT_ERROR;
                    r.band_rounds = 0;
                    L.out[first] = r;
                }
                __syncwarp(gmask);
                continue;
            }
        }
        GroupWork w;
        w.id[0] = w.id[1] = first;
        w.has_b = false;
        w.wait_failed = false;
        w.qoff[0] = w.qoff[1] = L.off1[first];
        w.m[0] = w.m[1] = (int32_t)(L.off1[first + 1] - w.qoff[0]);
        w.toff[0] = w.toff[1] = L.off2[first];
        w.n[0] = w.n[1] = (int32_t)(L.off2[first + 1] - w.toff[0]);
        w.qt[0] = w.qt[1] = nullptr;
        if (w.m[0] == 0 || w.n[0] == 0) {           // an empty sequence: no DP
            if (t == 0) {
                pa_result r;
                empty_pair_result(P, w.m[0], w.n[0], r);
                L.out[first] = r;
            }
            __syncwarp(gmask);
            continue;
        }
        {
            const int64_t a = P.match < 0 ? -(int64_t)P.match : P.match;
            const int64_t b = P.mismatch < 0 ? -(int64_t)P.mismatch : P.mismatch;
            const int64_t o = -(int64_t)P.gap_open, e = -(int64_t)P.gap_ext;
            const int64_t mn = w.m[0] < w.n[0] ? w.m[0] : w.n[0];
            if ((a + b) * mn + (o + e) * ((int64_t)w.m[0] + w.n[0] + 2) + 2 * o >= (1ll << 30)) {
                if (t == 0) {
                    pa_result r;
                    r.score = INT32_MIN;
                    r.end1 = r.end2 = 0;
                    r.width = 32;
                    r.flags = PA_RESULT_OVERFLOW;
                    r.band_rounds = 0;
                    L.out[first] = r;
                }
                __syncwarp(gmask);
                continue;
            }
        }
        for (int l = 0; l < 2; ++l) { w.cs[l] = MODE == M_LOCAL ? 0 : INT32_MIN; w.ci[l] = 0; w.cj[l] = 0; }
        w.ms = w.m[0];
        w.nh = w.n[0];
        w.rows_full = G * R;
        w.passes = (w.nh + w.rows_full - 1) / w.rows_full;
        w.buf = L.boundary + (L.off1[first] + first);
        w.bin = w.bout = w.buf;
        w.seen = INT32_MIN;
        w.Kt = 0;
        w.clampt = MODE == M_LOCAL ? 0 : INT32_MIN;
        w.floor_true = INT32_MIN;
        w.K = 0;
        w.CLAMP = (uint32_t)w.clampt;

        for (int p = 0; p < w.passes; ++p) {
            const int32_t rem = w.nh - p * w.rows_full;
            const int32_t rpt = rem >= w.rows_full ? R : ((rem + G * kChunk - 1) / (G * kChunk)) * kChunk;
            switch (rpt / kChunk) {
            case 1: run_pass<V, R, 4, MODE, true, 0>(L, P, w, p, t, G, gmask, snap_store); break;
            case 2: run_pass<V, R, 8, MODE, true, 0>(L, P, w, p, t, G, gmask, snap_store); break;
            case 3: run_pass<V, R, 12, MODE, true, 0>(L, P, w, p, t, G, gmask, snap_store); break;
            default: run_pass<V, R, R, MODE, true, 0>(L, P, w, p, t, G, gmask, snap_store); break;
            }
            __syncwarp(gmask);
        }
        for (int off = G >> 1; off >= 1; off >>= 1) {
            const int32_t os = __shfl_xor_sync(gmask, w.cs[0], off, G);
            const int32_t oi = __shfl_xor_sync(gmask, w.ci[0], off, G);
            const int32_t oj = __shfl_xor_sync(gmask, w.cj[0], off, G);
            if (better(os, oi, oj, w.cs[0], w.ci[0], w.cj[0])) { w.cs[0] = os; w.ci[0] = oi; w.cj[0] = oj; }
        }
        if (t == 0) {
            if (MODE == M_GLOBAL_FREE) {
                if (P.last_column_free) {
                    const int32_t x = border(P, P.first_row_free, w.n[0]);
                    if (better(x, 0, w.n[0], w.cs[0], w.ci[0], w.cj[0])) { w.cs[0] = x; w.ci[0] = 0; w.cj[0] = w.n[0]; }
                }
                if (P.last_row_free) {
                    const int32_t x = border(P, P.first_column_free, w.m[0]);
                    if (better(x, w.m[0], 0, w.cs[0], w.ci[0], w.cj[0])) { w.cs[0] = x; w.ci[0] = w.m[0]; w.cj[0] = 0; }
                }
            }
            pa_result r;
            r.score = w.cs[0];
            r.end1 = w.ci[0];
            r.end2 = w.cj[0];
            r.width = 32;
            r.flags = 0;
            r.band_rounds = 0;
            if (MODE == M_LOCAL && w.cs[0] <= 0) { r.end1 = 0; r.end2 = 0; }
            L.out[first] = r;
        }
        __syncwarp(gmask);
    }
}

// Device addresses of the static arrays on the current device.  Outside a stream capture
// they are looked up again on every call (cudaGetSymbolAddress is a host-side lookup), so a
// context that was reset and created again, which reloads this module at new addresses, is
// followed; while `stream` is being captured the addresses of the last call on this device
// are used, so the first call on a device must come before any capture.
pa_status static_slot(cudaStream_t stream, StaticSlot **out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return PA_ERR_NO_DEVICE; }
    if (dev < 0 || dev >= kMaxDevices) return PA_ERR_UNSUPPORTED;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(stream, &cap) != cudaSuccess) { cudaGetLastError(); return PA_ERR_CUDA; }
    std::lock_guard<std::mutex> lock(g_slots_mutex);
    StaticSlot &s = g_slots[dev];
    if (cap != cudaStreamCaptureStatusNone && !s.ready) return PA_ERR_UNSUPPORTED;
    if (cap == cudaStreamCaptureStatusNone) {
        void *b = nullptr, *c = nullptr;
        if (cudaGetSymbolAddress(&b, g_static_boundary) != cudaSuccess ||
            cudaGetSymbolAddress(&c, g_static_counters) != cudaSuccess) {
            cudaGetLastError();
            return PA_ERR_CUDA;
        }
        s.boundary = (pa::Cell *)b;
        s.counters = (uint32_t *)c;
        s.ready = true;
    }
    *out = &s;
    return PA_OK;
}

}  // namespace

extern "C" pa_status pa_align_batch_device_static(const pa_config *config, const uint8_t *d_seq1,
                                                  const uint64_t *d_off1, uint64_t seq1_bytes,
                                                  const uint8_t *d_seq2, const uint64_t *d_off2,
                                                  uint64_t seq2_bytes, uint64_t n_pairs, pa_result *d_out,
                                                  void *stream)
{
    using namespace pa;
    if (!config) return PA_ERR_INVALID_ARGUMENT;
    if (config->method != PA_METHOD_GLOBAL && config->method != PA_METHOD_LOCAL) return PA_ERR_INVALID_ARGUMENT;
    if (config->gap_extension > 0 || (int64_t)config->gap_open + config->gap_extension > 0) return PA_ERR_UNSUPPORTED;
    if (n_pairs == 0) return PA_OK;
    if (!d_seq1 || !d_off1 || !d_seq2 || !d_off2 || !d_out) return PA_ERR_INVALID_ARGUMENT;
    if (n_pairs >= (1ull << 31) || seq1_bytes + n_pairs > kStaticCells) return PA_ERR_TOO_LARGE;
    StaticSlot *slot = nullptr;
    const pa_status s = static_slot((cudaStream_t)stream, &slot);
    if (s != PA_OK) return s;

    const bool local = config->method == PA_METHOD_LOCAL;
    DpParams P;
    P.match = config->match;
    P.mismatch = config->mismatch;
    P.gap_open = config->gap_open;
    P.gap_ext = config->gap_extension;
    P.local = local;
    P.first_column_free = local || config->first_column_free;
    P.first_row_free = local || config->first_row_free;
    P.last_column_free = !local && config->last_column_free;
    P.last_row_free = !local && config->last_row_free;
    P.smax = config->match > config->mismatch ? config->match : config->mismatch;
    if (P.smax < 0) P.smax = 0;
    P.spad = config->match < config->mismatch ? config->match : config->mismatch;
    if (P.spad > 0) P.spad = 0;
    P.floor16 = 0;
    P.shift = 0;                 // s32 lanes hold H itself

    DpLaunch L;
    std::memset(&L, 0, sizeof(L));
    L.seq1 = d_seq1; L.off1 = d_off1; L.seq2 = d_seq2; L.off2 = d_off2;
    L.qtab = nullptr; L.order = nullptr; L.begin_ptr = nullptr; L.count_ptr = nullptr;
    L.unit_counter = slot->counters;
    L.out = d_out;
    L.boundary = slot->boundary;
    L.rerun_list = nullptr; L.rerun_count = nullptr; L.dp_cells = nullptr;
    L.G = kStaticG;
    L.rerun = 0;

    cudaStream_t st = (cudaStream_t)stream;
    // the queue head must start at zero; the array keeps the previous call's contents
    if (cudaMemsetAsync(slot->counters, 0, sizeof(uint32_t) * 64, st) != cudaSuccess) {
        cudaGetLastError();
        return PA_ERR_CUDA;
    }
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = 2 * sms;
    const uint32_t count = (uint32_t)n_pairs;
    const int mode = local ? M_LOCAL : ((P.last_column_free || P.last_row_free) ? M_GLOBAL_FREE : M_GLOBAL);
    if (mode == M_LOCAL) dp_kernel_static<M_LOCAL><<<grid, kBlock, 0, st>>>(L, P, count, seq1_bytes, seq2_bytes);
    else if (mode == M_GLOBAL) dp_kernel_static<M_GLOBAL><<<grid, kBlock, 0, st>>>(L, P, count, seq1_bytes, seq2_bytes);
    else dp_kernel_static<M_GLOBAL_FREE><<<grid, kBlock, 0, st>>>(L, P, count, seq1_bytes, seq2_bytes);
    if (cudaGetLastError() != cudaSuccess) return PA_ERR_CUDA;
    return PA_OK;
}
