// pa_capi.cu -- C ABI, context and launch sequence of the GB300 affine-gap DP.
//
// One call = one device pipeline on the context's stream, with no host
// synchronisation inside it (so it can be captured once into a CUDA graph and
// replayed):
//   1. k_classify    class, bucket key, score tables and empty-pair results
//   2. k_scan_*      exclusive scan of the bucket histogram (2^18 buckets)
//   3. k_scatter     bucket sort of the pair ids (order inside a bucket is free)
//   4. dp_kernel     persistent DP kernels per class (s16x2, s32, byte-compare),
//                    each pulling warp units from its own device queue, longest first
//   5. dp_kernel     s32 recomputation of s16 global results that failed their check
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "pa_common.cuh"
#include "pa_dp.cuh"
#include "pa_prep.cuh"
#include "pa_launch.h"

using namespace pa;

namespace {


constexpr int kR = 16;             // rows per thread per lane
constexpr int kDefaultG = 8;       // threads per group

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
};

struct GraphKey {
    const void *ptrs[6];
    uint64_t n_pairs, b1, b2;
    pa_config cfg;
    bool operator<(const GraphKey &o) const { return std::memcmp(this, &o, sizeof(GraphKey)) < 0; }
};

}  // namespace

struct pa_ctx {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr, ev3 = nullptr;
    cudaEvent_t ev_dp0 = nullptr, ev_dp1 = nullptr;   // bracket the DP kernels of the last call
    pa_options opt{};
    std::string err;
    // device work buffers (grow only)
    DevBuf keys, order, hist, starts, cursor, sums, ranges, counts, qtab, boundary, rerun, counters, pstats;
    DevBuf in_seq1, in_off1, in_seq2, in_off2, in_out;   // staging for the host-buffer entry points
    int G[3] = {kDefaultG, kDefaultG, kDefaultG};
    int variant[3] = {0, 0, 0};
    pa_tuning tuning{};           // per method (0 local, 1 global); applied to G/variant per call
    bool fixed_G = false, fixed_variant = false;
    int grid[3] = {0, 0, 0};
    std::map<GraphKey, cudaGraphExec_t> graphs;
    uint64_t last_launches = 0;
};

namespace {

pa_status fail(pa_ctx *c, pa_status s, const std::string &msg)
{
    if (c) c->err = msg;
    return s;
}

#define PA_CUDA(ctx, call)                                                                  \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) return fail((ctx), PA_ERR_CUDA, std::string(#call ": ") +    \
                                           cudaGetErrorString(e_));                         \
    } while (0)

pa_status ensure(pa_ctx *c, DevBuf &b, size_t bytes)
{
    if (bytes == 0) bytes = 16;
    if (b.cap >= bytes) return PA_OK;
    const size_t want = std::max(bytes, (size_t)(b.cap * 3 / 2));
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.cap = 0;
    cudaError_t e = cudaMalloc(&b.p, want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(c, PA_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    b.cap = want;
    // a grown buffer invalidates captured graphs
    for (auto &kv : c->graphs) cudaGraphExecDestroy(kv.second);
    c->graphs.clear();
    return PA_OK;
}

pa_status check_config(pa_ctx *c, const pa_config *cfg, DpParams &P, ClassCfg &C)
{
    if (!cfg) return fail(c, PA_ERR_INVALID_ARGUMENT, "config is null");
    if (cfg->method != PA_METHOD_GLOBAL && cfg->method != PA_METHOD_LOCAL)
        return fail(c, PA_ERR_INVALID_ARGUMENT, "method must be PA_METHOD_GLOBAL or PA_METHOD_LOCAL");
    if (cfg->gap_extension > 0 || (int64_t)cfg->gap_open + cfg->gap_extension > 0)
        return fail(c, PA_ERR_UNSUPPORTED, "positive gap scores are not supported");
    if (cfg->width_hint != 0 && cfg->width_hint != 16 && cfg->width_hint != 32)
        return fail(c, PA_ERR_INVALID_ARGUMENT, "width_hint must be 0, 16 or 32");
    if (cfg->band_mode != 0 && cfg->band_mode != 1)
        return fail(c, PA_ERR_INVALID_ARGUMENT, "band_mode must be 0 or 1");
    const bool local = cfg->method == PA_METHOD_LOCAL;
    std::memset(&P, 0, sizeof(P));
    P.match = cfg->match;
    P.mismatch = cfg->mismatch;
    P.gap_open = cfg->gap_open;
    P.gap_ext = cfg->gap_extension;
    P.local = local;
    P.first_column_free = local || cfg->first_column_free;   // method_local.hpp:41-49
    P.first_row_free = local || cfg->first_row_free;
    P.last_column_free = !local && cfg->last_column_free;
    P.last_row_free = !local && cfg->last_row_free;
    P.smax = std::max(0, std::max(cfg->match, cfg->mismatch));
    P.spad = std::min(0, std::min(cfg->match, cfg->mismatch));
    P.floor16 = -32768 + 1280;
    std::memset(&C, 0, sizeof(C));
    C.fast_scores = cfg->match >= -127 && cfg->match <= 127 && cfg->mismatch >= -127 && cfg->mismatch <= 0;
    C.s16_params = (int64_t)cfg->gap_open + cfg->gap_extension >= -1000 && cfg->gap_extension >= -1000;
    C.force32 = cfg->width_hint == 32;
    C.local = local;
    for (int k = 0; k < 3; ++k) {
        C.gcnt[k] = c->G[k];
        C.rpt[k] = kR;
        C.rows[k] = c->G[k] * kR;
    }
    return PA_OK;
}

}  // namespace

namespace pa {
int dp_occupancy_v0(bool lanes16, bool gen, int mode);
int dp_occupancy_v1(bool lanes16, bool gen, int mode);
int dp_occupancy_v2(bool lanes16, bool gen, int mode);
int dp_occupancy_v3(bool lanes16, bool gen, int mode);
int dp_occupancy_v4(bool lanes16, bool gen, int mode);
void dp_launch_v0(bool, bool, int, int, cudaStream_t, const DpLaunch &, const DpParams &);
void dp_launch_v1(bool, bool, int, int, cudaStream_t, const DpLaunch &, const DpParams &);
void dp_launch_v2(bool, bool, int, int, cudaStream_t, const DpLaunch &, const DpParams &);
void dp_launch_v3(bool, bool, int, int, cudaStream_t, const DpLaunch &, const DpParams &);
void dp_launch_v4(bool, bool, int, int, cudaStream_t, const DpLaunch &, const DpParams &);

int dp_occupancy(int variant, bool lanes16, bool gen, int mode)
{
    if (variant == 1) return dp_occupancy_v1(lanes16, gen, mode);
    if (variant == 2) return dp_occupancy_v2(lanes16, gen, mode);
    if (variant == 3) return dp_occupancy_v3(lanes16, gen, mode);
    if (variant == 4) return dp_occupancy_v4(lanes16, gen, mode);
    return dp_occupancy_v0(lanes16, gen, mode);
}

void dp_launch(int variant, bool lanes16, bool gen, int mode, int grid, cudaStream_t st, const DpLaunch &L,
               const DpParams &P)
{
    if (variant == 1) dp_launch_v1(lanes16, gen, mode, grid, st, L, P);
    else if (variant == 2) dp_launch_v2(lanes16, gen, mode, grid, st, L, P);
    else if (variant == 3) dp_launch_v3(lanes16, gen, mode, grid, st, L, P);
    else if (variant == 4) dp_launch_v4(lanes16, gen, mode, grid, st, L, P);
    else dp_launch_v0(lanes16, gen, mode, grid, st, L, P);
}
}  // namespace pa

namespace {

// Resident blocks per SM of every DP kernel, queried once outside any stream capture.
void warm_occupancy()
{
    for (int v = 0; v < 5; ++v)
        for (int mode = 0; mode < 3; ++mode) {
            dp_occupancy(v, true, false, mode);
            dp_occupancy(v, false, false, mode);
            dp_occupancy(v, false, true, mode);
        }
}

void launch_class(pa_ctx *c, int slot, int mode, bool lanes16, bool gen, const DpLaunch &L, const DpParams &P)
{
    const int v = c->variant[slot];
    int per_sm = dp_occupancy(v, lanes16, gen, mode);
    if (c->opt.blocks_per_sm > 0) per_sm = std::min(per_sm, (int)c->opt.blocks_per_sm);
    c->grid[slot] = per_sm * c->sm_count;
    dp_launch(v, lanes16, gen, mode, c->grid[slot], c->stream, L, P);
    c->last_launches++;
}

// Everything between inputs-on-device and results-on-device; no host sync.
pa_status enqueue(pa_ctx *c, const pa_config *cfg, const DpParams &P, const ClassCfg &C, const uint8_t *s1,
                  const uint64_t *o1, uint64_t b1, const uint8_t *s2, const uint64_t *o2, pa_result *out,
                  uint64_t n_pairs)
{
    cudaStream_t st = c->stream;
    uint32_t *counters = (uint32_t *)c->counters.p;   // [0..3] unit queues, [4] rerun count, [5] zero
    PA_CUDA(c, cudaMemsetAsync(c->hist.p, 0, sizeof(uint32_t) * kBuckets, st));
    PA_CUDA(c, cudaMemsetAsync(c->counters.p, 0, 64, st));
    PA_CUDA(c, cudaMemsetAsync(c->pstats.p, 0, sizeof(PrepStats), st));
    int cls_blocks = (int)std::min<uint64_t>((n_pairs * 32 + kBlock - 1) / kBlock, (uint64_t)c->sm_count * 64);
    if (cls_blocks < 1) cls_blocks = 1;
    k_classify<<<cls_blocks, kBlock, 0, st>>>(s1, o1, s2, o2, n_pairs, P, C, (uint32_t *)c->keys.p,
                                              (uint32_t *)c->hist.p, (uint32_t *)c->qtab.p, out,
                                              (PrepStats *)c->pstats.p);
    k_scan_blocks<<<kBuckets / 1024, 1024, 0, st>>>((uint32_t *)c->hist.p, (uint32_t *)c->starts.p,
                                                    (uint32_t *)c->sums.p);
    k_scan_sums<<<1, 256, 0, st>>>((uint32_t *)c->sums.p, kBuckets / 1024);
    k_scan_add<<<kBuckets / 1024, 1024, 0, st>>>((uint32_t *)c->starts.p, (uint32_t *)c->cursor.p,
                                                 (uint32_t *)c->sums.p, (uint32_t *)c->ranges.p);
    const int sc_blocks = (int)std::max<uint64_t>(1, (n_pairs + kBlock - 1) / kBlock);
    k_scatter<<<sc_blocks, kBlock, 0, st>>>((uint32_t *)c->keys.p, n_pairs, (uint32_t *)c->cursor.p,
                                            (uint32_t *)c->order.p, (uint32_t *)c->ranges.p,
                                            (uint32_t *)c->counts.p);
    c->last_launches += 6;

    const int mode = P.local ? M_LOCAL : ((P.last_column_free || P.last_row_free) ? M_GLOBAL_FREE : M_GLOBAL);
    DpLaunch L;
    std::memset(&L, 0, sizeof(L));
    L.seq1 = s1; L.off1 = o1; L.seq2 = s2; L.off2 = o2;
    L.qtab = (const uint32_t *)c->qtab.p;
    L.order = (const uint32_t *)c->order.p;
    L.out = out;
    L.boundary = (Cell *)c->boundary.p;
    L.rerun_list = (uint32_t *)c->rerun.p;
    L.rerun_count = counters + 4;
    (void)b1;

    const uint32_t *ranges = (const uint32_t *)c->ranges.p;
    const uint32_t *counts = (const uint32_t *)c->counts.p;
    cudaStreamCaptureStatus capturing = cudaStreamCaptureStatusNone;
    PA_CUDA(c, cudaStreamIsCapturing(st, &capturing));
    // inside a capture the record must become a graph node to fire on every replay
    const unsigned ev_flags = capturing == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : 0u;
    PA_CUDA(c, cudaEventRecordWithFlags(c->ev_dp0, st, ev_flags));
    // s16x2 class
    L.begin_ptr = ranges + K_S16; L.count_ptr = counts + K_S16; L.unit_counter = counters + 0; L.G = c->G[K_S16];
    launch_class(c, K_S16, mode, true, false, L, P);
    // s32 class
    L.begin_ptr = ranges + K_S32; L.count_ptr = counts + K_S32; L.unit_counter = counters + 1; L.G = c->G[K_S32];
    launch_class(c, K_S32, mode, false, false, L, P);
    // byte-compare class
    L.begin_ptr = ranges + K_GEN; L.count_ptr = counts + K_GEN; L.unit_counter = counters + 2; L.G = c->G[K_GEN];
    launch_class(c, K_GEN, mode, false, true, L, P);
    // s16 global results that failed the exactness check, recomputed in s32
    if (mode != M_LOCAL) {
        L.order = (const uint32_t *)c->rerun.p;
        L.begin_ptr = counters + 5;          // always zero
        L.count_ptr = counters + 4;
        L.unit_counter = counters + 3;
        L.rerun = 1;
        L.G = c->G[K_S32];
        launch_class(c, K_S32, mode, false, false, L, P);
    }
    PA_CUDA(c, cudaEventRecordWithFlags(c->ev_dp1, st, ev_flags));
    PA_CUDA(c, cudaGetLastError());
    (void)cfg;
    return PA_OK;
}

pa_status prepare_buffers(pa_ctx *c, uint64_t n_pairs, uint64_t b1)
{
    pa_status s;
    const uint64_t np = std::max<uint64_t>(n_pairs, 1);
    if ((s = ensure(c, c->keys, np * 4))) return s;
    if ((s = ensure(c, c->order, np * 4))) return s;
    if ((s = ensure(c, c->rerun, np * 4))) return s;
    if ((s = ensure(c, c->hist, sizeof(uint32_t) * kBuckets))) return s;
    if ((s = ensure(c, c->starts, sizeof(uint32_t) * kBuckets))) return s;
    if ((s = ensure(c, c->cursor, sizeof(uint32_t) * kBuckets))) return s;
    if ((s = ensure(c, c->sums, sizeof(uint32_t) * 1024))) return s;
    if ((s = ensure(c, c->ranges, 64))) return s;
    if ((s = ensure(c, c->counts, 64))) return s;
    if ((s = ensure(c, c->counters, 64))) return s;
    if ((s = ensure(c, c->pstats, sizeof(PrepStats)))) return s;
    if ((s = ensure(c, c->qtab, (b1 + np) * 4))) return s;
    if ((s = ensure(c, c->boundary, (b1 + np) * sizeof(Cell)))) return s;
    return PA_OK;
}

pa_status run_device(pa_ctx *c, const pa_config *cfg, const uint8_t *s1, const uint64_t *o1, uint64_t b1,
                     const uint8_t *s2, const uint64_t *o2, uint64_t b2, uint64_t n_pairs, pa_result *out,
                     pa_stats *stats, bool sync_for_stats)
{
    if (cfg) {
        const int mi = cfg->method == PA_METHOD_LOCAL ? 0 : 1;
        if (!c->fixed_variant) {
            c->variant[K_S16] = c->tuning.variant_s16[mi];
            c->variant[K_S32] = c->variant[K_GEN] = c->tuning.variant_s32[mi];
        }
        if (!c->fixed_G) {
            c->G[K_S16] = c->tuning.group_threads_s16[mi];
            c->G[K_S32] = c->G[K_GEN] = c->tuning.group_threads_s32[mi];
        }
    }
    DpParams P;
    ClassCfg C;
    pa_status s = check_config(c, cfg, P, C);
    if (s) return s;
    if (n_pairs == 0) {
        if (stats) std::memset(stats, 0, sizeof(*stats));
        return PA_OK;
    }
    if (!s1 || !o1 || !s2 || !o2 || !out) return fail(c, PA_ERR_INVALID_ARGUMENT, "null buffer");
    if (n_pairs >= (1ull << 31)) return fail(c, PA_ERR_TOO_LARGE, "n_pairs must be < 2^31");
    if ((s = prepare_buffers(c, n_pairs, b1))) return s;
    c->last_launches = 0;
    const bool use_graph = c->opt.use_graphs >= 0;
    PA_CUDA(c, cudaEventRecord(c->ev0, c->stream));
    if (use_graph) {
        GraphKey key;
        std::memset(&key, 0, sizeof(key));
        key.ptrs[0] = s1; key.ptrs[1] = o1; key.ptrs[2] = s2; key.ptrs[3] = o2; key.ptrs[4] = out;
        key.ptrs[5] = c->boundary.p;
        key.n_pairs = n_pairs; key.b1 = b1; key.b2 = b2; key.cfg = *cfg;
        auto it = c->graphs.find(key);
        if (it == c->graphs.end()) {
            cudaGraph_t g;
            PA_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            pa_status es = enqueue(c, cfg, P, C, s1, o1, b1, s2, o2, out, n_pairs);
            cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
            if (es) return es;
            if (ce != cudaSuccess) return fail(c, PA_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(ce));
            cudaGraphExec_t ex;
            ce = cudaGraphInstantiate(&ex, g, 0);
            cudaGraphDestroy(g);
            if (ce != cudaSuccess) return fail(c, PA_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(ce));
            it = c->graphs.emplace(key, ex).first;
        } else {
            c->last_launches = 6 + 3 + (P.local ? 0 : 1);
        }
        PA_CUDA(c, cudaGraphLaunch(it->second, c->stream));
    } else {
        if ((s = enqueue(c, cfg, P, C, s1, o1, b1, s2, o2, out, n_pairs))) return s;
    }
    PA_CUDA(c, cudaEventRecord(c->ev1, c->stream));
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->pairs = n_pairs;
        stats->kernel_launches = c->last_launches;
        if (sync_for_stats) {
            PA_CUDA(c, cudaEventSynchronize(c->ev1));
            PrepStats ps;
            uint32_t ctr[8];
            PA_CUDA(c, cudaMemcpy(&ps, c->pstats.p, sizeof(ps), cudaMemcpyDeviceToHost));
            PA_CUDA(c, cudaMemcpy(ctr, c->counters.p, sizeof(ctr), cudaMemcpyDeviceToHost));
            float ms = 0.f;
            cudaEventElapsedTime(&ms, c->ev0, c->ev1);
            stats->device_ms = ms;
            if (cudaEventElapsedTime(&ms, c->ev_dp0, c->ev_dp1) == cudaSuccess) stats->dp_ms = ms;
            cudaGetLastError();
            stats->cells = ps.cells;
            stats->pairs_s16 = ps.n_class[K_S16] - ctr[4];
            stats->pairs_s32 = ps.n_class[K_S32] + ctr[4];
            stats->pairs_general = ps.n_class[K_GEN];
            stats->pairs_trivial = ps.n_class[K_NONE];
            stats->pairs_rerun = ctr[4];
            if (ps.overflow) return fail(c, PA_ERR_OVERFLOW, "scores of some pairs could exceed int32");
        }
    }
    PA_CUDA(c, cudaGetLastError());
    return PA_OK;
}

// ---------------------------------------------------------------------------
// roofline microkernel: the cell-update instruction mix of dp_kernel on
// registers only (no memory, no shuffles), timed over the whole chip.
// ---------------------------------------------------------------------------
template <class V>
__global__ void __launch_bounds__(256) k_roofline(int steps, uint32_t seed, uint32_t *sink)
{
    constexpr int R = 16;
    uint32_t H[R], Fr[R], Sel[R];
    const uint32_t GOEA = V::cabs(-7), EXTA = V::cabs(-1), CLAMP = V::splat(2048);
#pragma unroll
    for (int k = 0; k < R; ++k) {
        H[k] = V::splat(2048 + (int)((seed + k * 7 + threadIdx.x) & 15));
        Fr[k] = V::splat(2040);
        Sel[k] = V::selector((k + threadIdx.x) & 3, (k * 3 + threadIdx.x) & 3);
    }
    uint32_t ta = 0x01fcfcfcu ^ (seed & 0x03000000u), tb = 0xfc01fcfcu, up = V::splat(2041), diag0 = V::splat(2048);
    for (int s = 0; s < steps; ++s) {
        uint32_t diag = diag0, Ed = up;
#pragma unroll
        for (int k = 0; k < R; ++k) {
            const uint32_t sc = prmt(ta, tb, Sel[k]);
            const uint32_t tt = V::addmax(diag, sc, Fr[k]);
            const uint32_t h = V::hmax(tt, Ed, CLAMP);
            diag = H[k];
            H[k] = h;
            const uint32_t hoe = V::subc(h, GOEA);
            Fr[k] = V::max2(V::subc(Fr[k], EXTA), hoe);
            Ed = V::max2(V::subc(Ed, EXTA), hoe);
        }
        diag0 = H[R - 1];
        up = Ed;
        ta = (ta << 8) | (ta >> 24);
        tb = (tb >> 8) | (tb << 24);
    }
    uint32_t acc = up;
#pragma unroll
    for (int k = 0; k < R; ++k) acc ^= H[k] ^ Fr[k];
    if (acc == 0x12345678u) sink[blockIdx.x] = acc;
}

}  // namespace

extern "C" {

int pa_abi_version(void) { return PA_ABI_VERSION; }

const char *pa_status_string(pa_status s)
{
    switch (s) {
    case PA_OK: return "ok";
    case PA_ERR_INVALID_ARGUMENT: return "invalid argument";
    case PA_ERR_CUDA: return "CUDA error";
    case PA_ERR_OUT_OF_MEMORY: return "out of device memory";
    case PA_ERR_OVERFLOW: return "score range exceeds int32";
    case PA_ERR_UNSUPPORTED: return "unsupported configuration";
    case PA_ERR_TIMEOUT: return "device wait timed out";
    case PA_ERR_NO_DEVICE: return "no CUDA device";
    case PA_ERR_TOO_LARGE: return "input exceeds a fixed capacity";
    }
    return "unknown status";
}

const char *pa_last_error(const pa_ctx *ctx) { return ctx ? ctx->err.c_str() : ""; }

pa_status pa_create(pa_ctx **out, int device_ordinal, const pa_options *options)
{
    if (!out) return PA_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return PA_ERR_NO_DEVICE;
    }
    if (device_ordinal < 0 || device_ordinal >= n) return PA_ERR_INVALID_ARGUMENT;
    pa_ctx *c = new pa_ctx();
    c->device = device_ordinal;
    if (options) c->opt = *options;
    if (cudaSetDevice(device_ordinal) != cudaSuccess ||
        cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device_ordinal) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess ||
        cudaEventCreate(&c->ev2) != cudaSuccess || cudaEventCreate(&c->ev3) != cudaSuccess ||
        cudaEventCreate(&c->ev_dp0) != cudaSuccess || cudaEventCreate(&c->ev_dp1) != cudaSuccess) {
        cudaGetLastError();
        delete c;
        return PA_ERR_CUDA;
    }
    // defaults measured on GB300 (262,144 pairs of 64..512 bp): local s16x2 is fastest with
    // variant 3, global with variant 4; 8 lanes per group
    c->tuning = pa_tuning{{3, 4}, {0, 4}, {8, 8}, {8, 8}, {0.0, 0.0}};
    if (c->opt.group_threads) {
        int g = c->opt.group_threads;
        if (g < 1 || g > 32 || (g & (g - 1))) { pa_destroy(c); return PA_ERR_INVALID_ARGUMENT; }
        for (int k = 0; k < 3; ++k) c->G[k] = g;
        c->fixed_G = true;
    }
    if (c->opt.rows_per_thread && c->opt.rows_per_thread != kR) { pa_destroy(c); return PA_ERR_UNSUPPORTED; }
    if (c->opt.kernel_variant >= 0 && c->opt.kernel_variant <= 4) {
        for (int k = 0; k < 3; ++k) c->variant[k] = c->opt.kernel_variant;
        c->fixed_variant = true;
    }
    else if (c->opt.kernel_variant != -1) { pa_destroy(c); return PA_ERR_INVALID_ARGUMENT; }
    warm_occupancy();
    *out = c;
    return PA_OK;
}

pa_status pa_destroy(pa_ctx *c)
{
    if (!c) return PA_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto &kv : c->graphs) cudaGraphExecDestroy(kv.second);
    DevBuf *bufs[] = {&c->keys, &c->order, &c->hist, &c->starts, &c->cursor, &c->sums, &c->ranges,
                      &c->counts, &c->qtab, &c->boundary, &c->rerun, &c->counters, &c->pstats,
                      &c->in_seq1, &c->in_off1, &c->in_seq2, &c->in_off2, &c->in_out};
    for (DevBuf *b : bufs)
        if (b->p) cudaFree(b->p);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->ev2) cudaEventDestroy(c->ev2);
    if (c->ev3) cudaEventDestroy(c->ev3);
    if (c->ev_dp0) cudaEventDestroy(c->ev_dp0);
    if (c->ev_dp1) cudaEventDestroy(c->ev_dp1);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return PA_OK;
}

pa_status pa_align_batch_device(pa_ctx *ctx, const pa_config *config, const uint8_t *d_seq1, const uint64_t *d_off1,
                                uint64_t seq1_bytes, const uint8_t *d_seq2, const uint64_t *d_off2,
                                uint64_t seq2_bytes, uint64_t n_pairs, pa_result *d_out, void *stream,
                                pa_stats *stats)
{
    if (!ctx) return PA_ERR_INVALID_ARGUMENT;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, PA_ERR_CUDA, "cudaSetDevice");
    cudaStream_t user = (cudaStream_t)stream;
    if (user && user != ctx->stream) {
        // order the context stream after the caller's work, and the caller's after ours
        PA_CUDA(ctx, cudaEventRecord(ctx->ev2, user));
        PA_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->ev2, 0));
    }
    pa_status s = run_device(ctx, config, d_seq1, d_off1, seq1_bytes, d_seq2, d_off2, seq2_bytes, n_pairs, d_out,
                             stats, stats != nullptr);
    if (s) return s;
    if (user && user != ctx->stream) {
        PA_CUDA(ctx, cudaEventRecord(ctx->ev3, ctx->stream));
        PA_CUDA(ctx, cudaStreamWaitEvent(user, ctx->ev3, 0));
    }
    return PA_OK;
}

pa_status pa_align_batch(pa_ctx *ctx, const pa_config *config, const uint8_t *seq1, const uint64_t *off1,
                         const uint8_t *seq2, const uint64_t *off2, uint64_t n_pairs, pa_result *out,
                         pa_stats *stats)
{
    if (!ctx) return PA_ERR_INVALID_ARGUMENT;
    if (n_pairs == 0) {
        DpParams P; ClassCfg C;
        pa_status s = check_config(ctx, config, P, C);
        if (stats) std::memset(stats, 0, sizeof(*stats));
        return s;
    }
    if (!seq1 || !off1 || !seq2 || !off2 || !out) return fail(ctx, PA_ERR_INVALID_ARGUMENT, "null buffer");
    for (uint64_t k = 0; k < n_pairs; ++k)
        if (off1[k + 1] < off1[k] || off2[k + 1] < off2[k])
            return fail(ctx, PA_ERR_INVALID_ARGUMENT, "offsets must be non-decreasing");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, PA_ERR_CUDA, "cudaSetDevice");
    // the device copies hold bytes [0, off[n]) with offsets rebased to 0
    const uint64_t base1 = off1[0], base2 = off2[0];
    const uint64_t b1 = off1[n_pairs] - base1, b2 = off2[n_pairs] - base2;
    pa_status s;
    if ((s = ensure(ctx, ctx->in_seq1, b1))) return s;
    if ((s = ensure(ctx, ctx->in_seq2, b2))) return s;
    if ((s = ensure(ctx, ctx->in_off1, (n_pairs + 1) * 8))) return s;
    if ((s = ensure(ctx, ctx->in_off2, (n_pairs + 1) * 8))) return s;
    if ((s = ensure(ctx, ctx->in_out, n_pairs * sizeof(pa_result)))) return s;
    cudaStream_t st = ctx->stream;
    std::vector<uint64_t> r1, r2;
    const uint64_t *h1 = off1, *h2 = off2;
    if (base1) { r1.assign(off1, off1 + n_pairs + 1); for (auto &v : r1) v -= base1; h1 = r1.data(); }
    if (base2) { r2.assign(off2, off2 + n_pairs + 1); for (auto &v : r2) v -= base2; h2 = r2.data(); }
    if (b1) PA_CUDA(ctx, cudaMemcpyAsync(ctx->in_seq1.p, seq1 + base1, b1, cudaMemcpyHostToDevice, st));
    if (b2) PA_CUDA(ctx, cudaMemcpyAsync(ctx->in_seq2.p, seq2 + base2, b2, cudaMemcpyHostToDevice, st));
    PA_CUDA(ctx, cudaMemcpyAsync(ctx->in_off1.p, h1, (n_pairs + 1) * 8, cudaMemcpyHostToDevice, st));
    PA_CUDA(ctx, cudaMemcpyAsync(ctx->in_off2.p, h2, (n_pairs + 1) * 8, cudaMemcpyHostToDevice, st));
    s = run_device(ctx, config, (const uint8_t *)ctx->in_seq1.p, (const uint64_t *)ctx->in_off1.p, b1,
                   (const uint8_t *)ctx->in_seq2.p, (const uint64_t *)ctx->in_off2.p, b2, n_pairs,
                   (pa_result *)ctx->in_out.p, stats, false);
    if (s) return s;
    PA_CUDA(ctx, cudaMemcpyAsync(out, ctx->in_out.p, n_pairs * sizeof(pa_result), cudaMemcpyDeviceToHost, st));
    PA_CUDA(ctx, cudaStreamSynchronize(st));
    if (stats) {
        PrepStats ps;
        uint32_t ctr[8];
        PA_CUDA(ctx, cudaMemcpy(&ps, ctx->pstats.p, sizeof(ps), cudaMemcpyDeviceToHost));
        PA_CUDA(ctx, cudaMemcpy(ctr, ctx->counters.p, sizeof(ctr), cudaMemcpyDeviceToHost));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
        stats->device_ms = ms;
        if (cudaEventElapsedTime(&ms, ctx->ev_dp0, ctx->ev_dp1) == cudaSuccess) stats->dp_ms = ms;
        cudaGetLastError();
        stats->cells = ps.cells;
        stats->pairs_s16 = ps.n_class[K_S16] - ctr[4];
        stats->pairs_s32 = ps.n_class[K_S32] + ctr[4];
        stats->pairs_general = ps.n_class[K_GEN];
        stats->pairs_trivial = ps.n_class[K_NONE];
        stats->pairs_rerun = ctr[4];
        if (ps.overflow) return fail(ctx, PA_ERR_OVERFLOW, "scores of some pairs could exceed int32");
    } else {
        PrepStats ps;
        PA_CUDA(ctx, cudaMemcpy(&ps, ctx->pstats.p, sizeof(ps), cudaMemcpyDeviceToHost));
        if (ps.overflow) return fail(ctx, PA_ERR_OVERFLOW, "scores of some pairs could exceed int32");
    }
    return PA_OK;
}

pa_status pa_align_one_to_many(pa_ctx *ctx, const pa_config *config, const uint8_t *query, uint64_t query_len,
                               const uint8_t *targets, const uint64_t *target_off, uint64_t n_targets,
                               pa_result *out, pa_stats *stats)
{
    if (!ctx) return PA_ERR_INVALID_ARGUMENT;
    if (n_targets && (!target_off || (!query && query_len))) return fail(ctx, PA_ERR_INVALID_ARGUMENT, "null buffer");
    // replicate the query per pair: the device path reads sequence1 through offsets
    std::vector<uint8_t> q((size_t)(query_len * std::max<uint64_t>(n_targets, 1)));
    std::vector<uint64_t> qo(n_targets + 1);
    for (uint64_t k = 0; k < n_targets; ++k) {
        if (query_len) std::memcpy(q.data() + k * query_len, query, query_len);
        qo[k] = k * query_len;
    }
    qo[n_targets] = n_targets * query_len;
    return pa_align_batch(ctx, config, q.data(), qo.data(), targets, target_off, n_targets, out, stats);
}

pa_status pa_get_tuning(const pa_ctx *ctx, pa_tuning *out)
{
    if (!ctx || !out) return PA_ERR_INVALID_ARGUMENT;
    *out = ctx->tuning;
    return PA_OK;
}

static bool valid_G(int g) { return g >= 1 && g <= 32 && (g & (g - 1)) == 0; }
static bool valid_variant(int v) { return v >= 0 && v <= 4; }

pa_status pa_set_tuning(pa_ctx *ctx, const pa_tuning *t)
{
    if (!ctx || !t) return PA_ERR_INVALID_ARGUMENT;
    for (int m = 0; m < 2; ++m)
        if (!valid_variant(t->variant_s16[m]) || !valid_variant(t->variant_s32[m]) || !valid_G(t->group_threads_s16[m]) ||
            !valid_G(t->group_threads_s32[m]))
            return fail(ctx, PA_ERR_INVALID_ARGUMENT, "tuning: variant must be 0..4 and group_threads 1..32, power of two");
    ctx->tuning = *t;
    ctx->fixed_G = ctx->fixed_variant = false;
    return PA_OK;
}

pa_status pa_autotune(pa_ctx *ctx, const pa_config *config, const uint8_t *seq1, const uint64_t *off1,
                      const uint8_t *seq2, const uint64_t *off2, uint64_t n_pairs, pa_tuning *out)
{
    if (!ctx || !config) return PA_ERR_INVALID_ARGUMENT;
    const int mi = config->method == PA_METHOD_LOCAL ? 0 : 1;
    const pa_tuning saved = ctx->tuning;
    const bool fg = ctx->fixed_G, fv = ctx->fixed_variant;
    ctx->fixed_G = ctx->fixed_variant = false;
    std::vector<pa_result> res(std::max<uint64_t>(n_pairs, 1));
    double best = 1e300;
    pa_tuning choice = saved;
    static const int kVariants[] = {0, 1, 3, 4};
    static const int kGroups[] = {4, 8, 16};
    for (int v : kVariants)
        for (int g : kGroups) {
            pa_tuning t = saved;
            t.variant_s16[mi] = t.variant_s32[mi] = v;
            t.group_threads_s16[mi] = t.group_threads_s32[mi] = g;
            ctx->tuning = t;
            double ms = 1e300;
            for (int rep = 0; rep < 3; ++rep) {                 // first run captures the graph
                pa_stats st;
                pa_status s = pa_align_batch(ctx, config, seq1, off1, seq2, off2, n_pairs, res.data(), &st);
                if (s) { ctx->tuning = saved; ctx->fixed_G = fg; ctx->fixed_variant = fv; return s; }
                if (rep > 0) ms = std::min(ms, st.dp_ms);
            }
            if (ms < best) { best = ms; choice = t; }
        }
    choice.best_ms[mi] = best;
    ctx->tuning = choice;
    if (out) *out = choice;
    return PA_OK;
}

pa_status pa_measure_roofline(pa_ctx *ctx, pa_roofline *out)
{
    if (!ctx || !out) return PA_ERR_INVALID_ARGUMENT;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, PA_ERR_CUDA, "cudaSetDevice");
    DevBuf sink;
    pa_status s = ensure(ctx, sink, 1 << 20);
    if (s) return s;
    int per16 = 0, per32 = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per16, k_roofline<L16>, 256, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per32, k_roofline<L32>, 256, 0);
    const int steps = 4096;
    double best16 = 0, best32 = 0;
    for (int rep = 0; rep < 4; ++rep) {
        for (int w = 0; w < 2; ++w) {
            const int per = w ? per32 : per16;
            const int grid = std::max(1, per) * ctx->sm_count;
            PA_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
            if (w) k_roofline<L32><<<grid, 256, 0, ctx->stream>>>(steps, rep, (uint32_t *)sink.p);
            else k_roofline<L16><<<grid, 256, 0, ctx->stream>>>(steps, rep, (uint32_t *)sink.p);
            PA_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
            PA_CUDA(ctx, cudaEventSynchronize(ctx->ev1));
            float ms = 0;
            cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
            const double cells = (double)grid * 256 * steps * 16 * (w ? 1 : 2);
            const double r = cells / (ms * 1e-3);
            if (w) best32 = std::max(best32, r); else best16 = std::max(best16, r);
        }
    }
    cudaFree(sink.p);
    int clk = 0;
    cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, ctx->device);
    out->s16x2_cells_per_s = best16;
    out->s32_cells_per_s = best32;
    out->sm_clock_mhz = clk / 1000.0;
    out->sm_count = ctx->sm_count;
    out->reserved = 0;
    return PA_OK;
}

}  // extern "C"
