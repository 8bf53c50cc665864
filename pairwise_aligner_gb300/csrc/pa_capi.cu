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
constexpr int64_t kDefaultRingM = 65536;   // device entry points: CTA mode up to this sequence1 length
constexpr int kDefaultG = 8;       // threads per group
// Page-locked host words of a context: [0, 8) band mode's bad-offset count, [16, 80) class
// ranges, [80, 144) class counts, [160, 224) the two band steps' totals, [224, 236) the long
// full-DP routing counts, [256, 280) full-DP list sizes (host to device), [512, 736) the
// counters of a finished call (stage_stats).  Each is read only after a wait on the stream
// that wrote it, and written only after the previous call's work on that stream finished.
constexpr size_t kPinnedBytes = 1024;
constexpr int kShortVariant = 9;   // variants 9, 10: dp_short (s16x2 unitary short pairs), 16 / 32 rows per thread
constexpr int kVariants = kShortVariant + kShortFormCount;   // 0..8: dp_kernel (pa_kern_v*.cu)
constexpr int kDefaultShortVariant = kShortVariant;          // with the rule below: 16 or 32 rows per thread

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
};

struct GraphKey {
    const void *ptrs[6];
    uint64_t n_pairs, b1, b2;
    pa_config cfg;
    int32_t G[3], variant[3];      // the launch shapes the call was captured with
    uint32_t wait_limit;
    bool operator<(const GraphKey &o) const { return std::memcmp(this, &o, sizeof(GraphKey)) < 0; }
};

// A captured call and when it was last replayed (calls of the context count up).
struct GraphEntry {
    cudaGraphExec_t exec;
    uint64_t last_use;
};
constexpr size_t kMaxGraphs = 8;   // captured calls kept per context; the least recently used goes first

}  // namespace

struct pa_ctx {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr, ev3 = nullptr;
    cudaEvent_t ev_dp0 = nullptr, ev_dp1 = nullptr;   // bracket the DP kernels of the last call
    cudaStream_t side = nullptr;                      // cluster-mode kernels run beside the others
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaStream_t side2 = nullptr;                     // team kernels run beside the CTA kernels
    cudaEvent_t ev_join2 = nullptr;
    uint8_t *pinned = nullptr;                        // page-locked host words for band mode's reads
    pa_options opt{};
    std::string err;
    // device work buffers (grow only)
    DevBuf keys, order, hist, starts, cursor, sums, ranges, counts, qtab, boundary, rerun, counters, pstats;
    DevBuf slots;                 // short-pair kernel: 16-byte column slots, (seq1_bytes + n_pairs)
    DevBuf ring, rerun_long;      // CTA mode: boundary rows per block; s16 long pairs to redo in s32
    int32_t ring_m = 0;           // longest sequence1 the ring rows hold (0: no CTA mode yet)
    int ring_grid = 0;            // blocks of every CTA-mode launch
    int64_t long_cells = 1ll << 20;   // pairs with at least this many cells use CTA mode
    int64_t huge_cells = 1ll << 28;   // ... and with this many (and n >= huge_min_n) cluster mode
    int32_t huge_min_n = 8192;
    int32_t team_max_n = 12288;       // CTA-mode pairs with at most this many rows run on 4-warp teams
    uint32_t wait_limit = kSpinLimit; // polls of a CTA-mode progress wait before it gives up
    int64_t want_ring_m = 0;          // the next call's longest CTA-mode sequence1 (host: exact)
    DevBuf in_seq1, in_off1, in_seq2, in_off2, in_out;   // staging for the host-buffer entry points
    int G[3] = {kDefaultG, kDefaultG, kDefaultG};
    int variant[3] = {0, 0, 0};
    pa_tuning tuning{};           // per method (0 local, 1 global) and s16 table; applied per call
    bool fixed_G = false, fixed_variant = false;
    int grid[3] = {0, 0, 0};
    std::map<GraphKey, GraphEntry> graphs;
    uint64_t graph_clock = 0;
    uint64_t last_launches = 0;
    // band mode
    pa_band_options band_opt{1.25f, 16, 64, 0.85f, 2, 0.65f, {0, 0}};
    DevBuf band_spec, band_win, band_code, band_bsum, band_ctr, band_in;
    DevBuf band_list[22];
    DevBuf mlp_w[6], mlp_feat, mlp_x, mlp_h1, mlp_h2, mlp_out;
    bool has_model = false;
    // substitution matrix (PA_SCORE_MATRIX): int8 rank per byte (-1: not a symbol), int32 scores
    DevBuf mat_rank, mat_scores;
    int32_t mat_dim = 0, mat_max = 0, mat_min = 0;
    // input path: rank table, invalid-symbol counter, packed staging of pa_align_batch_packed
    DevBuf io_tab, io_ctr, in_words1, in_words2;
    // traceback: direction words of one chunk, their per-pair offsets, alignments and ops
    DevBuf tb_dir, tb_dir_off, tb_aln, tb_ops;
};

namespace {

// The ring rows of cluster-mode launches (CTA-mode launches use the first region).
Cell *team_ring(pa_ctx *c)
{
    return (Cell *)c->ring.p + (size_t)2 * c->ring_grid * 8 * ((size_t)c->ring_m + 2);
}

Cell *cluster_ring(pa_ctx *c)
{
    return (Cell *)c->ring.p + (size_t)c->ring_grid * 8 * ((size_t)c->ring_m + 2);
}

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

void drop_graphs(pa_ctx *c)
{
    for (auto &kv : c->graphs) cudaGraphExecDestroy(kv.second.exec);
    c->graphs.clear();
}

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
    drop_graphs(c);
    return PA_OK;
}

pa_status check_config(pa_ctx *c, const pa_config *cfg, DpParams &P, ClassCfg &C)
{
    if (!cfg) return fail(c, PA_ERR_INVALID_ARGUMENT, "config is null");
    const int32_t method = cfg->method & ~PA_SCORE_MATRIX;
    const bool use_matrix = (cfg->method & PA_SCORE_MATRIX) != 0;
    if (method != PA_METHOD_GLOBAL && method != PA_METHOD_LOCAL)
        return fail(c, PA_ERR_INVALID_ARGUMENT,
                    "method must be PA_METHOD_GLOBAL or PA_METHOD_LOCAL (optionally | PA_SCORE_MATRIX)");
    if (use_matrix && (!c || c->mat_dim == 0))
        return fail(c, PA_ERR_INVALID_ARGUMENT, "PA_SCORE_MATRIX needs pa_set_substitution_matrix first");
    if (use_matrix && cfg->band_mode != 0)
        return fail(c, PA_ERR_UNSUPPORTED, "band mode scores with match/mismatch only");
    if (cfg->gap_extension > 0 || (int64_t)cfg->gap_open + cfg->gap_extension > 0)
        return fail(c, PA_ERR_UNSUPPORTED, "positive gap scores are not supported");
    if (cfg->width_hint != 0 && cfg->width_hint != 16 && cfg->width_hint != 32)
        return fail(c, PA_ERR_INVALID_ARGUMENT, "width_hint must be 0, 16 or 32");
    if (cfg->band_mode < 0 || cfg->band_mode > 2)
        return fail(c, PA_ERR_INVALID_ARGUMENT, "band_mode must be 0, 1 or 2");
    const bool local = method == PA_METHOD_LOCAL;
    std::memset(&P, 0, sizeof(P));
    // with a matrix, match / mismatch hold its largest and smallest score: the bounds that
    // the padding score, the column shift and the overflow check need
    P.match = use_matrix ? c->mat_max : cfg->match;
    P.mismatch = use_matrix ? c->mat_min : cfg->mismatch;
    P.gap_open = cfg->gap_open;
    P.gap_ext = cfg->gap_extension;
    P.local = local;
    P.first_column_free = local || cfg->first_column_free;   // method_local.hpp:41-49
    P.first_row_free = local || cfg->first_row_free;
    P.last_column_free = !local && cfg->last_column_free;
    P.last_row_free = !local && cfg->last_row_free;
    P.smax = std::max(0, std::max(P.match, P.mismatch));
    P.spad = std::min(0, std::min(P.match, P.mismatch));
    P.shift = local ? 0 : P.smax;
    P.floor16 = -32768 + 1280;
    std::memset(&C, 0, sizeof(C));
    C.fast_scores = !use_matrix && cfg->match >= -127 && cfg->match <= 127 && cfg->mismatch >= -127 &&
                    cfg->mismatch <= 0 && cfg->match - P.shift >= -128 &&
                    cfg->mismatch - P.shift >= -128;   // byte tables of shifted scores
    C.rank_map = use_matrix ? (const int8_t *)c->mat_rank.p : nullptr;
    C.s16_params = (int64_t)cfg->gap_open + cfg->gap_extension >= -1000 && cfg->gap_extension >= -1000;
    C.force32 = cfg->width_hint == 32;
    C.local = local;
    for (int k = 0; k < kClasses; ++k) {
        const bool cta = k >= (int)kLongOffset;
        C.gcnt[k] = cta ? 32 : c->G[k < 3 ? k : 0];
        C.rpt[k] = kR;
        C.rows[k] = C.gcnt[k] * kR;
    }
    C.long_cells = c->long_cells;
    C.huge_cells = c->huge_cells;
    C.huge_min_n = c->huge_min_n;
    C.team_max_n = c->team_max_n;
    C.long_max_m = c->ring.p ? c->ring_m : 0;
    C.qtab_s16 = 1;
    return PA_OK;
}

}  // namespace

namespace pa {
int dp_occupancy_v0(bool lanes16, bool gen, int mode);
int dp_occupancy_v1(bool lanes16, bool gen, int mode);
int dp_occupancy_v2(bool lanes16, bool gen, int mode);
int dp_occupancy_v3(bool lanes16, bool gen, int mode);
int dp_occupancy_v4(bool lanes16, bool gen, int mode);
int dp_occupancy_v5(bool lanes16, bool gen, int mode);
int dp_occupancy_v6(bool lanes16, bool gen, int mode);
int dp_occupancy_v7(bool lanes16, bool gen, int mode);
int dp_occupancy_v8(bool lanes16, bool gen, int mode);
void dp_launch_v0(bool, bool, int, int, cudaStream_t, const DpLaunch &, const DpParams &);
void dp_launch_v1(bool, bool, int, int, cudaStream_t, const DpLaunch &, const DpParams &);
void dp_launch_v2(bool, bool, int, int, cudaStream_t, const DpLaunch &, const DpParams &);
void dp_launch_v3(bool, bool, int, int, cudaStream_t, const DpLaunch &, const DpParams &);
void dp_launch_v4(bool, bool, int, int, cudaStream_t, const DpLaunch &, const DpParams &);
void dp_launch_v5(bool, bool, int, int, cudaStream_t, const DpLaunch &, const DpParams &);
void dp_launch_v6(bool, bool, int, int, cudaStream_t, const DpLaunch &, const DpParams &);
void dp_launch_v7(bool, bool, int, int, cudaStream_t, const DpLaunch &, const DpParams &);
void dp_launch_v8(bool, bool, int, int, cudaStream_t, const DpLaunch &, const DpParams &);

void rank_map_launch(const uint8_t *in, uint64_t n, int8_t *out, const int8_t *table, unsigned long long *invalid,
                     int sm_count, cudaStream_t st);
void pack_2bit_launch(const uint8_t *in, uint64_t n, uint32_t *words, unsigned long long *invalid, int sm_count,
                      cudaStream_t st);
void unpack_2bit_launch(const uint32_t *words, uint64_t first_base, uint64_t n, uint8_t *out, int sm_count,
                        cudaStream_t st);

int dp_short_occupancy_local(int G, int form);
void dp_short_launch_local(int G, int form, int grid, cudaStream_t st, const DpLaunch &L, const DpParams &P);
int dp_short_occupancy_global(int G, int form);
void dp_short_launch_global(int G, int form, int grid, cudaStream_t st, const DpLaunch &L, const DpParams &P);
int dp_short_occupancy_free(int G);
void dp_short_launch_free(int G, int grid, cudaStream_t st, const DpLaunch &L, const DpParams &P);

int dp_short_occupancy(int G, int form, int mode)
{
    return mode == M_LOCAL ? dp_short_occupancy_local(G, form)
         : mode == M_GLOBAL ? dp_short_occupancy_global(G, form) : dp_short_occupancy_free(G);
}

void dp_short_launch(int G, int form, int mode, int grid, cudaStream_t st, const DpLaunch &L, const DpParams &P)
{
    if (mode == M_LOCAL) dp_short_launch_local(G, form, grid, st, L, P);
    else if (mode == M_GLOBAL) dp_short_launch_global(G, form, grid, st, L, P);
    else dp_short_launch_free(G, grid, st, L, P);
}

int dp_occupancy(int variant, bool lanes16, bool gen, int mode)
{
    if (variant == 1) return dp_occupancy_v1(lanes16, gen, mode);
    if (variant == 2) return dp_occupancy_v2(lanes16, gen, mode);
    if (variant == 3) return dp_occupancy_v3(lanes16, gen, mode);
    if (variant == 4) return dp_occupancy_v4(lanes16, gen, mode);
    if (variant == 5) return dp_occupancy_v5(lanes16, gen, mode);
    if (variant == 6) return dp_occupancy_v6(lanes16, gen, mode);
    if (variant == 7) return dp_occupancy_v7(lanes16, gen, mode);
    if (variant == 8) return dp_occupancy_v8(lanes16, gen, mode);
    return dp_occupancy_v0(lanes16, gen, mode);
}

void band_labels_launch(bool reverse, int grid, cudaStream_t st, const DpLaunch &L, const DpParams &P);
void band_labels_cta_launch(bool reverse, int grid, cudaStream_t st, const DpLaunch &L, const DpParams &P);
int band_labels_occupancy();
int band_labels_cta_occupancy();
int band_dp_occupancy(bool lanes16, bool cta);
int band_cta_occupancy();
void band_dp_launch(bool lanes16, bool cta, int grid, cudaStream_t st, const DpLaunch &L, const DpParams &P);
void band_windows_launch(cudaStream_t st, const uint64_t *off1, const uint64_t *off2, const uint32_t *list,
                         uint32_t count, const BandSpec *spec, int32_t rows, int shift, float full_frac,
                         float team_frac, int32_t team_max_n, int2 *win, uint8_t *code,
                         unsigned long long *width_stats);
void size_code_launch(cudaStream_t st, const uint64_t *off1, const uint64_t *off2, const uint32_t *list,
                      uint32_t count, int32_t team_max_n, int64_t huge_cells, int32_t huge_min_n, uint8_t *code);
void band_decode_launch(cudaStream_t st, const float *out, const uint64_t *off1, const uint64_t *off2,
                        uint64_t n_pairs, const DpParams &P, float margin, int32_t w_min, BandSpec *spec);
void band_straight_launch(cudaStream_t st, const uint64_t *off1, const uint64_t *off2, uint64_t n_pairs,
                          int32_t w_start, int32_t w_min, BandSpec *spec);
void band_from_ints_launch(cudaStream_t st, const int32_t *in, uint64_t n_pairs, BandSpec *spec);
void compact_launch(cudaStream_t st, const uint32_t *list, const uint8_t *code, uint32_t count, uint8_t sel,
                    uint32_t *block_sum, uint32_t *out, uint32_t *total);
void mark_full_launch(cudaStream_t st, pa_result *out, uint64_t n_pairs);

void dp_launch(int variant, bool lanes16, bool gen, int mode, int grid, cudaStream_t st, const DpLaunch &L,
               const DpParams &P)
{
    if (variant == 1) dp_launch_v1(lanes16, gen, mode, grid, st, L, P);
    else if (variant == 2) dp_launch_v2(lanes16, gen, mode, grid, st, L, P);
    else if (variant == 3) dp_launch_v3(lanes16, gen, mode, grid, st, L, P);
    else if (variant == 4) dp_launch_v4(lanes16, gen, mode, grid, st, L, P);
    else if (variant == 5) dp_launch_v5(lanes16, gen, mode, grid, st, L, P);
    else if (variant == 6) dp_launch_v6(lanes16, gen, mode, grid, st, L, P);
    else if (variant == 7) dp_launch_v7(lanes16, gen, mode, grid, st, L, P);
    else if (variant == 8) dp_launch_v8(lanes16, gen, mode, grid, st, L, P);
    else dp_launch_v0(lanes16, gen, mode, grid, st, L, P);
}
}  // namespace pa

namespace {

// Resident blocks per SM of every DP kernel, queried once outside any stream capture.
void warm_occupancy()
{
    for (int v = 0; v < kShortVariant; ++v)
        for (int mode = 0; mode < 3; ++mode) {
            dp_occupancy(v, true, false, mode);
            dp_occupancy(v, false, false, mode);
            dp_occupancy(v, false, true, mode);
        }
    for (int g = 4; g <= 32; g *= 2)
        for (int form = 0; form < kShortFormCount; ++form)
            for (int mode = 0; mode < 3; ++mode) dp_short_occupancy(g, form, mode);
}

void launch_class(pa_ctx *c, int slot, int mode, bool lanes16, bool gen, const DpLaunch &L, const DpParams &P)
{
    int v = c->variant[slot];
    if (v >= kShortVariant) {
        // the short-pair kernel covers s16x2 lanes with unitary scores in the plain modes and
        // groups of 4..32 lanes; anything else takes the default dp_kernel form
        if (lanes16 && !gen && mode <= M_GLOBAL_FREE && dp_short_supports(L.G) && L.slots) {
            // the free-end-gap form keeps 16 rows per thread (32 do not fit its registers)
            const int form = mode == M_GLOBAL_FREE ? 0 : v - kShortVariant;
            int per_sm = dp_short_occupancy(L.G, form, mode);
            if (c->opt.blocks_per_sm > 0) per_sm = std::min(per_sm, (int)c->opt.blocks_per_sm);
            c->grid[slot] = per_sm * c->sm_count;
            dp_short_launch(L.G, form, mode, c->grid[slot], c->stream, L, P);
            c->last_launches++;
            return;
        }
        v = mode == M_LOCAL ? 7 : 4;
    }
    int per_sm = dp_occupancy(v, lanes16, gen, mode);
    if (c->opt.blocks_per_sm > 0) per_sm = std::min(per_sm, (int)c->opt.blocks_per_sm);
    c->grid[slot] = per_sm * c->sm_count;
    dp_launch(v, lanes16, gen, mode, c->grid[slot], c->stream, L, P);
    c->last_launches++;
}

// Classify, bucket and sort the pairs (steps 1-3); no host sync.
pa_status enqueue_prep(pa_ctx *c, const DpParams &P, const ClassCfg &C, const uint8_t *s1, const uint64_t *o1,
                       uint64_t b1, const uint8_t *s2, const uint64_t *o2, uint64_t b2, pa_result *out,
                       uint64_t n_pairs)
{
    cudaStream_t st = c->stream;
    PA_CUDA(c, cudaMemsetAsync(c->hist.p, 0, sizeof(uint32_t) * kBuckets, st));
    PA_CUDA(c, cudaMemsetAsync(c->counters.p, 0, 128, st));
    PA_CUDA(c, cudaMemsetAsync(c->pstats.p, 0, sizeof(PrepStats), st));
    // one resident wave (16 blocks of 4 warps per SM), each warp a stride of pairs: every block
    // adds its statistics to the same few global counters once, so fewer blocks contend less
    int cls_blocks = (int)std::min<uint64_t>((n_pairs * 32 + 127) / 128, (uint64_t)c->sm_count * 16);
    if (cls_blocks < 1) cls_blocks = 1;
    k_classify<<<cls_blocks, 128, 0, st>>>(s1, o1, b1, s2, o2, b2, n_pairs, P, C, (uint32_t *)c->keys.p,
                                              (uint32_t *)c->hist.p, (uint32_t *)c->qtab.p, out,
                                              (PrepStats *)c->pstats.p);
    k_scan_blocks<<<kBuckets / 1024, 1024, 0, st>>>((uint32_t *)c->hist.p, (uint32_t *)c->starts.p,
                                                    (uint32_t *)c->sums.p);
    k_scan_sums<<<1, kBuckets / 1024, 0, st>>>((uint32_t *)c->sums.p, kBuckets / 1024);
    k_scan_add<<<kBuckets / 1024, 1024, 0, st>>>((uint32_t *)c->starts.p, (uint32_t *)c->cursor.p,
                                                 (uint32_t *)c->sums.p, (uint32_t *)c->ranges.p);
    const int sc_blocks = (int)std::max<uint64_t>(1, (n_pairs + kBlock - 1) / kBlock);
    k_scatter<<<sc_blocks, kBlock, 0, st>>>((uint32_t *)c->keys.p, n_pairs, (uint32_t *)c->cursor.p,
                                            (uint32_t *)c->order.p, (uint32_t *)c->ranges.p,
                                            (uint32_t *)c->counts.p, (const PrepStats *)c->pstats.p, out);
    c->last_launches += 6;
    PA_CUDA(c, cudaGetLastError());
    return PA_OK;
}

// Everything between inputs-on-device and results-on-device; no host sync.
pa_status enqueue(pa_ctx *c, const pa_config *cfg, const DpParams &P, const ClassCfg &C, const uint8_t *s1,
                  const uint64_t *o1, uint64_t b1, const uint8_t *s2, const uint64_t *o2, uint64_t b2,
                  pa_result *out, uint64_t n_pairs)
{
    cudaStream_t st = c->stream;
    // counters: [0..3] group queues, [4] rerun count, [5] zero, [6] long rerun count, [8] error
    // bits, [9..12] CTA queues, [13..15] cluster queues, [16..21] routing of the largest pairs
    uint32_t *counters = (uint32_t *)c->counters.p;
    pa_status ps = enqueue_prep(c, P, C, s1, o1, b1, s2, o2, b2, out, n_pairs);
    if (ps) return ps;
    const int cl_grid = c->ring.p ? dp_cluster_grid(true, false, P.local ? M_LOCAL : M_GLOBAL, c->ring_grid) : 0;
    if (c->ring.p) {
        k_route_huge<<<1, 1, 0, st>>>((const uint32_t *)c->counts.p, (uint32_t)(cl_grid / kClusterBlocks),
                                      counters + 16);
        c->last_launches++;
    }

    const int mode = P.local ? M_LOCAL : ((P.last_column_free || P.last_row_free) ? M_GLOBAL_FREE : M_GLOBAL);
    DpLaunch L;
    std::memset(&L, 0, sizeof(L));
    L.seq1 = s1; L.off1 = o1; L.seq2 = s2; L.off2 = o2;
    L.qtab = (const uint32_t *)c->qtab.p;
    L.order = (const uint32_t *)c->order.p;
    L.out = out;
    L.boundary = (Cell *)c->boundary.p;
    L.slots = (Slot *)c->slots.p;
    L.spin_limit = c->wait_limit;
    L.rerun_list = (uint32_t *)c->rerun.p;
    L.rerun_count = counters + 4;
    if (C.rank_map) {
        L.rank_map = C.rank_map;
        L.matrix = (const int32_t *)c->mat_scores.p;
        L.mdim = c->mat_dim;
    }
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
    // the largest pairs, on the side stream forked after the group kernels: clusters of blocks
    // per pair, beside the CTA-mode kernels below, which fill the SMs the clusters leave free
    DpLaunch LL = L;
    if (c->ring.p) {
        LL.ring = (Cell *)c->ring.p;
        LL.ring_stride = (uint64_t)c->ring_m + 2;
        LL.error = counters + 8;
        LL.rerun_list = (uint32_t *)c->rerun_long.p;
        LL.rerun_count = counters + 6;
        LL.G = 32;
        PA_CUDA(c, cudaEventRecord(c->ev_fork, st));
        PA_CUDA(c, cudaStreamWaitEvent(c->side, c->ev_fork, 0));
        DpLaunch LC = LL;
        LC.ring = cluster_ring(c);
        const Klass hc[3] = {K_S16H, K_S32H, K_GENH};
        for (int k = 0; k < 3; ++k) {
            LC.begin_ptr = ranges + hc[k]; LC.count_ptr = counters + 16 + k; LC.unit_counter = counters + 13 + k;
            PA_CUDA(c, dp_cluster_launch(k == 0, k == 2, mode, dp_cluster_grid(k == 0, k == 2, mode, c->ring_grid),
                                         c->side, LC, P));
        }
        PA_CUDA(c, cudaEventRecord(c->ev_join, c->side));
    }
    // long pairs: whole blocks per pair; their s16 results that fail the check are redone in s32
    if (c->ring.p) {
        const Klass lc[3] = {K_S16L, K_S32L, K_GENL}, hl[3] = {K_S16H, K_S32H, K_GENH};
        for (int k = 0; k < 3; ++k) {
            LL.begin_ptr = ranges + lc[k]; LL.count_ptr = counts + lc[k]; LL.unit_counter = counters + 9 + k;
            LL.lead_order = (const uint32_t *)c->order.p;          // the largest pairs the router left here
            LL.lead_begin_ptr = ranges + hl[k];
            LL.lead_count_ptr = counters + 19 + k;
            dp_cta_launch(k == 0, k == 2, mode, c->ring_grid, st, LL, P);
        }
        LL.lead_order = nullptr;
        LL.lead_begin_ptr = nullptr;
        LL.lead_count_ptr = nullptr;
        // long pairs with few passes: teams of 4 warps on a second side stream with their own
        // ring rows, launched after the CTA-mode kernels so that those take the SMs first; the
        // teams fill the SMs that the blocks of the longer pairs release
        if (C.team_max_n > 0) {
            PA_CUDA(c, cudaStreamWaitEvent(c->side2, c->ev_fork, 0));
            DpLaunch LT = LL;
            LT.ring = team_ring(c);
            const Klass mc[3] = {K_S16M, K_S32M, K_GENM};
            for (int k = 0; k < 3; ++k) {
                LT.begin_ptr = ranges + mc[k]; LT.count_ptr = counts + mc[k]; LT.unit_counter = counters + 22 + k;
                dp_team_launch(k == 0, k == 2, mode, c->ring_grid, c->side2, LT, P);
            }
            PA_CUDA(c, cudaEventRecord(c->ev_join2, c->side2));
            PA_CUDA(c, cudaStreamWaitEvent(st, c->ev_join2, 0));   // the team kernels' results and redo list
        }
        PA_CUDA(c, cudaStreamWaitEvent(st, c->ev_join, 0));   // the cluster kernels' results and redo list
        if (mode != M_LOCAL) {
            LL.order = (const uint32_t *)c->rerun_long.p;
            LL.begin_ptr = counters + 5;
            LL.count_ptr = counters + 6;
            LL.unit_counter = counters + 12;
            LL.rerun = 1;
            dp_cta_launch(false, false, mode, c->ring_grid, st, LL, P);
        }
        c->last_launches += (mode != M_LOCAL ? 7 : 6) + (C.team_max_n > 0 ? 3 : 0);
    }
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

// Ring rows of CTA mode for sequence1 lengths up to `max_m` (grow only).
pa_status ensure_ring(pa_ctx *c, int64_t max_m)
{
    if (max_m <= 0) return PA_OK;
    if (max_m > (1 << 20)) max_m = 1 << 20;
    if (c->ring.p && c->ring_m >= max_m) return PA_OK;
    int per_sm = 1;
    for (int mode = 0; mode < 3; ++mode) {
        per_sm = std::max(per_sm, dp_cta_occupancy(true, false, mode));
        per_sm = std::max(per_sm, dp_cta_occupancy(false, false, mode));
        per_sm = std::max(per_sm, dp_cta_occupancy(false, true, mode));
        per_sm = std::max(per_sm, dp_team_occupancy(true, false, mode));
        per_sm = std::max(per_sm, dp_team_occupancy(false, false, mode));
        per_sm = std::max(per_sm, dp_team_occupancy(false, true, mode));
    }
    per_sm = std::max(per_sm, band_cta_occupancy());
    per_sm = std::max(per_sm, band_labels_cta_occupancy());
    const int grid = per_sm * c->sm_count;
    const int32_t m = (int32_t)std::max<int64_t>(max_m, c->ring_m);
    // two regions: CTA-mode blocks and cluster-mode blocks run at the same time
    // three regions: CTA-mode blocks, cluster-mode blocks and team blocks run at the same time
    pa_status s = ensure(c, c->ring, (size_t)3 * grid * 8 * ((size_t)m + 2) * sizeof(Cell));
    if (s) return s;
    c->ring_m = m;
    c->ring_grid = grid;
    return PA_OK;
}

pa_status prepare_buffers(pa_ctx *c, uint64_t n_pairs, uint64_t b1)
{
    pa_status s;
    const uint64_t np = std::max<uint64_t>(n_pairs, 1);
    if ((s = ensure(c, c->keys, np * 4))) return s;
    if ((s = ensure(c, c->order, np * 4))) return s;
    if ((s = ensure(c, c->rerun, np * 4))) return s;
    if ((s = ensure(c, c->rerun_long, np * 4))) return s;
    if ((s = ensure(c, c->hist, sizeof(uint32_t) * kBuckets))) return s;
    if ((s = ensure(c, c->starts, sizeof(uint32_t) * kBuckets))) return s;
    if ((s = ensure(c, c->cursor, sizeof(uint32_t) * kBuckets))) return s;
    if ((s = ensure(c, c->sums, sizeof(uint32_t) * 1024))) return s;
    if ((s = ensure(c, c->ranges, 64))) return s;
    if ((s = ensure(c, c->counts, 64))) return s;
    if ((s = ensure(c, c->counters, 128))) return s;
    if ((s = ensure(c, c->pstats, sizeof(PrepStats)))) return s;
    if ((s = ensure(c, c->qtab, (b1 + np) * 4))) return s;
    if ((s = ensure(c, c->boundary, (b1 + np) * sizeof(Cell)))) return s;
    if ((s = ensure(c, c->slots, (b1 + np) * sizeof(Slot)))) return s;
    return PA_OK;
}

// Buckets of the s16x2 tuning table (pa_tuning::s16): batch-size class and pair-size class.
int tune_size_class(uint64_t n_pairs)
{
    for (int s = 0; s < PA_TUNE_SIZES - 1; ++s)
        if (n_pairs < (1ull << (12 + 2 * s))) return s;
    return PA_TUNE_SIZES - 1;
}

int tune_shape_class(uint64_t n_pairs, uint64_t b1, uint64_t b2)
{
    const double mean = n_pairs ? ((double)b1 / (double)n_pairs) * ((double)b2 / (double)n_pairs) : 0.0;
    for (int h = 0; h < PA_TUNE_SHAPES - 1; ++h)
        if (mean < (double)(1ull << (14 + 2 * h))) return h;
    return PA_TUNE_SHAPES - 1;
}

// The built-in group size: the smallest group (fewest fill and drain steps per pass) that
// still gives every resident warp about eight work units, so the persistent queue's tail
// stays short.  A warp unit holds 32 / G groups of `lanes` pairs.
int rule_group_threads(const pa_ctx *c, uint64_t n_pairs, int lanes)
{
    const double warps = (double)c->sm_count * (2 * kBlock / 32);
    for (int g = 4; g < 32; g *= 2)
        if ((double)n_pairs * g / (32.0 * lanes) >= 8.0 * warps) return g;
    return 32;
}

void apply_tuning(pa_ctx *c, const pa_config *cfg, uint64_t n_pairs, uint64_t b1, uint64_t b2)
{
    if (!cfg) return;
    const int mi = (cfg->method & ~PA_SCORE_MATRIX) == PA_METHOD_LOCAL ? 0 : 1;
    const pa_tune_entry &e = c->tuning.s16[mi][tune_size_class(n_pairs)][tune_shape_class(n_pairs, b1, b2)];
    if (!c->fixed_variant) {
        c->variant[K_S16] = e.group_threads ? e.variant : c->tuning.variant_s16[mi];
        c->variant[K_S32] = c->variant[K_GEN] = c->tuning.variant_s32[mi];
    }
    if (!c->fixed_G) {
        int g16 = e.group_threads ? e.group_threads : c->tuning.group_threads_s16[mi];
        int g32 = c->tuning.group_threads_s32[mi];
        c->G[K_S16] = g16 ? g16 : rule_group_threads(c, n_pairs, 2);
        c->G[K_S32] = c->G[K_GEN] = g32 ? g32 : rule_group_threads(c, n_pairs, 1);
        // untuned short-pair kernel: 32 rows per thread where groups are small (large batches;
        // half the column steps of 16 rows), 16 where they are large (few pairs: 32 rows would
        // make passes of 512-1,024 rows, mostly padding for short pairs)
        if (!e.group_threads && !g16 && !c->fixed_variant && c->tuning.variant_s16[mi] >= kShortVariant)
            c->variant[K_S16] = c->G[K_S16] <= 8 ? kShortVariant + 1 : kShortVariant;
    }
}

// Band predictor inference on the device: features, MLP, decode to BandSpec.
pa_status band_predict(pa_ctx *c, const DpParams &P, const uint8_t *s1, const uint64_t *o1, const uint8_t *s2,
                       const uint64_t *o2, uint64_t np, BandSpec *spec)
{
    const uint64_t chunk = std::min<uint64_t>(np, 65536);
    pa_status s;
    if ((s = ensure(c, c->mlp_feat, chunk * 130 * 4))) return s;
    if ((s = ensure(c, c->mlp_x, chunk * 144 * 2))) return s;
    if ((s = ensure(c, c->mlp_h1, chunk * 256 * 2))) return s;
    if ((s = ensure(c, c->mlp_h2, chunk * 256 * 2))) return s;
    if ((s = ensure(c, c->mlp_out, chunk * 16 * 4))) return s;
    cudaStream_t st = c->stream;
    float *feat = (float *)c->mlp_feat.p, *out = (float *)c->mlp_out.p;
    void *x = c->mlp_x.p, *h1 = c->mlp_h1.p, *h2 = c->mlp_h2.p;
    const float *b1 = (const float *)c->mlp_w[1].p, *b2 = (const float *)c->mlp_w[3].p,
                *b3 = (const float *)c->mlp_w[5].p;
    for (uint64_t start = 0; start < np; start += chunk) {
        const int cnt = (int)std::min<uint64_t>(chunk, np - start);
        if ((s = pa_band_features_device(s1, o1 + start, s2, o2 + start, cnt, feat, st)) ||
            (s = pa_mlp_to_bf16(feat, cnt, 130, 144, x, st)) ||
            (s = pa_mlp_gemm(x, c->mlp_w[0].p, nullptr, h1, b1, cnt, 256, 144, 144, 256, 256, 0, 0, 1, 0.f, st)) ||
            (s = pa_mlp_gemm(h1, c->mlp_w[2].p, nullptr, h2, b2, cnt, 256, 256, 256, 256, 256, 0, 0, 1, 0.f, st)) ||
            (s = pa_mlp_gemm(h2, c->mlp_w[4].p, out, nullptr, b3, cnt, 16, 256, 256, 16, 16, 0, 0, 0, 0.f, st)))
            return fail(c, s, "band predictor launch failed");
        band_decode_launch(st, out, o1 + start, o2 + start, cnt, P, c->band_opt.margin, c->band_opt.w_min,
                           spec + start);
        c->last_launches += 6;
    }
    PA_CUDA(c, cudaGetLastError());
    return PA_OK;
}

pa_status read_stats(pa_ctx *c, pa_stats *stats, bool staged = false);
void stage_stats(pa_ctx *c, cudaStream_t st);

// Band mode (host-synchronous between rounds): classify and sort as the plain
// path, build every pair's band, then per round and work class: windows ->
// (too wide: full-DP list) -> banded DP -> certified results, pairs to widen,
// and s16 results to redo in s32; finally the full DP for what is left.
pa_status run_band(pa_ctx *c, const pa_config *cfg, const uint8_t *s1, const uint64_t *o1, uint64_t b1,
                   const uint8_t *s2, const uint64_t *o2, uint64_t b2, uint64_t n_pairs, pa_result *out,
                   const int32_t *h_bands, pa_stats *stats, bool sync_at_end)
{
    apply_tuning(c, cfg, n_pairs, b1, b2);
    pa_status s = n_pairs ? ensure_ring(c, c->want_ring_m) : PA_OK;
    if (s) return s;
    DpParams P;
    ClassCfg C;
    if ((s = check_config(c, cfg, P, C))) return s;
    C.team_max_n = 0;                                 // band mode has its own team choice
    if (P.local || P.first_column_free || P.first_row_free || P.last_column_free || P.last_row_free)
        return fail(c, PA_ERR_UNSUPPORTED, "band mode needs global alignment with penalised end gaps");
    if (!h_bands && cfg->band_mode == 1 && !c->has_model)
        return fail(c, PA_ERR_INVALID_ARGUMENT, "band_mode 1 needs a band model (pa_set_band_model)");
    if (stats) std::memset(stats, 0, sizeof(*stats));
    if (n_pairs == 0) return PA_OK;
    if (!s1 || !o1 || !s2 || !o2 || !out) return fail(c, PA_ERR_INVALID_ARGUMENT, "null buffer");
    if (n_pairs >= (1ull << 31)) return fail(c, PA_ERR_TOO_LARGE, "n_pairs must be < 2^31");
    if ((s = prepare_buffers(c, n_pairs, b1))) return s;
    const uint64_t np = n_pairs;
    // the band work classes: {lanes16, cta} -> s16 groups, s32 groups, s16 blocks, s32 blocks
    // the band work classes: s16x2 / s32 lanes x one group / one block / one cluster per unit
    struct BandClass {
        bool lanes16;
        int kind;                 // 0 groups, 1 CTA mode, 2 cluster mode
        Klass klass;
        int rows;
    };
    constexpr int NB = 6;
    BandClass bc[NB] = {{true, 0, K_S16, c->G[K_S16] * kR}, {false, 0, K_S32, c->G[K_S32] * kR},
                        {true, 1, K_S16L, 32 * kR},         {false, 1, K_S32L, 32 * kR},
                        {true, 2, K_S16H, 32 * kR},         {false, 2, K_S32H, 32 * kR}};
    const int min_rows = std::min(std::min(bc[0].rows, bc[1].rows), 32 * kR);
    if ((s = ensure(c, c->band_spec, np * sizeof(BandSpec)))) return s;
    if ((s = ensure(c, c->band_win, (b2 / min_rows + np + 1) * sizeof(int2)))) return s;
    if ((s = ensure(c, c->band_code, np))) return s;
    if ((s = ensure(c, c->band_bsum, (np / 1024 + 2) * 4))) return s;
    if ((s = ensure(c, c->band_ctr, 256))) return s;
    for (DevBuf &b : c->band_list)
        if ((s = ensure(c, b, np * 4))) return s;
    cudaStream_t st = c->stream;
    c->last_launches = 0;
    uint32_t *counters = (uint32_t *)c->counters.p;
    uint32_t *ctr = (uint32_t *)c->band_ctr.p;      // [0] zero, [1..31] totals and queues, [32..33] cells
    PA_CUDA(c, cudaEventRecord(c->ev0, st));
    PA_CUDA(c, cudaMemsetAsync(c->counters.p, 0, 128, st));
    PA_CUDA(c, cudaMemsetAsync(c->band_ctr.p, 0, 256, st));
    if ((s = enqueue_prep(c, P, C, s1, o1, b1, s2, o2, b2, out, np))) return s;
    BandSpec *spec = (BandSpec *)c->band_spec.p;
    DpLaunch L;
    std::memset(&L, 0, sizeof(L));
    L.seq1 = s1; L.off1 = o1; L.seq2 = s2; L.off2 = o2;
    L.qtab = (const uint32_t *)c->qtab.p;
    L.out = out;
    L.boundary = (Cell *)c->boundary.p;
    L.slots = (Slot *)c->slots.p;
    L.band_win = (const int2 *)c->band_win.p;
    L.band = spec;
    L.band_code = (uint8_t *)c->band_code.p;
    L.dp_cells = (unsigned long long *)(ctr + 32);
    L.ring = (Cell *)c->ring.p;
    L.ring_stride = (uint64_t)c->ring_m + 2;
    L.error = counters + 8;
    L.spin_limit = c->wait_limit;
    // Predicted bands (modes 1 and 2) are tried on long pairs only, the block and cluster classes
    // (m * n at least the CTA threshold, 2^20 by default).  On shorter pairs the full DP of the
    // short-pair kernel is faster than the band machinery can save (their predicted bands cover
    // most of the matrix anyway), so they go straight to the full DP; a batch without long pairs
    // skips the band prediction altogether.  Caller-given bands are tried on every pair.
    const bool short_full = h_bands == nullptr;
    // page-locked host words: the copies below do not wait for the stream, so the group
    // classes' full DP is queued before the host waits for the class counts
    unsigned long long *h_bad = (unsigned long long *)c->pinned;
    uint32_t *h_ranges = (uint32_t *)(c->pinned + 16), *h_counts = (uint32_t *)(c->pinned + 80);
    uint32_t ranges[16], counts[16];
    {
        // the classifier checked the offsets; a batch with inconsistent ones is not aligned (and
        // the band features, which read the sequences, must not run on it)
        PA_CUDA(c, cudaMemcpyAsync(h_bad, &((PrepStats *)c->pstats.p)->bad_offsets, 8, cudaMemcpyDeviceToHost, st));
        PA_CUDA(c, cudaMemcpyAsync(h_ranges, c->ranges.p, 64, cudaMemcpyDeviceToHost, st));
        PA_CUDA(c, cudaMemcpyAsync(h_counts, c->counts.p, 4 * kClasses, cudaMemcpyDeviceToHost, st));
        PA_CUDA(c, cudaEventRecord(c->ev_join, st));
        if (short_full) {
            // the group classes take the full DP whatever the counts: start it now from the
            // device-side class ranges (as the plain path does), so that it runs while the host
            // reads them; with offsets that failed the check the classes are empty
            DpLaunch F = L;
            F.order = (const uint32_t *)c->order.p;
            F.rerun_list = (uint32_t *)c->rerun.p;
            F.rerun_count = counters + 4;
            const Klass gk[2] = {K_S16, K_S32};
            for (int k = 0; k < 2; ++k) {
                F.begin_ptr = (const uint32_t *)c->ranges.p + gk[k];
                F.count_ptr = (const uint32_t *)c->counts.p + gk[k];
                F.unit_counter = counters + k;
                F.G = c->G[gk[k]];
                launch_class(c, gk[k], M_GLOBAL, k == 0, false, F, P);
            }
        }
        PA_CUDA(c, cudaEventSynchronize(c->ev_join));
        std::memcpy(ranges, h_ranges, sizeof(ranges));
        std::memcpy(counts, h_counts, 4 * kClasses);
        if (*h_bad) {
            PA_CUDA(c, cudaStreamSynchronize(st));
            return fail(c, PA_ERR_INVALID_ARGUMENT,
                        "offsets decrease or run past seq1_bytes / seq2_bytes; no pair was aligned");
        }
    }
    const uint32_t n_long = counts[K_S16L] + counts[K_S32L] + counts[K_S16H] + counts[K_S32H];
    if (short_full && n_long == 0) {
        // nothing to band
    } else if (h_bands) {
        if ((s = ensure(c, c->band_in, np * 40))) return s;
        PA_CUDA(c, cudaMemcpyAsync(c->band_in.p, h_bands, np * 40, cudaMemcpyHostToDevice, st));
        band_from_ints_launch(st, (const int32_t *)c->band_in.p, np, spec);
        c->last_launches++;
    } else if (cfg->band_mode == 2) {
        band_straight_launch(st, o1, o2, np, c->band_opt.straight_w0, c->band_opt.w_min, spec);
        c->last_launches++;
    } else if ((s = band_predict(c, P, s1, o1, s2, o2, np, spec))) {
        return s;
    }
    // the largest pairs go to clusters only when their units fit in two waves of clusters
    if (c->ring.p) {
        const int slots = dp_cluster_grid(true, false, M_BAND, c->ring_grid) / kClusterBlocks;
        if ((counts[K_S16H] + 1) / 2 + counts[K_S32H] > 2u * (uint32_t)slots) bc[4].kind = bc[5].kind = 1;
    }

    // the full DP of a list: group kernels (with the s16 -> s32 redo list), whole blocks or clusters
    auto full_dp = [&](int k, const uint32_t *list, uint32_t *count_word, uint32_t *queue) -> pa_status {
        DpLaunch F = L;
        F.order = list;
        F.begin_ptr = ctr + 0;
        F.count_ptr = count_word;
        F.unit_counter = queue;
        F.rerun = 0;
        F.team = 0;                                   // whole blocks per pair
        F.rerun_list = (uint32_t *)(bc[k].kind ? c->rerun_long.p : c->rerun.p);
        F.rerun_count = counters + (bc[k].kind ? 6 : 4);
        if (bc[k].kind == 2) {
            F.G = 32;
            F.ring = cluster_ring(c);
            PA_CUDA(c, dp_cluster_launch(bc[k].lanes16, false, M_GLOBAL,
                                         dp_cluster_grid(bc[k].lanes16, false, M_GLOBAL, c->ring_grid), st, F, P));
            c->last_launches++;
        } else if (bc[k].kind == 1) {
            F.G = 32;
            dp_cta_launch(bc[k].lanes16, false, M_GLOBAL, c->ring_grid, st, F, P);
            c->last_launches++;
        } else {
            F.G = c->G[bc[k].klass];
            launch_class(c, bc[k].klass, M_GLOBAL, bc[k].lanes16, false, F, P);
        }
        return PA_OK;
    };
    // byte-compare classes: the full DP
    {
        DpLaunch F = L;
        F.order = (const uint32_t *)c->order.p;
        F.rerun_list = (uint32_t *)c->rerun.p;
        F.rerun_count = counters + 4;
        F.begin_ptr = (const uint32_t *)c->ranges.p + K_GEN;
        F.count_ptr = (const uint32_t *)c->counts.p + K_GEN;
        F.unit_counter = counters + 2;
        F.G = c->G[K_GEN];
        launch_class(c, K_GEN, M_GLOBAL, false, true, F, P);
        if (counts[K_GENL]) {
            F.begin_ptr = (const uint32_t *)c->ranges.p + K_GENL;
            F.count_ptr = (const uint32_t *)c->counts.p + K_GENL;
            F.unit_counter = counters + 11;
            F.G = 32;
            F.rerun_list = (uint32_t *)c->rerun_long.p;
            F.rerun_count = counters + 6;
            dp_cta_launch(false, true, M_GLOBAL, c->ring_grid, st, F, P);
            c->last_launches++;
        }
        if (counts[K_GENH]) {
            F.begin_ptr = (const uint32_t *)c->ranges.p + K_GENH;
            F.count_ptr = (const uint32_t *)c->counts.p + K_GENH;
            F.unit_counter = counters + 15;
            F.G = 32;
            F.ring = cluster_ring(c);
            F.rerun_list = (uint32_t *)c->rerun_long.p;
            F.rerun_count = counters + 6;
            PA_CUDA(c, dp_cluster_launch(false, true, M_GLOBAL, dp_cluster_grid(false, true, M_GLOBAL, c->ring_grid),
                                         st, F, P));
            c->last_launches++;
        }
    }

    uint32_t *cur[NB], *nxt[NB], *full[NB];
    for (int k = 0; k < NB; ++k) {
        cur[k] = (uint32_t *)c->band_list[k].p;
        nxt[k] = (uint32_t *)c->band_list[NB + k].p;
        full[k] = (uint32_t *)c->band_list[2 * NB + k].p;
    }
    uint32_t *tmp = (uint32_t *)c->band_list[3 * NB].p, *redo = (uint32_t *)c->band_list[3 * NB + 1].p;
    uint32_t ncur[NB], nfull[NB] = {};
    uint64_t short_pairs = 0;                         // group-class pairs already on the full DP
    for (int k = 0; k < NB; ++k) {
        const uint32_t cnt = counts[bc[k].klass];
        if (short_full && bc[k].kind == 0) {          // short pairs: no band rounds (launched above)
            ncur[k] = 0;
            short_pairs += cnt;
            continue;
        }
        ncur[k] = cnt;
        if (cnt)
            PA_CUDA(c, cudaMemcpyAsync(cur[k], (const uint32_t *)c->order.p + ranges[bc[k].klass], cnt * 4ull,
                                       cudaMemcpyDeviceToDevice, st));
    }
    uint64_t banded = 0, rounds = 0;
    uint8_t *code = (uint8_t *)c->band_code.p;
    uint32_t *bsum = (uint32_t *)c->band_bsum.p;
    const float full_frac = c->band_opt.full_frac;
    // One round of work class k over `list`: pairs to widen go to `next`, s16 results to redo in
    // s32 to `redo_out` (or nowhere).  A step has its own list, code, counter and stream slots,
    // so that two steps can run their banded DP at the same time: open() queues the windows and
    // their compaction, read() collects the counts (host wait), dp() launches the banded DP on
    // the step's stream and ring rows, close() compacts its outcome, collect() reads it.
    struct Step {
        int k = 0;
        const uint32_t *list = nullptr;
        uint32_t count = 0;
        bool rerun = false;
        uint32_t *next = nullptr, *n_next = nullptr, *redo_out = nullptr;
        uint32_t n_redo = 0;
        uint32_t *tmpl = nullptr;                    // the pairs that run the banded DP
        uint8_t *code = nullptr;                     // per list position
        uint32_t *cw = nullptr;                      // 5 device words: full, banded, queue, widen, redo
        unsigned long long *ws = nullptr;            // 2 device words: window cells, passes
        cudaStream_t stream = nullptr;
        Cell *ring = nullptr;
        size_t pin = 0;                              // its page-locked host words (32 bytes)
        uint32_t nb = 0;
        int team = 1;
    };
    const auto *opt = &c->band_opt;
    auto step_open = [&](Step &S, int r) -> pa_status {
        const BandClass &B = bc[S.k];
        PA_CUDA(c, cudaMemsetAsync(S.ws, 0, 16, st));
        band_windows_launch(st, o1, o2, S.list, S.count, spec, B.rows, r, full_frac, opt->team_full_frac,
                            c->team_max_n, (int2 *)c->band_win.p, S.code, S.ws);
        compact_launch(st, S.list, S.code, S.count, 2, bsum, full[S.k] + nfull[S.k], S.cw + 0);
        compact_launch(st, S.list, S.code, S.count, 0, bsum, S.tmpl, S.cw + 1);
        c->last_launches += 7;
        return PA_OK;
    };
    auto step_read = [&](Step &S) -> pa_status {
        const BandClass &B = bc[S.k];
        uint32_t *h = (uint32_t *)(c->pinned + S.pin);
        unsigned long long *w = (unsigned long long *)(c->pinned + S.pin + 8);
        PA_CUDA(c, cudaMemcpyAsync(h, S.cw, 8, cudaMemcpyDeviceToHost, st));
        PA_CUDA(c, cudaMemcpyAsync(w, S.ws, 16, cudaMemcpyDeviceToHost, st));
        PA_CUDA(c, cudaStreamSynchronize(st));
        nfull[S.k] += h[0];
        S.nb = h[1];
        // CTA mode: a team of warps per pair, at most half the passes a window keeps in flight
        // (a window of W columns keeps about W / rows passes going); more pairs with fewer
        // warps each beat fewer pairs with waiting warps.  Measured on 262,144 config-5 pairs:
        // for the 1,000-10,000-base class (mean window 1,600-2,500 columns) one warp per pair
        // was 1-2 % faster than two or four and eight was 1.30x slower; for the largest pairs
        // (mean window 8,900-14,800) eight warps were 1.16x faster than four, 1.83x than two
        const double mean_width = w[1] ? (double)w[0] / (double)w[1] : 0.0;
        S.team = mean_width >= 16.0 * B.rows ? 8 : mean_width >= 8.0 * B.rows ? 4 : mean_width >= 4.0 * B.rows ? 2 : 1;
        return PA_OK;
    };
    auto step_dp = [&](Step &S, int r) -> pa_status {
        if (S.nb == 0) return PA_OK;
        const BandClass &B = bc[S.k];
        DpLaunch LB = L;
        PA_CUDA(c, cudaMemsetAsync(S.cw + 2, 0, 4, S.stream));
        LB.team = S.team;
        LB.order = S.tmpl;
        LB.begin_ptr = ctr + 0;
        LB.count_ptr = S.cw + 1;
        LB.unit_counter = S.cw + 2;
        LB.band_code = S.code;
        LB.G = B.kind ? 32 : c->G[B.klass];
        LB.band_rows = B.rows;
        LB.band_round = r;
        LB.rerun = S.rerun ? 1 : 0;
        if (B.kind == 2) {
            LB.ring = cluster_ring(c);
            PA_CUDA(c, dp_cluster_launch(B.lanes16, false, M_BAND, dp_cluster_grid(B.lanes16, false, M_BAND, c->ring_grid),
                                         S.stream, LB, P));
        } else {
            LB.ring = S.ring;
            band_dp_launch(B.lanes16, B.kind == 1,
                           B.kind ? c->ring_grid : band_dp_occupancy(B.lanes16, false) * c->sm_count, S.stream, LB, P);
        }
        c->last_launches++;
        return PA_OK;
    };
    auto step_close = [&](Step &S) -> pa_status {
        if (S.nb == 0) return PA_OK;
        compact_launch(st, S.tmpl, S.code, S.nb, 1, bsum, S.next + *S.n_next, S.cw + 3);
        compact_launch(st, S.tmpl, S.code, S.nb, 3, bsum, S.redo_out ? S.redo_out : S.tmpl, S.cw + 4);
        c->last_launches += 6;
        return PA_OK;
    };
    auto step_collect = [&](Step &S) -> pa_status {
        if (S.nb == 0) return PA_OK;
        uint32_t *h = (uint32_t *)(c->pinned + S.pin + 24);
        PA_CUDA(c, cudaMemcpyAsync(h, S.cw + 3, 8, cudaMemcpyDeviceToHost, st));
        PA_CUDA(c, cudaStreamSynchronize(st));
        PA_CUDA(c, cudaGetLastError());
        *S.n_next += h[0];
        S.n_redo = S.redo_out ? h[1] : 0;
        banded += S.nb - h[0] - h[1];
        return PA_OK;
    };
    uint32_t *tmp2 = (uint32_t *)c->band_list[3 * NB + 2].p, *redo2 = (uint32_t *)c->band_list[3 * NB + 3].p;
    // slot 0: the call's stream and the block-mode ring rows; slot 1: the first side stream and
    // the team region of the ring (cluster steps use the cluster region in either slot)
    auto make_step = [&](int slot, int k, const uint32_t *list, uint32_t count, bool rerun, uint32_t *next,
                         uint32_t *n_next, uint32_t *redo_out, uint32_t code_off) {
        Step S;
        S.k = k; S.list = list; S.count = count; S.rerun = rerun;
        S.next = next; S.n_next = n_next; S.redo_out = redo_out;
        S.tmpl = slot ? tmp2 : tmp;
        S.code = code + code_off;
        S.cw = slot ? ctr + 22 : ctr + 1;
        S.ws = (unsigned long long *)(slot ? ctr + 28 : ctr + 36);
        S.stream = slot ? c->side : st;
        S.pin = slot ? 192 : 160;
        S.ring = slot ? team_ring(c) : (Cell *)c->ring.p;
        return S;
    };
    // one step alone, on slot 0
    auto band_step = [&](int k, const uint32_t *list, uint32_t count, int r, bool rerun, uint32_t *next,
                         uint32_t &n_next, uint32_t *redo_out, uint32_t &n_redo) -> pa_status {
        Step S = make_step(0, k, list, count, rerun, next, &n_next, redo_out, 0);
        pa_status e;
        if ((e = step_open(S, r)) || (e = step_read(S)) || (e = step_dp(S, r)) || (e = step_close(S)) ||
            (e = step_collect(S)))
            return e;
        n_redo = S.n_redo;
        return PA_OK;
    };
    // two steps whose banded DPs run at the same time (the long and the largest pairs)
    auto band_pair = [&](Step &A, Step &B, int r) -> pa_status {
        pa_status e;
        if ((e = step_open(A, r)) || (e = step_open(B, r)) || (e = step_read(A)) || (e = step_read(B))) return e;
        PA_CUDA(c, cudaEventRecord(c->ev_fork, st));
        PA_CUDA(c, cudaStreamWaitEvent(B.stream, c->ev_fork, 0));
        if ((e = step_dp(A, r)) || (e = step_dp(B, r))) return e;
        PA_CUDA(c, cudaEventRecord(c->ev_join, B.stream));
        PA_CUDA(c, cudaStreamWaitEvent(st, c->ev_join, 0));
        if ((e = step_close(A)) || (e = step_close(B)) || (e = step_collect(A)) || (e = step_collect(B))) return e;
        return PA_OK;
    };
    auto open_pairs = [&]() {
        uint32_t t = 0;
        for (int k = 0; k < NB; ++k) t += ncur[k];
        return t;
    };
    for (int r = 0; r < opt->max_rounds && open_pairs(); ++r) {
        ++rounds;
        uint32_t nn[NB] = {};
        uint32_t nredo[NB] = {}, none = 0;
        uint32_t *redo_of[NB] = {redo, nullptr, redo, nullptr, redo2, nullptr};
        // the s16 group class (caller-given bands only), then its s32 redo and the s32 groups
        if (ncur[0] && (s = band_step(0, cur[0], ncur[0], r, false, nxt[0], nn[0], redo, nredo[0]))) return s;
        if (nredo[0] && (s = band_step(1, redo, nredo[0], r, true, nxt[1], nn[1], nullptr, none))) return s;
        if (ncur[1] && (s = band_step(1, cur[1], ncur[1], r, false, nxt[1], nn[1], nullptr, none))) return s;
        // the s16 long and largest classes: both banded DPs at once when both have pairs
        if (ncur[2] && ncur[4]) {
            Step A = make_step(0, 2, cur[2], ncur[2], false, nxt[2], &nn[2], redo_of[2], 0);
            Step B = make_step(1, 4, cur[4], ncur[4], false, nxt[4], &nn[4], redo_of[4], ncur[2]);
            if ((s = band_pair(A, B, r))) return s;
            nredo[2] = A.n_redo;
            nredo[4] = B.n_redo;
        } else {
            for (int k16 : {2, 4})
                if (ncur[k16] &&
                    (s = band_step(k16, cur[k16], ncur[k16], r, false, nxt[k16], nn[k16], redo_of[k16], nredo[k16])))
                    return s;
        }
        for (int k16 : {2, 4}) {                      // their s32 redo, then the s32 classes
            if (nredo[k16] && (s = band_step(k16 + 1, redo_of[k16], nredo[k16], r, true, nxt[k16 + 1], nn[k16 + 1],
                                             nullptr, none)))
                return s;
            if (ncur[k16 + 1] && (s = band_step(k16 + 1, cur[k16 + 1], ncur[k16 + 1], r, false, nxt[k16 + 1],
                                                nn[k16 + 1], nullptr, none)))
                return s;
        }
        for (int k = 0; k < NB; ++k) {
            std::swap(cur[k], nxt[k]);
            ncur[k] = nn[k];
        }
    }
    L.team = 0;                                       // the full DP below: whole blocks per pair
    // still open after the last round: full DP
    uint32_t hc[NB];
    for (int k = 0; k < NB; ++k) {
        if (ncur[k])
            PA_CUDA(c, cudaMemcpyAsync(full[k] + nfull[k], cur[k], ncur[k] * 4ull, cudaMemcpyDeviceToDevice, st));
        nfull[k] += ncur[k];
        hc[k] = nfull[k];
    }
    bool any_full = false;
    for (int k = 0; k < NB; ++k) any_full |= nfull[k] != 0;
    if (any_full) {
        uint32_t *h_hc = (uint32_t *)(c->pinned + 256);
        std::memcpy(h_hc, hc, sizeof(hc));
        PA_CUDA(c, cudaMemcpyAsync(ctr + 6, h_hc, sizeof(hc), cudaMemcpyHostToDevice, st));
    }
    for (int k = 0; k < 2; ++k)                      // group classes
        if (nfull[k] && (s = full_dp(k, full[k], ctr + 6 + k, ctr + 16 + k))) return s;
    // Long classes: the full DP routed as the plain path routes it -- teams of 4 warps for pairs
    // of at most team_max_n rows, clusters for the largest pairs when their units fit in two
    // waves of clusters (else whole blocks take them first), whole blocks for the rest -- the
    // three kinds at the same time, on the call's two side streams.
    for (int l = 0; l < 2; ++l) {
        const int kl = 2 + l, kh = 4 + l;
        const uint32_t total = nfull[kl] + nfull[kh];
        if (!total) continue;
        const bool lanes16 = l == 0;
        uint32_t *all = cur[kl], *lc = cur[kh], *lb = nxt[kl], *lt = nxt[kh];   // free after the rounds
        // the largest pairs first: the cluster-class list, then the block-class list
        if (nfull[kh]) PA_CUDA(c, cudaMemcpyAsync(all, full[kh], nfull[kh] * 4ull, cudaMemcpyDeviceToDevice, st));
        if (nfull[kl])
            PA_CUDA(c, cudaMemcpyAsync(all + nfull[kh], full[kl], nfull[kl] * 4ull, cudaMemcpyDeviceToDevice, st));
        uint32_t *cnt = ctr + 40 + 3 * l, *queue = ctr + 48 + 3 * l;
        size_code_launch(st, o1, o2, all, total, c->team_max_n, c->huge_cells, c->huge_min_n, code);
        compact_launch(st, all, code, total, 2, bsum, lc, cnt + 0);
        compact_launch(st, all, code, total, 1, bsum, lb, cnt + 1);
        compact_launch(st, all, code, total, 0, bsum, lt, cnt + 2);
        c->last_launches += 10;
        uint32_t *h = (uint32_t *)(c->pinned + 224);
        PA_CUDA(c, cudaMemcpyAsync(h, cnt, 12, cudaMemcpyDeviceToHost, st));
        PA_CUDA(c, cudaStreamSynchronize(st));
        DpLaunch F = L;
        F.begin_ptr = ctr + 0;
        F.rerun = 0;
        F.team = 0;
        F.G = 32;
        F.rerun_list = (uint32_t *)c->rerun_long.p;
        F.rerun_count = counters + 6;
        const int slots = dp_cluster_grid(lanes16, false, M_GLOBAL, c->ring_grid) / kClusterBlocks;
        const uint32_t cl_units = lanes16 ? (h[0] + 1) / 2 : h[0];
        const bool clusters = h[0] > 0 && slots > 0 && cl_units <= 2u * (uint32_t)slots;
        PA_CUDA(c, cudaEventRecord(c->ev_fork, st));
        if (clusters) {
            PA_CUDA(c, cudaStreamWaitEvent(c->side, c->ev_fork, 0));
            DpLaunch FC = F;
            FC.order = lc;
            FC.count_ptr = cnt + 0;
            FC.unit_counter = queue + 0;
            FC.ring = cluster_ring(c);
            PA_CUDA(c, dp_cluster_launch(lanes16, false, M_GLOBAL,
                                         dp_cluster_grid(lanes16, false, M_GLOBAL, c->ring_grid), c->side, FC, P));
            PA_CUDA(c, cudaEventRecord(c->ev_join, c->side));
            c->last_launches++;
        }
        if (h[2]) {
            PA_CUDA(c, cudaStreamWaitEvent(c->side2, c->ev_fork, 0));
            DpLaunch FT = F;
            FT.order = lt;
            FT.count_ptr = cnt + 2;
            FT.unit_counter = queue + 2;
            FT.ring = team_ring(c);
            dp_team_launch(lanes16, false, M_GLOBAL, c->ring_grid, c->side2, FT, P);
            PA_CUDA(c, cudaEventRecord(c->ev_join2, c->side2));
            c->last_launches++;
        }
        if (h[1] || (h[0] && !clusters)) {
            DpLaunch FB = F;
            FB.order = lb;
            FB.count_ptr = cnt + 1;
            FB.unit_counter = queue + 1;
            if (h[0] && !clusters) {                  // the largest pairs ahead of the block list
                FB.lead_order = lc;
                FB.lead_begin_ptr = ctr + 0;
                FB.lead_count_ptr = cnt + 0;
            }
            dp_cta_launch(lanes16, false, M_GLOBAL, c->ring_grid, st, FB, P);
            c->last_launches++;
        }
        if (clusters) PA_CUDA(c, cudaStreamWaitEvent(st, c->ev_join, 0));
        if (h[2]) PA_CUDA(c, cudaStreamWaitEvent(st, c->ev_join2, 0));
    }
    if (nfull[0] || (short_full && counts[K_S16])) {  // s16 group results that failed their check
        DpLaunch F = L;
        F.order = (const uint32_t *)c->rerun.p;
        F.begin_ptr = counters + 5;
        F.count_ptr = counters + 4;
        F.unit_counter = counters + 3;
        F.rerun = 1;
        F.G = c->G[K_S32];
        launch_class(c, K_S32, M_GLOBAL, false, false, F, P);
    }
    if (nfull[2] || nfull[4]) {                       // the same for s16 long and largest pairs
        DpLaunch F = L;
        F.order = (const uint32_t *)c->rerun_long.p;
        F.begin_ptr = counters + 5;
        F.count_ptr = counters + 6;
        F.unit_counter = counters + 12;
        F.rerun = 1;
        F.G = 32;
        dp_cta_launch(false, false, M_GLOBAL, c->ring_grid, st, F, P);
        c->last_launches++;
    }
    mark_full_launch(st, out, np);
    c->last_launches++;
    PA_CUDA(c, cudaEventRecord(c->ev1, st));
    if (!sync_at_end) {
        // like the plain device entry without stats: the call returns once the work is queued,
        // and errors found on the device are in the pairs' results
        PA_CUDA(c, cudaGetLastError());
        return PA_OK;
    }
    PA_CUDA(c, cudaStreamSynchronize(st));
    PA_CUDA(c, cudaGetLastError());
    unsigned long long cells = 0;
    PA_CUDA(c, cudaMemcpy(&cells, ctr + 32, 8, cudaMemcpyDeviceToHost));
    pa_stats local;
    pa_stats *st_out = stats ? stats : &local;
    std::memset(st_out, 0, sizeof(*st_out));
    s = read_stats(c, st_out);
    st_out->pairs = np;
    st_out->kernel_launches = c->last_launches;
    st_out->dp_ms = st_out->device_ms;
    st_out->pairs_banded = banded;
    st_out->pairs_full_dp = counts[K_GEN] + counts[K_GENL] + counts[K_GENH];
    st_out->pairs_full_dp += short_pairs;
    for (int k = 0; k < NB; ++k) st_out->pairs_full_dp += nfull[k];
    st_out->band_cells = cells;
    st_out->band_rounds = rounds;
    return s;
}

// Queue the copies of the call's counters into page-locked host words (read_stats with
// staged = true reads them after the caller's wait on `st`).
constexpr size_t kPinStats = 512;      // PrepStats, then 16 counter words
void stage_stats(pa_ctx *c, cudaStream_t st)
{
    static_assert(kPinStats + sizeof(PrepStats) + 64 <= kPinnedBytes, "page-locked words");
    cudaMemcpyAsync(c->pinned + kPinStats, c->pstats.p, sizeof(PrepStats), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(c->pinned + kPinStats + sizeof(PrepStats), c->counters.p, 64, cudaMemcpyDeviceToHost, st);
}

// Counters of the finished call (after a sync): class sizes, reruns, error bits.
pa_status read_stats(pa_ctx *c, pa_stats *stats, bool staged)
{
    PrepStats ps;
    uint32_t ctr[16];
    if (staged) {
        std::memcpy(&ps, c->pinned + kPinStats, sizeof(ps));
        std::memcpy(ctr, c->pinned + kPinStats + sizeof(PrepStats), sizeof(ctr));
    } else {
        PA_CUDA(c, cudaMemcpy(&ps, c->pstats.p, sizeof(ps), cudaMemcpyDeviceToHost));
        PA_CUDA(c, cudaMemcpy(ctr, c->counters.p, sizeof(ctr), cudaMemcpyDeviceToHost));
    }
    if (stats) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev0, c->ev1);
        stats->device_ms = ms;
        if (cudaEventElapsedTime(&ms, c->ev_dp0, c->ev_dp1) == cudaSuccess) stats->dp_ms = ms;
        cudaGetLastError();
        const uint64_t rr = (uint64_t)ctr[4] + ctr[6];
        stats->cells = ps.cells;
        stats->pairs_s16 = ps.n_class[K_S16] + ps.n_class[K_S16L] + ps.n_class[K_S16H] + ps.n_class[K_S16M] - rr;
        stats->pairs_s32 = ps.n_class[K_S32] + ps.n_class[K_S32L] + ps.n_class[K_S32H] + ps.n_class[K_S32M] + rr;
        stats->pairs_general = ps.n_class[K_GEN] + ps.n_class[K_GENL] + ps.n_class[K_GENH] + ps.n_class[K_GENM];
        stats->pairs_trivial = ps.n_class[K_NONE];
        stats->pairs_rerun = rr;
    }
    if (ps.bad_offsets)
        return fail(c, PA_ERR_INVALID_ARGUMENT,
                    "offsets decrease or run past seq1_bytes / seq2_bytes; no pair was aligned");
    if (ctr[8]) return fail(c, PA_ERR_TIMEOUT, "a CTA-mode progress wait ran out");
    if (ps.overflow) return fail(c, PA_ERR_OVERFLOW, "scores of some pairs could exceed int32");
    if (ps.invalid) return fail(c, PA_ERR_INVALID_ARGUMENT, "a sequence holds a symbol outside the substitution matrix");
    return PA_OK;
}

pa_status run_device(pa_ctx *c, const pa_config *cfg, const uint8_t *s1, const uint64_t *o1, uint64_t b1,
                     const uint8_t *s2, const uint64_t *o2, uint64_t b2, uint64_t n_pairs, pa_result *out,
                     pa_stats *stats, bool sync_for_stats)
{
    if (cfg && cfg->band_mode)
        return run_band(c, cfg, s1, o1, b1, s2, o2, b2, n_pairs, out, nullptr, stats, sync_for_stats || stats);
    apply_tuning(c, cfg, n_pairs, b1, b2);
    pa_status s = n_pairs ? ensure_ring(c, c->want_ring_m) : PA_OK;
    if (s) return s;
    DpParams P;
    ClassCfg C;
    s = check_config(c, cfg, P, C);
    if (s) return s;
    // local pairs of the s16x2 class that the short-pair kernel takes (launch_class) never go
    // back to dp_kernel (no s32 redo in local mode): the kernel builds its own column tables
    if (P.local && c->variant[K_S16] >= kShortVariant && dp_short_supports(c->G[K_S16])) C.qtab_s16 = 0;
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
        for (int k = 0; k < 3; ++k) { key.G[k] = c->G[k]; key.variant[k] = c->variant[k]; }
        key.wait_limit = c->wait_limit;
        auto it = c->graphs.find(key);
        if (it == c->graphs.end()) {
            if (c->graphs.size() >= kMaxGraphs) {
                // a caller that rotates buffers would otherwise keep one graph per buffer set
                auto lru = c->graphs.begin();
                for (auto g = c->graphs.begin(); g != c->graphs.end(); ++g)
                    if (g->second.last_use < lru->second.last_use) lru = g;
                cudaGraphExecDestroy(lru->second.exec);
                c->graphs.erase(lru);
            }
            cudaGraph_t g;
            PA_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            pa_status es = enqueue(c, cfg, P, C, s1, o1, b1, s2, o2, b2, out, n_pairs);
            cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
            if (es) return es;
            if (ce != cudaSuccess) return fail(c, PA_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(ce));
            cudaGraphExec_t ex;
            ce = cudaGraphInstantiate(&ex, g, 0);
            cudaGraphDestroy(g);
            if (ce != cudaSuccess) return fail(c, PA_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(ce));
            it = c->graphs.emplace(key, GraphEntry{ex, 0}).first;
        } else {
            c->last_launches = 6 + 3 + (P.local ? 0 : 1) + (c->ring.p ? (P.local ? 7 : 8) + (C.team_max_n > 0 ? 3 : 0) : 0);
        }
        it->second.last_use = ++c->graph_clock;
        PA_CUDA(c, cudaGraphLaunch(it->second.exec, c->stream));
    } else {
        if ((s = enqueue(c, cfg, P, C, s1, o1, b1, s2, o2, b2, out, n_pairs))) return s;
    }
    PA_CUDA(c, cudaEventRecord(c->ev1, c->stream));
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->pairs = n_pairs;
        stats->kernel_launches = c->last_launches;
        if (sync_for_stats) {
            PA_CUDA(c, cudaEventSynchronize(c->ev1));
            if ((s = read_stats(c, stats))) return s;
        }
    }
    PA_CUDA(c, cudaGetLastError());
    return PA_OK;
}

// ---------------------------------------------------------------------------
// roofline microkernel: the cell-update instruction mix of dp_kernel on
// registers only (no memory, no shuffles), timed over the whole chip.  TRACK adds
// what local scoring needs on top of the recurrence: the column maximum of the
// thread's rows (three-operand max tree) and the test for a strict improvement.
// ---------------------------------------------------------------------------
template <class V, bool TRACK = false>
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
    uint32_t best = V::splat(2048), moved = 0;
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
        if (TRACK) {
            const uint32_t nb = V::max2(best, tree_max<V, R>(H));
            moved += (nb ^ best) != 0u;
            best = nb;
        }
        diag0 = H[R - 1];
        up = Ed;
        ta = (ta << 8) | (ta >> 24);
        tb = (tb >> 8) | (tb << 24);
    }
    uint32_t acc = up ^ best ^ moved;
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
        cudaEventCreate(&c->ev_dp0) != cudaSuccess || cudaEventCreate(&c->ev_dp1) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->side2, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_join2, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaHostAlloc((void **)&c->pinned, kPinnedBytes, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        pa_destroy(c);
        return PA_ERR_CUDA;
    }
    // defaults measured on GB300 (262,144 pairs of 64..512 bp): local s16x2 is fastest with
    // variant 7, global with variant 4; 8 lanes per group
    c->tuning = pa_tuning{};
    c->tuning.variant_s16[0] = c->tuning.variant_s16[1] = kDefaultShortVariant;
    c->tuning.variant_s32[0] = 0;
    c->tuning.variant_s32[1] = 4;                 // group sizes 0: the built-in rule
    if (c->opt.group_threads) {
        int g = c->opt.group_threads;
        if (g < 1 || g > 32 || (g & (g - 1))) { pa_destroy(c); return PA_ERR_INVALID_ARGUMENT; }
        for (int k = 0; k < 3; ++k) c->G[k] = g;
        c->fixed_G = true;
    }
    if (c->opt.rows_per_thread && c->opt.rows_per_thread != kR) { pa_destroy(c); return PA_ERR_UNSUPPORTED; }
    if (c->opt.kernel_variant >= 0 && c->opt.kernel_variant < kVariants) {
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
    drop_graphs(c);
    DevBuf *bufs[] = {&c->keys, &c->order, &c->hist, &c->starts, &c->cursor, &c->sums, &c->ranges,
                      &c->counts, &c->qtab, &c->boundary, &c->slots, &c->rerun, &c->counters, &c->pstats,
                      &c->in_seq1, &c->in_off1, &c->in_seq2, &c->in_off2, &c->in_out,
                      &c->band_spec, &c->band_win, &c->band_code, &c->band_bsum, &c->band_ctr, &c->band_in,
                      &c->mlp_feat, &c->mlp_x, &c->mlp_h1, &c->mlp_h2, &c->mlp_out,
                      &c->ring, &c->rerun_long, &c->mat_rank, &c->mat_scores,
                      &c->io_tab, &c->io_ctr, &c->in_words1, &c->in_words2,
                      &c->tb_dir, &c->tb_dir_off, &c->tb_aln, &c->tb_ops};
    for (DevBuf *b : bufs)
        if (b->p) cudaFree(b->p);
    for (DevBuf &b : c->band_list)
        if (b.p) cudaFree(b.p);
    for (DevBuf &b : c->mlp_w)
        if (b.p) cudaFree(b.p);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->ev2) cudaEventDestroy(c->ev2);
    if (c->ev3) cudaEventDestroy(c->ev3);
    if (c->ev_dp0) cudaEventDestroy(c->ev_dp0);
    if (c->ev_dp1) cudaEventDestroy(c->ev_dp1);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->side2) cudaStreamDestroy(c->side2);
    if (c->ev_join2) cudaEventDestroy(c->ev_join2);
    if (c->pinned) cudaFreeHost(c->pinned);
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
    // sequence lengths are on the device: CTA mode covers sequence1 up to the default ring
    ctx->want_ring_m = std::max<int64_t>(ctx->ring_m, kDefaultRingM);
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

static pa_status align_host(pa_ctx *ctx, const pa_config *config, const uint8_t *seq1, const uint64_t *off1,
                            const uint8_t *seq2, const uint64_t *off2, uint64_t n_pairs, pa_result *out,
                            pa_stats *stats, const int32_t *bands, const uint32_t *words1 = nullptr,
                            const uint32_t *words2 = nullptr);

pa_status pa_align_batch(pa_ctx *ctx, const pa_config *config, const uint8_t *seq1, const uint64_t *off1,
                         const uint8_t *seq2, const uint64_t *off2, uint64_t n_pairs, pa_result *out,
                         pa_stats *stats)
{
    return align_host(ctx, config, seq1, off1, seq2, off2, n_pairs, out, stats, nullptr);
}

pa_status pa_align_batch_banded(pa_ctx *ctx, const pa_config *config, const uint8_t *seq1, const uint64_t *off1,
                                const uint8_t *seq2, const uint64_t *off2, uint64_t n_pairs, const int32_t *bands,
                                pa_result *out, pa_stats *stats)
{
    if (!ctx) return PA_ERR_INVALID_ARGUMENT;
    if (n_pairs && !bands) return fail(ctx, PA_ERR_INVALID_ARGUMENT, "bands is null");
    if (!config) return fail(ctx, PA_ERR_INVALID_ARGUMENT, "config is null");
    pa_config cfg = *config;
    cfg.band_mode = 1;
    return align_host(ctx, &cfg, seq1, off1, seq2, off2, n_pairs, out, stats, bands);
}

pa_status pa_set_cta_threshold(pa_ctx *ctx, uint64_t cells)
{
    if (!ctx) return PA_ERR_INVALID_ARGUMENT;
    ctx->long_cells = cells > (uint64_t)INT64_MAX ? INT64_MAX : (int64_t)std::max<uint64_t>(cells, 1);
    drop_graphs(ctx);   // the classifier's rule changed
    return PA_OK;
}

pa_status pa_get_graph_count(const pa_ctx *ctx, uint32_t *out)
{
    if (!ctx || !out) return PA_ERR_INVALID_ARGUMENT;
    *out = (uint32_t)ctx->graphs.size();
    return PA_OK;
}

pa_status pa_set_wait_limit(pa_ctx *ctx, uint32_t polls)
{
    if (!ctx) return PA_ERR_INVALID_ARGUMENT;
    ctx->wait_limit = polls;
    return PA_OK;
}

pa_status pa_set_team_threshold(pa_ctx *ctx, uint32_t max_rows)
{
    if (!ctx) return PA_ERR_INVALID_ARGUMENT;
    ctx->team_max_n = (int32_t)std::min<uint32_t>(max_rows, 1u << 30);
    drop_graphs(ctx);
    return PA_OK;
}

pa_status pa_set_cluster_threshold(pa_ctx *ctx, uint64_t cells, uint32_t min_rows)
{
    if (!ctx) return PA_ERR_INVALID_ARGUMENT;
    ctx->huge_cells = cells > (uint64_t)INT64_MAX ? INT64_MAX : (int64_t)std::max<uint64_t>(cells, 1);
    ctx->huge_min_n = (int32_t)std::min<uint32_t>(std::max<uint32_t>(min_rows, 1), 1u << 30);
    drop_graphs(ctx);
    return PA_OK;
}

// The reference keeps the matrix as one flat array indexed by rank(sequence1 symbol) * dim +
// rank(sequence2 symbol) (score_model/score_model_matrix.hpp:53-63; the ranks come from its
// alphabet conversion, configuration/score_model_matrix.hpp:203-222).  Here the rank map is
// a byte -> int8 table, so any byte alphabet of up to 32 symbols works.
pa_status pa_set_substitution_matrix(pa_ctx *ctx, const uint8_t *symbols, uint32_t dim, const int32_t *scores)
{
    if (!ctx) return PA_ERR_INVALID_ARGUMENT;
    if (!symbols || !scores) return fail(ctx, PA_ERR_INVALID_ARGUMENT, "null matrix");
    if (dim < 1 || dim > 32) return fail(ctx, PA_ERR_INVALID_ARGUMENT, "matrix dim must be 1..32");
    int8_t rank[256];
    std::memset(rank, -1, sizeof(rank));
    for (uint32_t r = 0; r < dim; ++r) {
        if (rank[symbols[r]] >= 0) return fail(ctx, PA_ERR_INVALID_ARGUMENT, "matrix symbols must be distinct");
        rank[symbols[r]] = (int8_t)r;
    }
    int32_t hi = INT32_MIN, lo = INT32_MAX;
    for (uint32_t k = 0; k < dim * dim; ++k) {
        if (scores[k] > (1 << 20) || scores[k] < -(1 << 20))
            return fail(ctx, PA_ERR_INVALID_ARGUMENT, "matrix scores must lie in [-2^20, 2^20]");
        hi = std::max(hi, scores[k]);
        lo = std::min(lo, scores[k]);
    }
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, PA_ERR_CUDA, "cudaSetDevice");
    PA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));      // no call in flight reads the old matrix
    PA_CUDA(ctx, cudaStreamSynchronize(ctx->side));
    pa_status s;
    if ((s = ensure(ctx, ctx->mat_rank, 256)) || (s = ensure(ctx, ctx->mat_scores, 32 * 32 * 4))) return s;
    PA_CUDA(ctx, cudaMemcpy(ctx->mat_rank.p, rank, 256, cudaMemcpyHostToDevice));
    PA_CUDA(ctx, cudaMemcpy(ctx->mat_scores.p, scores, (size_t)dim * dim * 4, cudaMemcpyHostToDevice));
    ctx->mat_dim = (int32_t)dim;
    ctx->mat_max = hi;
    ctx->mat_min = lo;
    drop_graphs(ctx);   // they hold the old dim
    return PA_OK;
}

pa_status pa_set_band_options(pa_ctx *ctx, const pa_band_options *o)
{
    if (!ctx || !o) return PA_ERR_INVALID_ARGUMENT;
    if (!(o->margin > 0.f) || o->w_min < 1 || o->straight_w0 < 1 || !(o->full_frac > 0.f) || o->max_rounds < 0 ||
        o->max_rounds > 30 || !(o->team_full_frac >= 0.f))
        return fail(ctx, PA_ERR_INVALID_ARGUMENT, "band options out of range");
    ctx->band_opt = *o;
    return PA_OK;
}

pa_status pa_get_band_options(const pa_ctx *ctx, pa_band_options *out)
{
    if (!ctx || !out) return PA_ERR_INVALID_ARGUMENT;
    *out = ctx->band_opt;
    return PA_OK;
}

pa_status pa_set_band_model(pa_ctx *ctx, const float *w1, const float *b1, const float *w2, const float *b2,
                            const float *w3, const float *b3)
{
    if (!ctx) return PA_ERR_INVALID_ARGUMENT;
    if (!w1 || !b1 || !w2 || !b2 || !w3 || !b3) return fail(ctx, PA_ERR_INVALID_ARGUMENT, "null weight");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, PA_ERR_CUDA, "cudaSetDevice");
    const float *src[6] = {w1, b1, w2, b2, w3, b3};
    const int rows[6] = {144, 1, 256, 1, 256, 1}, cols[6] = {256, 256, 256, 256, 16, 16};
    void *tmp = nullptr;
    if (cudaMalloc(&tmp, 256 * 256 * 4) != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, PA_ERR_OUT_OF_MEMORY, "band model upload");
    }
    pa_status s = PA_OK;
    for (int k = 0; k < 6 && !s; ++k) {
        const size_t n = (size_t)rows[k] * cols[k];
        const bool weight = (k % 2) == 0;
        if ((s = ensure(ctx, ctx->mlp_w[k], n * (weight ? 2 : 4)))) break;
        bool ok;
        if (weight)          // BF16 copy on the device, rounded as the training kernels round
            ok = cudaMemcpy(tmp, src[k], n * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
                 pa_mlp_to_bf16((const float *)tmp, rows[k], cols[k], cols[k], ctx->mlp_w[k].p, nullptr) == PA_OK &&
                 cudaDeviceSynchronize() == cudaSuccess;
        else
            ok = cudaMemcpy(ctx->mlp_w[k].p, src[k], n * 4, cudaMemcpyHostToDevice) == cudaSuccess;
        if (!ok) s = fail(ctx, PA_ERR_CUDA, "band model upload");
    }
    cudaFree(tmp);
    if (s) return s;
    ctx->has_model = true;
    return PA_OK;
}

// Host buffers in, host results out.  With words1 / words2 the sequences are 2-bit packed host
// streams (offsets count bases): the packed words are copied and unpacked on the device.
static pa_status align_host(pa_ctx *ctx, const pa_config *config, const uint8_t *seq1, const uint64_t *off1,
                            const uint8_t *seq2, const uint64_t *off2, uint64_t n_pairs, pa_result *out,
                            pa_stats *stats, const int32_t *bands, const uint32_t *words1,
                            const uint32_t *words2)
{
    if (!ctx) return PA_ERR_INVALID_ARGUMENT;
    const bool packed = words1 != nullptr;
    if (n_pairs == 0) {
        DpParams P; ClassCfg C;
        pa_status s = check_config(ctx, config, P, C);
        if (stats) std::memset(stats, 0, sizeof(*stats));
        return s;
    }
    if ((packed ? (!words1 || !words2) : (!seq1 || !seq2)) || !off1 || !off2 || !out)
        return fail(ctx, PA_ERR_INVALID_ARGUMENT, "null buffer");
    if (off1[n_pairs] < off1[0] || off2[n_pairs] < off2[0])
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
    // the two sequence sets go over two copy engines at once (side stream joins before the DP)
    PA_CUDA(ctx, cudaEventRecord(ctx->ev_fork, st));
    PA_CUDA(ctx, cudaStreamWaitEvent(ctx->side, ctx->ev_fork, 0));
    if (packed) {
        // words [base / 16, (base + bytes + 15) / 16) of each stream, unpacked into the staging bytes
        const uint64_t q1 = base1 >> 4, nw1 = ((base1 + b1 + 15) >> 4) - q1;
        const uint64_t q2 = base2 >> 4, nw2 = ((base2 + b2 + 15) >> 4) - q2;
        if ((s = ensure(ctx, ctx->in_words1, nw1 * 4))) return s;
        if ((s = ensure(ctx, ctx->in_words2, nw2 * 4))) return s;
        if (b1) {
            PA_CUDA(ctx, cudaMemcpyAsync(ctx->in_words1.p, words1 + q1, nw1 * 4, cudaMemcpyHostToDevice, ctx->side));
            unpack_2bit_launch((const uint32_t *)ctx->in_words1.p, base1 & 15, b1, (uint8_t *)ctx->in_seq1.p,
                               ctx->sm_count, ctx->side);
        }
        if (b2) {
            PA_CUDA(ctx, cudaMemcpyAsync(ctx->in_words2.p, words2 + q2, nw2 * 4, cudaMemcpyHostToDevice, st));
            unpack_2bit_launch((const uint32_t *)ctx->in_words2.p, base2 & 15, b2, (uint8_t *)ctx->in_seq2.p,
                               ctx->sm_count, st);
        }
    } else {
        if (b1) PA_CUDA(ctx, cudaMemcpyAsync(ctx->in_seq1.p, seq1 + base1, b1, cudaMemcpyHostToDevice, ctx->side));
        if (b2) PA_CUDA(ctx, cudaMemcpyAsync(ctx->in_seq2.p, seq2 + base2, b2, cudaMemcpyHostToDevice, st));
    }
    PA_CUDA(ctx, cudaMemcpyAsync(ctx->in_off1.p, h1, (n_pairs + 1) * 8, cudaMemcpyHostToDevice, ctx->side));
    PA_CUDA(ctx, cudaMemcpyAsync(ctx->in_off2.p, h2, (n_pairs + 1) * 8, cudaMemcpyHostToDevice, st));
    PA_CUDA(ctx, cudaEventRecord(ctx->ev_join, ctx->side));
    PA_CUDA(ctx, cudaStreamWaitEvent(st, ctx->ev_join, 0));
    // the offsets' check and the longest block-mode sequence1 (ring-row size), while the copies
    // above run; nothing is launched on the copied bytes before the check passes
    int64_t long_m = 0;
    for (uint64_t k = 0; k < n_pairs; ++k) {
        if (off1[k + 1] < off1[k] || off2[k + 1] < off2[k]) {
            PA_CUDA(ctx, cudaStreamSynchronize(st));
            return fail(ctx, PA_ERR_INVALID_ARGUMENT, "offsets must be non-decreasing");
        }
        const int64_t m = (int64_t)(off1[k + 1] - off1[k]), n = (int64_t)(off2[k + 1] - off2[k]);
        if (m * n >= ctx->long_cells) long_m = std::max(long_m, m);
    }
    ctx->want_ring_m = long_m;      // exact: the ring rows hold the longest CTA-mode sequence1
    if (config && config->band_mode) {
        s = run_band(ctx, config, (const uint8_t *)ctx->in_seq1.p, (const uint64_t *)ctx->in_off1.p, b1,
                     (const uint8_t *)ctx->in_seq2.p, (const uint64_t *)ctx->in_off2.p, b2, n_pairs,
                     (pa_result *)ctx->in_out.p, bands, stats, true);
        if (s && s != PA_ERR_OVERFLOW) return s;
        PA_CUDA(ctx, cudaMemcpyAsync(out, ctx->in_out.p, n_pairs * sizeof(pa_result), cudaMemcpyDeviceToHost, st));
        PA_CUDA(ctx, cudaStreamSynchronize(st));
        return s;
    }
    s = run_device(ctx, config, (const uint8_t *)ctx->in_seq1.p, (const uint64_t *)ctx->in_off1.p, b1,
                   (const uint8_t *)ctx->in_seq2.p, (const uint64_t *)ctx->in_off2.p, b2, n_pairs,
                   (pa_result *)ctx->in_out.p, stats, false);
    if (s) return s;
    PA_CUDA(ctx, cudaMemcpyAsync(out, ctx->in_out.p, n_pairs * sizeof(pa_result), cudaMemcpyDeviceToHost, st));
    stage_stats(ctx, st);
    PA_CUDA(ctx, cudaStreamSynchronize(st));
    return read_stats(ctx, stats, true);
}

// Traceback: inputs staged like pa_align_batch; pairs in chunks whose direction words fit
// kTbBudgetWords; one kernel launch per chunk.
constexpr uint64_t kTbBudgetWords = 1ull << 30;      // 4 GiB of direction words per chunk

pa_status pa_traceback_batch(pa_ctx *ctx, const pa_config *config, const uint8_t *seq1, const uint64_t *off1,
                             const uint8_t *seq2, const uint64_t *off2, uint64_t n_pairs, pa_result *out,
                             pa_alignment *alignments, uint8_t *ops, pa_stats *stats)
{
    if (!ctx) return PA_ERR_INVALID_ARGUMENT;
    DpParams P;
    ClassCfg C;
    pa_status s = check_config(ctx, config, P, C);
    if (s) return s;
    if (stats) std::memset(stats, 0, sizeof(*stats));
    if (n_pairs == 0) return PA_OK;
    if (!seq1 || !off1 || !seq2 || !off2 || !out || !alignments || !ops)
        return fail(ctx, PA_ERR_INVALID_ARGUMENT, "null buffer");
    if (n_pairs >= (1ull << 31)) return fail(ctx, PA_ERR_TOO_LARGE, "n_pairs must be < 2^31");
    const bool use_matrix = C.rank_map != nullptr;
    std::vector<uint64_t> words(n_pairs);
    uint64_t cells = 0;
    for (uint64_t k = 0; k < n_pairs; ++k) {
        if (off1[k + 1] < off1[k] || off2[k + 1] < off2[k])
            return fail(ctx, PA_ERR_INVALID_ARGUMENT, "offsets must be non-decreasing");
        const int64_t m = (int64_t)(off1[k + 1] - off1[k]), n = (int64_t)(off2[k + 1] - off2[k]);
        if (m >= (1ll << 30) || n >= (1ll << 30)) return fail(ctx, PA_ERR_TOO_LARGE, "sequence longer than 2^30");
        const int64_t a = std::abs((int64_t)P.match), b = std::abs((int64_t)P.mismatch);
        const int64_t o = -(int64_t)P.gap_open, e = -(int64_t)P.gap_ext;
        if ((a + b) * std::min(m, n) + (o + e) * (m + n + 2) + 2 * o >= (1ll << 30))
            return fail(ctx, PA_ERR_OVERFLOW, "scores of some pairs could exceed int32");
        words[k] = (m && n) ? (uint64_t)((n + kTracebackPassRows - 1) / kTracebackPassRows) * (m + 31) * 32 : 0;
        if (words[k] > kTbBudgetWords) return fail(ctx, PA_ERR_TOO_LARGE, "a pair needs more than 4 GiB of directions");
        cells += (uint64_t)(m * n);
    }
    if (use_matrix) {                                  // every symbol needs a rank
        int8_t rank[256];
        PA_CUDA(ctx, cudaMemcpy(rank, ctx->mat_rank.p, 256, cudaMemcpyDeviceToHost));
        for (uint64_t x = off1[0]; x < off1[n_pairs]; ++x)
            if (rank[seq1[x]] < 0) return fail(ctx, PA_ERR_INVALID_ARGUMENT, "a symbol outside the substitution matrix");
        for (uint64_t x = off2[0]; x < off2[n_pairs]; ++x)
            if (rank[seq2[x]] < 0) return fail(ctx, PA_ERR_INVALID_ARGUMENT, "a symbol outside the substitution matrix");
    }
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, PA_ERR_CUDA, "cudaSetDevice");
    const uint64_t base1 = off1[0], base2 = off2[0];
    const uint64_t b1 = off1[n_pairs] - base1, b2 = off2[n_pairs] - base2;
    if ((s = ensure(ctx, ctx->in_seq1, b1)) || (s = ensure(ctx, ctx->in_seq2, b2)) ||
        (s = ensure(ctx, ctx->in_off1, (n_pairs + 1) * 8)) || (s = ensure(ctx, ctx->in_off2, (n_pairs + 1) * 8)) ||
        (s = ensure(ctx, ctx->in_out, n_pairs * sizeof(pa_result))) ||
        (s = ensure(ctx, ctx->boundary, (b1 + n_pairs) * sizeof(Cell))) ||
        (s = ensure(ctx, ctx->tb_aln, n_pairs * sizeof(pa_alignment))) || (s = ensure(ctx, ctx->tb_ops, b1 + b2)) ||
        (s = ensure(ctx, ctx->tb_dir_off, n_pairs * 8)))
        return s;
    std::vector<uint64_t> r1(off1, off1 + n_pairs + 1), r2(off2, off2 + n_pairs + 1);
    for (auto &v : r1) v -= base1;
    for (auto &v : r2) v -= base2;
    cudaStream_t st = ctx->stream;
    PA_CUDA(ctx, cudaEventRecord(ctx->ev0, st));
    if (b1) PA_CUDA(ctx, cudaMemcpyAsync(ctx->in_seq1.p, seq1 + base1, b1, cudaMemcpyHostToDevice, st));
    if (b2) PA_CUDA(ctx, cudaMemcpyAsync(ctx->in_seq2.p, seq2 + base2, b2, cudaMemcpyHostToDevice, st));
    PA_CUDA(ctx, cudaMemcpyAsync(ctx->in_off1.p, r1.data(), (n_pairs + 1) * 8, cudaMemcpyHostToDevice, st));
    PA_CUDA(ctx, cudaMemcpyAsync(ctx->in_off2.p, r2.data(), (n_pairs + 1) * 8, cudaMemcpyHostToDevice, st));
    // chunks: consecutive pairs whose direction words fit the budget
    std::vector<uint64_t> dir_off(n_pairs);
    TbLaunch L;
    std::memset(&L, 0, sizeof(L));
    L.seq1 = (const uint8_t *)ctx->in_seq1.p;
    L.seq2 = (const uint8_t *)ctx->in_seq2.p;
    L.off1 = (const uint64_t *)ctx->in_off1.p;
    L.off2 = (const uint64_t *)ctx->in_off2.p;
    L.bnd = (Cell *)ctx->boundary.p;
    L.out = (pa_result *)ctx->in_out.p;
    L.aln = (pa_alignment *)ctx->tb_aln.p;
    L.ops = (uint8_t *)ctx->tb_ops.p;
    if (use_matrix) {
        L.rank = (const int8_t *)ctx->mat_rank.p;
        L.matrix = (const int32_t *)ctx->mat_scores.p;
        L.dim = ctx->mat_dim;
    }
    const int grid = traceback_grid(ctx->sm_count);
    uint64_t launches = 0;
    for (uint64_t first = 0; first < n_pairs;) {
        uint64_t total = 0, end = first;
        while (end < n_pairs && total + words[end] <= kTbBudgetWords) {
            dir_off[end - first] = total;
            total += words[end];
            ++end;
        }
        if ((s = ensure(ctx, ctx->tb_dir, std::max<uint64_t>(total, 1) * 4))) return s;
        // the previous chunk's kernel may still read the offsets: copy them in stream order
        PA_CUDA(ctx, cudaMemcpyAsync(ctx->tb_dir_off.p, dir_off.data(), (end - first) * 8, cudaMemcpyHostToDevice, st));
        PA_CUDA(ctx, cudaStreamSynchronize(st));        // dir_off is reused by the next chunk
        L.first = (uint32_t)first;
        L.count = (uint32_t)(end - first);
        L.dir_off = (const uint64_t *)ctx->tb_dir_off.p;
        L.dir = (uint32_t *)ctx->tb_dir.p;
        traceback_launch(grid, st, L, P);
        ++launches;
        first = end;
    }
    PA_CUDA(ctx, cudaGetLastError());
    PA_CUDA(ctx, cudaEventRecord(ctx->ev1, st));
    PA_CUDA(ctx, cudaMemcpyAsync(out, ctx->in_out.p, n_pairs * sizeof(pa_result), cudaMemcpyDeviceToHost, st));
    PA_CUDA(ctx, cudaMemcpyAsync(alignments, ctx->tb_aln.p, n_pairs * sizeof(pa_alignment), cudaMemcpyDeviceToHost, st));
    if (b1 + b2) PA_CUDA(ctx, cudaMemcpyAsync(ops, ctx->tb_ops.p, b1 + b2, cudaMemcpyDeviceToHost, st));
    PA_CUDA(ctx, cudaStreamSynchronize(st));
    if (stats) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
        stats->pairs = n_pairs;
        stats->cells = cells;
        stats->pairs_s32 = n_pairs;
        stats->kernel_launches = launches;
        stats->device_ms = ms;
        stats->dp_ms = ms;
    }
    return PA_OK;
}

pa_status pa_align_batch_packed(pa_ctx *ctx, const pa_config *config, const uint32_t *seq1_words,
                                const uint64_t *off1, const uint32_t *seq2_words, const uint64_t *off2,
                                uint64_t n_pairs, pa_result *out, pa_stats *stats)
{
    if (!ctx) return PA_ERR_INVALID_ARGUMENT;
    if (n_pairs && (!seq1_words || !seq2_words)) return fail(ctx, PA_ERR_INVALID_ARGUMENT, "null buffer");
    static const uint32_t kNone = 0;     // n_pairs == 0: any non-null pointer selects the packed path
    return align_host(ctx, config, nullptr, off1, nullptr, off2, n_pairs, out, stats, nullptr,
                      seq1_words ? seq1_words : &kNone, seq2_words ? seq2_words : &kNone);
}

// The input-path kernels on the caller's stream (or the context's); a non-null n_invalid waits
// for the count.  The counter belongs to the context: calls on one context are not concurrent.
static pa_status io_counter(pa_ctx *ctx, cudaStream_t st)
{
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, PA_ERR_CUDA, "cudaSetDevice");
    pa_status s = ensure(ctx, ctx->io_ctr, 8);
    if (s) return s;
    PA_CUDA(ctx, cudaMemsetAsync(ctx->io_ctr.p, 0, 8, st));
    return PA_OK;
}

static pa_status io_finish(pa_ctx *ctx, cudaStream_t st, uint64_t *n_invalid)
{
    PA_CUDA(ctx, cudaGetLastError());
    if (n_invalid) {
        unsigned long long v = 0;
        PA_CUDA(ctx, cudaMemcpyAsync(&v, ctx->io_ctr.p, 8, cudaMemcpyDeviceToHost, st));
        PA_CUDA(ctx, cudaStreamSynchronize(st));
        *n_invalid = v;
    }
    return PA_OK;
}

pa_status pa_rank_map_device(pa_ctx *ctx, const uint8_t *symbols, uint32_t n_symbols, const uint8_t *d_in,
                             uint64_t n, int8_t *d_out, void *stream, uint64_t *n_invalid)
{
    if (!ctx) return PA_ERR_INVALID_ARGUMENT;
    if (!symbols || n_symbols == 0) return fail(ctx, PA_ERR_INVALID_ARGUMENT, "the symbol list is empty");
    if (n_symbols > 127) return fail(ctx, PA_ERR_INVALID_ARGUMENT, "at most 127 symbols (int8 ranks)");
    if (n && (!d_in || !d_out)) return fail(ctx, PA_ERR_INVALID_ARGUMENT, "null buffer");
    int8_t table[256];
    std::memset(table, -1, sizeof(table));
    for (uint32_t r = 0; r < n_symbols; ++r) table[symbols[r]] = (int8_t)r;   // a repeat keeps its last rank
    const cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    pa_status s;
    if ((s = io_counter(ctx, st)) || (s = ensure(ctx, ctx->io_tab, 256))) return s;
    PA_CUDA(ctx, cudaMemcpyAsync(ctx->io_tab.p, table, 256, cudaMemcpyHostToDevice, st));
    PA_CUDA(ctx, cudaStreamSynchronize(st));      // `table` is a stack array
    if (n) rank_map_launch(d_in, n, d_out, (const int8_t *)ctx->io_tab.p, (unsigned long long *)ctx->io_ctr.p,
                           ctx->sm_count, st);
    return io_finish(ctx, st, n_invalid);
}

pa_status pa_pack_2bit_device(pa_ctx *ctx, const uint8_t *d_in, uint64_t n, uint32_t *d_words, void *stream,
                              uint64_t *n_invalid)
{
    if (!ctx) return PA_ERR_INVALID_ARGUMENT;
    if (n && (!d_in || !d_words)) return fail(ctx, PA_ERR_INVALID_ARGUMENT, "null buffer");
    const cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    pa_status s;
    if ((s = io_counter(ctx, st))) return s;
    if (n) pack_2bit_launch(d_in, n, d_words, (unsigned long long *)ctx->io_ctr.p, ctx->sm_count, st);
    return io_finish(ctx, st, n_invalid);
}

pa_status pa_unpack_2bit_device(pa_ctx *ctx, const uint32_t *d_words, uint64_t first_base, uint64_t n,
                                uint8_t *d_out, void *stream)
{
    if (!ctx) return PA_ERR_INVALID_ARGUMENT;
    if (n && (!d_words || !d_out)) return fail(ctx, PA_ERR_INVALID_ARGUMENT, "null buffer");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, PA_ERR_CUDA, "cudaSetDevice");
    const cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    if (n) unpack_2bit_launch(d_words, first_base, n, d_out, ctx->sm_count, st);
    return io_finish(ctx, st, nullptr);
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

pa_status pa_band_labels(pa_ctx *ctx, const pa_config *config, const uint8_t *seq1, const uint64_t *off1,
                         const uint8_t *seq2, const uint64_t *off2, uint64_t n_pairs, int32_t *labels)
{
    if (!ctx || !config || (n_pairs && (!seq1 || !off1 || !seq2 || !off2 || !labels)))
        return fail(ctx, PA_ERR_INVALID_ARGUMENT, "null argument");
    if (config->method != PA_METHOD_GLOBAL) return fail(ctx, PA_ERR_UNSUPPORTED, "band labels are for global alignment");
    DpParams P;
    ClassCfg C;
    pa_status s = check_config(ctx, config, P, C);
    if (s) return s;
    if (n_pairs == 0) return PA_OK;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, PA_ERR_CUDA, "cudaSetDevice");
    const uint64_t b1 = off1[n_pairs] - off1[0], b2 = off2[n_pairs] - off2[0];
    // reversed copies of every pair, offsets rebased to 0
    std::vector<uint8_t> r1(std::max<uint64_t>(b1, 1)), r2(std::max<uint64_t>(b2, 1));
    std::vector<uint64_t> o1(n_pairs + 1), o2(n_pairs + 1);
    for (uint64_t k = 0; k <= n_pairs; ++k) { o1[k] = off1[k] - off1[0]; o2[k] = off2[k] - off2[0]; }
    for (uint64_t k = 0; k < n_pairs; ++k) {
        const uint64_t m = o1[k + 1] - o1[k], n = o2[k + 1] - o2[k];
        for (uint64_t x = 0; x < m; ++x) r1[o1[k] + x] = seq1[off1[0] + o1[k] + m - 1 - x];
        for (uint64_t x = 0; x < n; ++x) r2[o2[k] + x] = seq2[off2[0] + o2[k] + n - 1 - x];
    }
    std::memset(labels, 0, sizeof(int32_t) * 8 * n_pairs);
    std::vector<void *> bufs;
    auto dalloc = [&](size_t bytes) -> void * {
        void *p = nullptr;
        if (cudaMalloc(&p, std::max<size_t>(bytes, 16)) != cudaSuccess) { cudaGetLastError(); return nullptr; }
        bufs.push_back(p);
        return p;
    };
    auto cleanup = [&]() { for (void *p : bufs) cudaFree(p); };
    uint8_t *d1 = (uint8_t *)dalloc(b1), *d2 = (uint8_t *)dalloc(b2), *dr1 = (uint8_t *)dalloc(b1),
            *dr2 = (uint8_t *)dalloc(b2);
    uint64_t *do1 = (uint64_t *)dalloc(8 * (n_pairs + 1)), *do2 = (uint64_t *)dalloc(8 * (n_pairs + 1));
    uint64_t *ddoff = (uint64_t *)dalloc(8 * n_pairs);
    int32_t *dlab = (int32_t *)dalloc(sizeof(int32_t) * 8 * n_pairs);
    pa_result *dout = (pa_result *)dalloc(sizeof(pa_result) * n_pairs);
    Cell *dbound = (Cell *)dalloc(sizeof(Cell) * (b1 + n_pairs));
    uint32_t *dorder = (uint32_t *)dalloc(4 * n_pairs), *dctr = (uint32_t *)dalloc(64);
    const uint64_t kDumpBudget = 64ull << 20;                    // int32 entries per chunk (256 MB)
    int32_t *ddump = (int32_t *)dalloc(4 * kDumpBudget);
    if (!d1 || !d2 || !dr1 || !dr2 || !do1 || !do2 || !ddoff || !dlab || !dout || !dbound || !dorder || !dctr || !ddump) {
        cleanup();
        return fail(ctx, PA_ERR_OUT_OF_MEMORY, "band labels: cudaMalloc failed");
    }
    cudaStream_t st = ctx->stream;
    bool ok = cudaMemsetAsync(dctr, 0, 64, st) == cudaSuccess &&
              cudaMemcpyAsync(d1, seq1 + off1[0], b1, cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaMemcpyAsync(d2, seq2 + off2[0], b2, cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaMemcpyAsync(dr1, r1.data(), b1, cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaMemcpyAsync(dr2, r2.data(), b2, cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaMemcpyAsync(do1, o1.data(), 8 * (n_pairs + 1), cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaMemcpyAsync(do2, o2.data(), 8 * (n_pairs + 1), cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaMemsetAsync(dlab, 0, sizeof(int32_t) * 8 * n_pairs, st) == cudaSuccess;
    const int grid = band_labels_occupancy() * ctx->sm_count;
    // long pairs go to the CTA-mode labeller (whole blocks per pair, ring rows per block)
    int64_t long_m = 0;
    for (uint64_t k = 0; k < n_pairs; ++k) {
        const int64_t m = (int64_t)(o1[k + 1] - o1[k]), n = (int64_t)(o2[k + 1] - o2[k]);
        if (m * n >= ctx->long_cells && m <= (1 << 20) && n <= (1 << 20)) long_m = std::max(long_m, m);
    }
    if (ok && long_m && ensure_ring(ctx, long_m) != PA_OK) ok = false;
    const int64_t ring_m = ctx->ring.p ? ctx->ring_m : 0;
    std::vector<uint64_t> doff(n_pairs, 0);
    std::vector<uint32_t> order;
    uint64_t k = 0;
    while (ok && k < n_pairs) {
        order.clear();
        std::vector<uint32_t> longs;
        uint64_t used = 0;
        for (; k < n_pairs; ++k) {
            const uint64_t m = o1[k + 1] - o1[k], n = o2[k + 1] - o2[k];
            if (m < 9 || n == 0) continue;                        // checkpoints need 9 columns
            const uint64_t need = 8 * (n + 1);
            if (need > kDumpBudget) { ok = false; break; }
            if (used + need > kDumpBudget) break;
            doff[k] = used;
            used += need;
            const bool lng = (int64_t)(m * n) >= ctx->long_cells && (int64_t)m <= ring_m && n <= (1u << 20);
            (lng ? longs : order).push_back((uint32_t)k);
        }
        if (!ok || (order.empty() && longs.empty())) break;
        const uint32_t ns = (uint32_t)order.size();
        order.insert(order.end(), longs.begin(), longs.end());
        const uint32_t ctr[4] = {0u, ns, ns, (uint32_t)longs.size()};   // begin, count per list
        ok = cudaMemcpyAsync(ddoff, doff.data(), 8 * n_pairs, cudaMemcpyHostToDevice, st) == cudaSuccess &&
             cudaMemcpyAsync(dorder, order.data(), 4 * order.size(), cudaMemcpyHostToDevice, st) == cudaSuccess &&
             cudaMemcpyAsync(dctr + 8, ctr, sizeof(ctr), cudaMemcpyHostToDevice, st) == cudaSuccess;
        for (int rev = 0; ok && rev < 2; ++rev) {
            DpLaunch L;
            std::memset(&L, 0, sizeof(L));
            L.seq1 = rev ? dr1 : d1; L.off1 = do1; L.seq2 = rev ? dr2 : d2; L.off2 = do2;
            L.order = dorder; L.begin_ptr = dctr + 8; L.count_ptr = dctr + 9; L.unit_counter = dctr;
            L.out = dout; L.boundary = dbound; L.G = 8;
            L.dump = ddump; L.dump_off = ddoff; L.labels = dlab;
            L.error = dctr + 4;
            L.spin_limit = ctx->wait_limit;
            ok = cudaMemsetAsync(dctr, 0, 8, st) == cudaSuccess;
            if (ok && ns) band_labels_launch(rev == 1, grid, st, L, P);
            if (ok && !longs.empty()) {
                L.begin_ptr = dctr + 10; L.count_ptr = dctr + 11; L.unit_counter = dctr + 1; L.G = 32;
                L.ring = (Cell *)ctx->ring.p;
                L.ring_stride = (uint64_t)ctx->ring_m + 2;
                band_labels_cta_launch(rev == 1, ctx->ring_grid, st, L, P);
            }
            ok = ok && cudaGetLastError() == cudaSuccess;
        }
        ok = ok && cudaStreamSynchronize(st) == cudaSuccess;      // the host staging arrays are reused
    }
    uint32_t err_bits = 0;
    if (ok && (cudaMemcpy(&err_bits, dctr + 4, 4, cudaMemcpyDeviceToHost) != cudaSuccess || err_bits)) ok = false;
    ok = ok && cudaMemcpyAsync(labels, dlab, sizeof(int32_t) * 8 * n_pairs, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
         cudaStreamSynchronize(st) == cudaSuccess;
    cleanup();
    if (!ok) {
        cudaGetLastError();
        return fail(ctx, PA_ERR_CUDA, "band labels: a CUDA call failed or a pair exceeds the dump budget");
    }
    return PA_OK;
}

pa_status pa_get_tuning(const pa_ctx *ctx, pa_tuning *out)
{
    if (!ctx || !out) return PA_ERR_INVALID_ARGUMENT;
    *out = ctx->tuning;
    return PA_OK;
}

static bool valid_G(int g) { return g == 0 || (g >= 1 && g <= 32 && (g & (g - 1)) == 0); }
static bool valid_variant(int v) { return v >= 0 && v < kVariants; }

pa_status pa_set_tuning(pa_ctx *ctx, const pa_tuning *t)
{
    if (!ctx || !t) return PA_ERR_INVALID_ARGUMENT;
    for (int m = 0; m < 2; ++m)
        if (!valid_variant(t->variant_s16[m]) || !valid_variant(t->variant_s32[m]) || !valid_G(t->group_threads_s16[m]) ||
            !valid_G(t->group_threads_s32[m]))
            return fail(ctx, PA_ERR_INVALID_ARGUMENT,
                        "tuning: variant must be 0..10 and group_threads 0 or 1..32, power of two");
    for (int m = 0; m < 2; ++m)
        for (int a = 0; a < PA_TUNE_SIZES; ++a)
            for (int b = 0; b < PA_TUNE_SHAPES; ++b) {
                const pa_tune_entry &e = t->s16[m][a][b];
                if (!valid_variant(e.variant) || !valid_G(e.group_threads))
                    return fail(ctx, PA_ERR_INVALID_ARGUMENT, "tuning table: variant 0..10, group_threads 0..32");
            }
    ctx->tuning = *t;
    ctx->fixed_G = ctx->fixed_variant = false;
    return PA_OK;
}

pa_status pa_autotune(pa_ctx *ctx, const pa_config *config, const uint8_t *seq1, const uint64_t *off1,
                      const uint8_t *seq2, const uint64_t *off2, uint64_t n_pairs, pa_tuning *out)
{
    if (!ctx || !config) return PA_ERR_INVALID_ARGUMENT;
    if (n_pairs && (!off1 || !off2)) return fail(ctx, PA_ERR_INVALID_ARGUMENT, "null offsets");
    const int mi = (config->method & ~PA_SCORE_MATRIX) == PA_METHOD_LOCAL ? 0 : 1;
    const uint64_t b1 = n_pairs ? off1[n_pairs] - off1[0] : 0, b2 = n_pairs ? off2[n_pairs] - off2[0] : 0;
    pa_tune_entry &slot = ctx->tuning.s16[mi][tune_size_class(n_pairs)][tune_shape_class(n_pairs, b1, b2)];
    const pa_tune_entry saved = slot;
    const bool fg = ctx->fixed_G, fv = ctx->fixed_variant;
    ctx->fixed_G = ctx->fixed_variant = false;
    std::vector<pa_result> res(std::max<uint64_t>(n_pairs, 1));
    // the short-pair kernel with 16 and 32 rows per thread at every group size it has, and the
    // general kernel down to one pair per lane (two per thread in s16x2 halves)
    struct Cand { int v, g; };
    std::vector<Cand> cands;
    for (int v = kShortVariant; v < kVariants; ++v)
        for (int g : {4, 8, 16, 32}) cands.push_back({v, g});
    for (int g : {1, 2, 4, 8, 16, 32}) cands.push_back({mi == 0 ? 7 : 4, g});
    double best = 1e300;
    pa_tune_entry choice = saved;
    for (const Cand &cd : cands) {
        slot = pa_tune_entry{(int16_t)cd.v, (int16_t)cd.g, 0.f};
        double ms = 1e300;
        for (int rep = 0; rep < 3; ++rep) {                 // first run captures the graph
            pa_stats st;
            pa_status s = pa_align_batch(ctx, config, seq1, off1, seq2, off2, n_pairs, res.data(), &st);
            if (s) { slot = saved; ctx->fixed_G = fg; ctx->fixed_variant = fv; return s; }
            if (rep > 0) ms = std::min(ms, st.dp_ms);
        }
        if (ms < best) { best = ms; choice = slot; choice.dp_ms = (float)ms; }
    }
    slot = choice;
    ctx->tuning.best_ms[mi] = best;
    ctx->fixed_G = fg;
    ctx->fixed_variant = fv;
    drop_graphs(ctx);                                       // the candidates' captures
    if (out) *out = ctx->tuning;
    return PA_OK;
}

pa_status pa_measure_roofline(pa_ctx *ctx, pa_roofline *out)
{
    if (!ctx || !out) return PA_ERR_INVALID_ARGUMENT;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, PA_ERR_CUDA, "cudaSetDevice");
    DevBuf sink;
    pa_status s = ensure(ctx, sink, 1 << 20);
    if (s) return s;
    int per[3] = {0, 0, 0};
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per[0], k_roofline<L16>, 256, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per[1], k_roofline<L32>, 256, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per[2], k_roofline<L16, true>, 256, 0);
    const int steps = 4096;
    double best[3] = {0, 0, 0};
    for (int rep = 0; rep < 4; ++rep) {
        for (int w = 0; w < 3; ++w) {
            const int grid = std::max(1, per[w]) * ctx->sm_count;
            PA_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
            if (w == 1) k_roofline<L32><<<grid, 256, 0, ctx->stream>>>(steps, rep, (uint32_t *)sink.p);
            else if (w == 2) k_roofline<L16, true><<<grid, 256, 0, ctx->stream>>>(steps, rep, (uint32_t *)sink.p);
            else k_roofline<L16><<<grid, 256, 0, ctx->stream>>>(steps, rep, (uint32_t *)sink.p);
            PA_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
            PA_CUDA(ctx, cudaEventSynchronize(ctx->ev1));
            float ms = 0;
            cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
            const double cells = (double)grid * 256 * steps * 16 * (w == 1 ? 1 : 2);
            best[w] = std::max(best[w], cells / (ms * 1e-3));
        }
    }
    cudaFree(sink.p);
    int clk = 0;
    cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, ctx->device);
    out->s16x2_cells_per_s = best[0];
    out->s32_cells_per_s = best[1];
    out->sm_clock_mhz = clk / 1000.0;
    out->sm_count = ctx->sm_count;
    out->reserved = 0;
    out->s16x2_local_cells_per_s = best[2];
    return PA_OK;
}

}  // extern "C"
