/*
 * pairwise_aligner_gb300.h -- C ABI of the GB300 (sm_103a) affine-gap score DP.
 *
 * The reference library (rrahn/pairwise_aligner) is header-only C++20 and has no
 * FFI; its plug point for this path is the score-model rule category
 * (include/pairwise_aligner/configuration/rule_category.hpp:24-30) whose traits
 * return the interface object, and the call a user makes is
 *     auto a = cfg::configure_aligner(cfg::method_global(cfg::gap_model_affine(
 *                  cfg::score_model_unitary_simd_saturated(match, mismatch), open, ext), lead, trail));
 *     for (auto r : a.compute(seqs1, seqs2)) r.score();
 * (test/unit/configuration/configure_aligner_saturated_test.cpp:22-41).  The
 * entry points below are what that interface object's compute() binds to in
 * this project: pairwise_aligner_gb300.hpp (header-only C++20, same cfg::
 * names) and pairwise_aligner_gb300/ (Python) call them.
 *
 * Conventions shared by every entry point:
 *  - Plain pointers and sizes only.  Sequences are concatenated bytes plus
 *    n_pairs+1 uint64 offsets (pair k is bytes [off[k], off[k+1])).  Bytes are
 *    compared raw, like score_model_unitary::score (score_model_unitary.hpp:52-59).
 *  - Scores use the reference's signs: match > 0, mismatch < 0, gap_open <= 0,
 *    gap_extension <= 0; a gap of length k scores gap_open + k * gap_extension
 *    (affine_initialisation_strategy.hpp:38-51, affine_dp_algorithm.hpp:149-155).
 *  - Errors are status codes; nothing throws across the ABI.
 *  - One context per host thread (or external locking).  A context owns one
 *    CUDA stream, its device buffers and its CUDA-graph cache.
 */
#ifndef PAIRWISE_ALIGNER_GB300_H
#define PAIRWISE_ALIGNER_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PA_ABI_VERSION 2

typedef enum pa_status {
    PA_OK = 0,
    PA_ERR_INVALID_ARGUMENT = 1,  /* null pointer, bad offsets, bad config            */
    PA_ERR_CUDA = 2,              /* a CUDA runtime call failed (see pa_last_error)    */
    PA_ERR_OUT_OF_MEMORY = 3,
    PA_ERR_OVERFLOW = 4,          /* scores could exceed int32 for this input          */
    PA_ERR_UNSUPPORTED = 5,       /* e.g. a positive gap score                         */
    PA_ERR_TIMEOUT = 6,           /* a bounded device-side wait gave up                */
    PA_ERR_NO_DEVICE = 7,
    PA_ERR_TOO_LARGE = 8          /* sizes beyond a fixed capacity                     */
} pa_status;

typedef enum pa_method { PA_METHOD_GLOBAL = 0, PA_METHOD_LOCAL = 1 } pa_method;

/* Added to pa_config.method: score with the context's substitution matrix
 * (pa_set_substitution_matrix; cfg::score_model_matrix) instead of match/mismatch. */
#define PA_SCORE_MATRIX 0x100

/* Alignment configuration.  Replaces the compile-time rule chain
 * cfg::method_global / cfg::method_local (method_global.hpp:121-145,
 * method_local.hpp:118-137), cfg::gap_model_affine (gap_model_affine.hpp:130-155)
 * and cfg::score_model_unitary* (score_model_unitary_simd_saturated.hpp:259-284).
 * The end-gap flags follow cfg::leading_end_gap / cfg::trailing_end_gap
 * (end_gap_policy.hpp:26-36); method_local forces all four free. */
typedef struct pa_config {
    int32_t method;             /* pa_method                                              */
    int32_t match;
    int32_t mismatch;
    int32_t gap_open;
    int32_t gap_extension;
    uint8_t first_column_free;  /* leading gap in sequence1 free: H(i,0) = 0              */
    uint8_t first_row_free;     /* leading gap in sequence2 free: H(0,j) = 0              */
    uint8_t last_column_free;   /* the result may end anywhere in column n                */
    uint8_t last_row_free;      /* the result may end anywhere in row m                   */
    int32_t width_hint;         /* 0 auto (s16x2 then s32), 16, or 32                     */
    int32_t band_mode;          /* 0: plain full DP.  Global alignment with penalised end
                                   gaps only: 1 learned band (pa_set_band_model), 2 the
                                   straight-line band; both with certificate, doubling and
                                   the full DP as fallback, so scores are unchanged      */
} pa_config;

/* Per-pair result (16 bytes).  score mirrors aligner_result::score()
 * (result/aligner_result.hpp:32-105); end1/end2 are 1-based end positions in
 * sequence1/sequence2 (the reference has none: "TODO: optimal_coordinate()"),
 * ties to the smallest end1, then the smallest end2.  Local: a score of 0 gives
 * (0,0); an empty sequence gives INT32_MIN and (0,0), like
 * tracker_local_scalar.hpp:38. */
typedef struct pa_result {
    int32_t score;
    int32_t end1;
    int32_t end2;
    uint8_t width;              /* 16 or 32: arithmetic width that produced the score      */
    uint8_t flags;              /* PA_RESULT_* bits                                        */
    uint16_t band_rounds;       /* band doublings used (band_mode 1), else 0               */
} pa_result;

#define PA_RESULT_RERUN      0x01u  /* s16 result failed its exactness check, rerun at s32 */
#define PA_RESULT_BANDED     0x02u  /* certified banded result                              */
#define PA_RESULT_FULL_DP    0x04u  /* band fell back to the full DP                        */
#define PA_RESULT_TRIVIAL    0x08u  /* an empty sequence: answered without a DP             */
#define PA_RESULT_OVERFLOW   0x10u  /* the pair's scores could exceed int32: not aligned,
                                       score INT32_MIN (the call returns PA_ERR_OVERFLOW when
                                       it reports errors)                                     */
#define PA_RESULT_ERROR      0x20u  /* no valid score, INT32_MIN: the pair's offsets are
                                       inconsistent (a device entry point, see below), a
                                       symbol is outside the substitution matrix, or a
                                       bounded device wait gave up (PA_ERR_TIMEOUT)           */

/* Context options; zero-initialised means defaults. */
typedef struct pa_options {
    int32_t group_threads;      /* threads per pair group: 0 auto, else 1,2,4,8,16,32      */
    int32_t rows_per_thread;    /* rows a thread holds per lane: 0 auto, else 8,16,32      */
    int32_t blocks_per_sm;      /* persistent grid occupancy: 0 auto                       */
    int32_t use_graphs;         /* 0 auto(on), 1 on, -1 off                                */
    int32_t autotune;           /* 0 off, 1 on first use                                   */
    int32_t kernel_variant;     /* inner-loop form: -1 auto (tuning table), else 0..10 (pa_tuning) */
    int32_t reserved[2];
} pa_options;

/* Counters of the last call. */
typedef struct pa_stats {
    uint64_t pairs;
    uint64_t cells;             /* sum of m*n over pairs (full-matrix cells)              */
    uint64_t pairs_s16;         /* pairs finished in s16x2 lanes                          */
    uint64_t pairs_s32;         /* pairs finished in s32 lanes (incl. reruns)             */
    uint64_t pairs_general;     /* pairs whose sequence2 is not all A/C/G/T               */
    uint64_t pairs_rerun;       /* s16 results promoted to s32                            */
    uint64_t pairs_trivial;
    uint64_t kernel_launches;   /* kernels this call launched                             */
    double   device_ms;         /* device time of the whole call (CUDA events)            */
    double   dp_ms;             /* device time of the DP kernels alone                    */
    uint64_t pairs_banded;      /* band mode: results accepted by the certificate         */
    uint64_t pairs_full_dp;     /* band mode: results of the full-DP fallback             */
    uint64_t band_cells;        /* band mode: cells the banded DP computed (all rounds)   */
    uint64_t band_rounds;       /* band mode: band widths tried                           */
} pa_stats;

typedef struct pa_ctx pa_ctx;

/* Create / destroy a context bound to a CUDA device ordinal. */
pa_status pa_create(pa_ctx **out, int device_ordinal, const pa_options *options);
pa_status pa_destroy(pa_ctx *ctx);

/* Align n_pairs pairs given in HOST memory; synchronous.  Replaces
 * interface_one_to_one_bulk::compute (interface/interface_one_to_one_bulk.hpp:47-100)
 * without its "<= lane count" batch limit (:55-57): any n_pairs.  Host buffers
 * may be pageable or pinned; out has n_pairs entries.  stats may be NULL. */
pa_status pa_align_batch(pa_ctx *ctx, const pa_config *config,
                         const uint8_t *seq1, const uint64_t *off1,
                         const uint8_t *seq2, const uint64_t *off2,
                         uint64_t n_pairs, pa_result *out, pa_stats *stats);

/* Same, with every buffer already in device memory of the context's device.
 * Asynchronous on `stream` (a cudaStream_t; NULL = the context's stream,
 * cudaStreamLegacy / cudaStreamPerThread are accepted);
 * seq1_bytes / seq2_bytes are the sizes of the two byte buffers.  When stats
 * is non-NULL the call synchronises to fill it.
 * The offsets are checked on the device: if any pair has off[k] > off[k+1] or an
 * offset past seq1_bytes / seq2_bytes, no pair is aligned and every result is
 * INT32_MIN with PA_RESULT_ERROR.  Errors found on the device (those offsets,
 * PA_ERR_OVERFLOW, PA_ERR_TIMEOUT, symbols outside a substitution matrix) are
 * returned as a status only when stats is non-NULL (the call then waits for the
 * device); without stats the call returns as soon as the work is queued, and the
 * affected pairs carry PA_RESULT_OVERFLOW / PA_RESULT_ERROR in their results.
 * Band mode waits on the host for the class counts and for every band round; without
 * stats it returns once its last launches are queued. */
pa_status pa_align_batch_device(pa_ctx *ctx, const pa_config *config,
                                const uint8_t *d_seq1, const uint64_t *d_off1, uint64_t seq1_bytes,
                                const uint8_t *d_seq2, const uint64_t *d_off2, uint64_t seq2_bytes,
                                uint64_t n_pairs, pa_result *d_out, void *stream, pa_stats *stats);

/* Same alignment with NO allocation of any kind; this entry point has no
 * counterpart in the reference.  It is for callers that cannot allocate device
 * memory when they align: runtimes whose own allocator must own every byte,
 * code that runs while a CUDA graph is captured (cudaMalloc is not allowed
 * there), or latency-critical paths that must not stall on an allocation.
 * No context is needed: the caller passes device inputs and the device output
 * (n_pairs pa_result) and a stream (NULL = the legacy default stream).
 *  - Scratch: the pass-boundary rows live in a file-scope device array of
 *    4,194,304 cells (32 MiB) that every GPU loading the library holds until
 *    the process exits.  seq1_bytes + n_pairs must not exceed 4,194,304,
 *    else PA_ERR_TOO_LARGE is returned and nothing is launched.
 *  - Every call made outside a stream capture looks up that array's device
 *    address (cudaGetSymbolAddress) with the device current, so a device that
 *    was reset is followed.  A call made while `stream` is captured uses the
 *    address of the last call on that device: make the first call on a device
 *    before any stream capture (else PA_ERR_UNSUPPORTED).
 *  - All calls share the array: calls whose work overlaps on the GPU (other
 *    streams, other host threads) race.  Serialise them.
 *  - Arithmetic is s32 with raw byte comparison, pairs in input order.
 *  - Errors are per pair (the call returns before the device runs): a pair
 *    whose scores could exceed int32 gets INT32_MIN and PA_RESULT_OVERFLOW; a
 *    pair whose offsets decrease or run past seq1_bytes / seq2_bytes is not
 *    aligned and gets INT32_MIN and PA_RESULT_ERROR (its scratch row could
 *    leave the array); other pairs of a batch with such offsets have undefined
 *    scores, since their scratch rows may overlap.
 * Scores and end positions equal those of pa_align_batch_device.  The other
 * fields differ: width is always 32 and PA_RESULT_RERUN never appears; over-
 * bound pairs are flagged here while pa_align_batch_device also returns
 * PA_ERR_OVERFLOW when it reports errors; and NULL `stream` means the legacy
 * default stream here but the context's stream there. */
pa_status pa_align_batch_device_static(const pa_config *config,
                                       const uint8_t *d_seq1, const uint64_t *d_off1, uint64_t seq1_bytes,
                                       const uint8_t *d_seq2, const uint64_t *d_off2, uint64_t seq2_bytes,
                                       uint64_t n_pairs, pa_result *d_out, void *stream);

/* One query against many targets (interface/interface_one_to_many_bulk.hpp:47-92):
 * pair k is (query, targets[k]).  Host buffers, synchronous. */
pa_status pa_align_one_to_many(pa_ctx *ctx, const pa_config *config,
                               const uint8_t *query, uint64_t query_len,
                               const uint8_t *targets, const uint64_t *target_off,
                               uint64_t n_targets, pa_result *out, pa_stats *stats);

/* Band-predictor training labels (global alignment only; no counterpart in the
 * reference): for every pair the diagonal j - i_c of the optimal path at the 8
 * checkpoint columns i_c = c*m/9 (c = 1..8) of sequence1, from a forward and a
 * reverse full DP on the GPU (the argmax over j of the best score through
 * (i_c, j); ties to the smallest j).  Host buffers; labels has 8 * n_pairs
 * entries (0 for pairs with m < 9 or an empty sequence2). */
pa_status pa_band_labels(pa_ctx *ctx, const pa_config *config,
                         const uint8_t *seq1, const uint64_t *off1,
                         const uint8_t *seq2, const uint64_t *off2,
                         uint64_t n_pairs, int32_t *labels);

/* Band predictor building blocks (device pointers, asynchronous on `stream`;
 * no counterpart in the reference).  pa_band_features_device writes 130 floats
 * per pair: the 128-bin histogram of diagonal offsets j - i of shared 12-mers
 * (bins over [-m, n], divided by the number of sequence1 12-mers), m/1024, n/1024.
 * The pa_mlp_* calls are the training and inference kernels of the BF16 MLP
 * 130 -> 256 -> 256 -> 9: a BF16 tensor-core GEMM with FP32 accumulation and a
 * fused bias/ReLU epilogue, the MSE loss gradient, the ReLU derivative, bias
 * gradients, Adam on FP32 master weights, and FP32 -> BF16 padding. */
pa_status pa_band_features_device(const uint8_t *d_seq1, const uint64_t *d_off1,
                                  const uint8_t *d_seq2, const uint64_t *d_off2,
                                  uint64_t n_pairs, float *d_features, void *stream);
pa_status pa_mlp_gemm(const void *A, const void *B, float *C32, void *C16, const float *bias,
                      int M, int N, int K, int lda, int ldb, int ldc, int ta, int tb, int relu,
                      float beta, void *stream);
pa_status pa_mlp_mse(const float *out, const float *target, const float *mask, int batch,
                     void *dout, float *loss_sum, void *stream);
pa_status pa_mlp_relu_grad(void *dh, const void *h, int n, void *stream);
pa_status pa_mlp_colsum(const void *d, int batch, int n_cols, float *db, void *stream);
pa_status pa_mlp_adam(float *w, void *w16, const float *grad, float *m1, float *m2, int n,
                      float lr, float beta1, float beta2, float eps, int step, float weight_decay,
                      void *stream);
pa_status pa_mlp_to_bf16(const float *src, int rows, int cols, int ld_dst, void *dst, void *stream);

/* Pairs with at least `cells` = m * n cells are computed by whole thread blocks
 * (the warps of a block pipeline the pair's row passes) instead of one group of
 * lanes; default 2^20.  1 sends every pair there, UINT64_MAX none. */
pa_status pa_set_cta_threshold(pa_ctx *ctx, uint64_t cells);

/* Calls the context keeps captured as CUDA graphs (replayed when a call repeats the
 * same buffers, sizes, configuration and launch shapes; at most 8, the least recently
 * replayed is dropped first).  No counterpart in the reference. */
pa_status pa_get_graph_count(const pa_ctx *ctx, uint32_t *out);

/* Polls a CTA-mode progress wait makes after its first look before it gives up
 * (default 2^24, with a short sleep between polls).  A wait that gives up marks its
 * pair PA_RESULT_ERROR and the call returns PA_ERR_TIMEOUT; 0 gives up at the first
 * look (tests use it to exercise that path).  No counterpart in the reference. */
pa_status pa_set_wait_limit(pa_ctx *ctx, uint32_t polls);

/* Of those, pairs whose sequence2 has at most `max_rows` rows (few 512-row passes) run on
 * teams of 4 warps, two pairs per block, instead of all 8 warps of a block (beside
 * them, on the SMs their blocks release); default 12288 (24 passes), 0 keeps every
 * such pair on whole blocks. */
pa_status pa_set_team_threshold(pa_ctx *ctx, uint32_t max_rows);

/* Of those, pairs with at least `cells` cells and `min_rows` rows of sequence2 are
 * computed by clusters of 4 thread blocks (co-scheduled; their 32 warps pipeline the
 * pair's passes); defaults 2^28 and 8192. */
pa_status pa_set_cluster_threshold(pa_ctx *ctx, uint64_t cells, uint32_t min_rows);

/* Substitution-matrix scoring (configuration/score_model_matrix.hpp:203-222,
 * score_model/score_model_matrix.hpp:53-63): symbols[r] is the symbol of rank r,
 * scores[r1 * dim + r2] the score of a sequence1 symbol of rank r1 against a
 * sequence2 symbol of rank r2 (dim <= 32, |score| <= 2^20).  Calls whose config has
 * PA_SCORE_MATRIX use it; every symbol of their sequences must be in `symbols`
 * (else PA_ERR_INVALID_ARGUMENT).  Not with band mode. */
pa_status pa_set_substitution_matrix(pa_ctx *ctx, const uint8_t *symbols, uint32_t dim, const int32_t *scores);

/* Band mode (no counterpart in the reference, which has no banded mode).
 * A pair's band: the centre line through (0, 0), the checkpoints
 * (i_c, i_c + diag[c]) with i_c = (c + 1) * m / 9, c = 0..7, and (m, n),
 * widened to also cover the diagonal n - m; the half-width tapers linearly
 * from w_start at column 0 to w_min at column m.  Every round the banded DP
 * proves its score or the band doubles; a pair whose band would cover more
 * than full_frac of its matrix, or that is still open after max_rounds, is
 * computed by the full DP.  margin scales the learned starting width;
 * straight_w0 is the starting width of band_mode 2.  Pairs of at most
 * pa_set_team_threshold rows use team_full_frac instead of full_frac (0: full_frac):
 * their full DP runs on teams of 4 warps, fast enough that a band pays only when it
 * is much narrower than the matrix.  The full DP of long pairs is routed as in the
 * plain path (teams, whole blocks, clusters, at the same time). */
typedef struct pa_band_options {
    float margin;               /* default 1.25 */
    int32_t w_min;              /* default 16   */
    int32_t straight_w0;        /* default 64   */
    float full_frac;            /* default 0.85 */
    int32_t max_rounds;         /* default 2    */
    float team_full_frac;       /* default 0.65 */
    int32_t reserved[2];
} pa_band_options;

pa_status pa_set_band_options(pa_ctx *ctx, const pa_band_options *options);
pa_status pa_get_band_options(const pa_ctx *ctx, pa_band_options *out);

/* Load the band predictor of band_mode 1: FP32 host arrays of the MLP
 * 130 -> 256 -> 256 -> 9 in padded row-major layout, w1 144 x 256 (rows
 * 130..143 unused), b1 256, w2 256 x 256, b2 256, w3 256 x 16 (columns 9..15
 * unused), b3 16.  Outputs 0..7 are the checkpoint diagonals divided by
 * (m + n) / 4, output 8 is log2(1 + smax (m + n) - 2 score) / 16. */
pa_status pa_set_band_model(pa_ctx *ctx, const float *w1, const float *b1, const float *w2,
                            const float *b2, const float *w3, const float *b3);

/* Band mode with caller-given bands: 10 int32 per pair (diag[8], w_start,
 * w_min), otherwise as pa_align_batch (config->band_mode is ignored). */
pa_status pa_align_batch_banded(pa_ctx *ctx, const pa_config *config,
                                const uint8_t *seq1, const uint64_t *off1,
                                const uint8_t *seq2, const uint64_t *off2,
                                uint64_t n_pairs, const int32_t *bands,
                                pa_result *out, pa_stats *stats);

/* Kernel choices of a context.  Replaces nothing in the reference (its tile
 * shapes are compile-time lane widths, simd/simd_base.hpp:28-57).
 * variant: inner-loop form of the DP: 0..8 the general kernel (0 three-operand max,
 * 1 short chain, 2 three-operand with at most 85 registers, 3 branch-free top input with
 * L1 prefetch, 4 as 3 with a two-op vertical-gap chain, 5 / 6 as 3 / 4 with one prefetch
 * per 8 columns, 7 / 8 as 3 / 4 without the score-table prefetch), 9 / 10 the short-pair
 * s16x2 kernel with 16 / 32 rows of sequence2 per thread (unitary DNA scores; other
 * classes take the general kernel's default); group_threads: lanes per pair group (1..32,
 * power of two; 0: the built-in rule, which picks it from the batch size).  Index 0 =
 * local, 1 = global.
 * The s16x2 class also has a table of tuned entries, one per method, batch-size class
 * and pair-size class: size class s = 0..3 when n_pairs < 2^(12 + 2s), else 4; pair-size
 * class h = 0..2 when the mean m*n per pair < 2^(14 + 2h), else 3.  An entry with
 * group_threads 0 falls back to variant_s16 / group_threads_s16; when that group size is
 * 0 too and variant_s16 is a short-pair variant, the rule also picks its rows per thread
 * (32 for groups of up to 8 lanes, else 16). */
#define PA_TUNE_SIZES 5
#define PA_TUNE_SHAPES 4
typedef struct pa_tune_entry {
    int16_t variant;            /* 0..10                                                   */
    int16_t group_threads;      /* 1..32, power of two; 0: not tuned                       */
    float dp_ms;                /* pa_autotune: device time of the chosen candidate        */
} pa_tune_entry;

typedef struct pa_tuning {
    int32_t variant_s16[2];
    int32_t variant_s32[2];
    int32_t group_threads_s16[2];
    int32_t group_threads_s32[2];
    double best_ms[2];          /* pa_autotune: device time of the chosen candidate        */
    pa_tune_entry s16[2][PA_TUNE_SIZES][PA_TUNE_SHAPES];
} pa_tuning;

/* Time every (variant, group_threads) candidate of the s16x2 class on this batch (host
 * buffers, as pa_align_batch) and keep the fastest in the table entry of the batch's
 * method, size class and pair-size class; the whole tuning is also written to *out (may be
 * NULL). */
pa_status pa_autotune(pa_ctx *ctx, const pa_config *config,
                      const uint8_t *seq1, const uint64_t *off1,
                      const uint8_t *seq2, const uint64_t *off2,
                      uint64_t n_pairs, pa_tuning *out);
pa_status pa_get_tuning(const pa_ctx *ctx, pa_tuning *out);
pa_status pa_set_tuning(pa_ctx *ctx, const pa_tuning *tuning);

/* Measured whole-chip throughput of the cell-update instruction mix, used as
 * the roofline denominator: packed s16x2 DPX cell updates per second and s32
 * cell updates per second, from a timed in-register microkernel. */
typedef struct pa_roofline {
    double s16x2_cells_per_s;
    double s32_cells_per_s;
    double sm_clock_mhz;
    int32_t sm_count;
    int32_t reserved;
    double s16x2_local_cells_per_s;   /* the s16x2 mix plus local scoring's column maximum */
} pa_roofline;
pa_status pa_measure_roofline(pa_ctx *ctx, pa_roofline *out);

/* ---- Traceback ---------------------------------------------------------------
 * The optimal alignment, which the reference does not compute (its trackers carry
 * "TODO: optimal_coordinate()"): for every pair the pa_result of pa_align_batch (same
 * score and end cell) plus the begin cell and the path as SAM-style ops, one byte per
 * alignment column: '=' equal symbols, 'X' different symbols, 'D' a symbol of
 * sequence1 against a gap, 'I' a symbol of sequence2 against a gap.  The path runs
 * from just after cell (begin1, begin2) to (end1, end2): ops hold end1 - begin1
 * sequence1 symbols ('=', 'X', 'D') and end2 - begin2 sequence2 symbols ('=', 'X',
 * 'I').  A free leading gap shows as a begin > 0; a penalised one as ops.  Ties: the
 * diagonal before a gap along sequence1 ('D') before one along sequence2 ('I'); a gap
 * opens unless extending it is strictly better; a local path starts after the last
 * cell whose score is 0.  Local pairs with a score <= 0 (or an empty sequence) have
 * no ops.  Host buffers, synchronous; ops must hold (off1[n] - off1[0]) + (off2[n] -
 * off2[0]) bytes, pair k's at (off1[k] - off1[0]) + (off2[k] - off2[0]).  Device
 * memory: 4 bits per cell, in chunks of pairs of at most 4 GiB (a pair needing more
 * is PA_ERR_TOO_LARGE). */
typedef struct pa_alignment {
    int32_t begin1;
    int32_t begin2;
    uint32_t n_ops;
    uint32_t reserved;
} pa_alignment;

pa_status pa_traceback_batch(pa_ctx *ctx, const pa_config *config,
                             const uint8_t *seq1, const uint64_t *off1,
                             const uint8_t *seq2, const uint64_t *off2,
                             uint64_t n_pairs, pa_result *out, pa_alignment *alignments,
                             uint8_t *ops, pa_stats *stats);

/* ---- Input path ------------------------------------------------------------
 * Symbol -> rank conversion (alphabet_conversion/alphabet_rank_map_scalar.hpp and
 * alphabet_rank_map_simd.hpp:31-117): symbols[r] gets rank r (a repeated symbol
 * keeps its last rank, as the reference's fill loop does), every other byte -1.
 * n_symbols 1..127 (an empty list is PA_ERR_INVALID_ARGUMENT, as the reference
 * throws std::invalid_argument).  Device buffers of n bytes, asynchronous on
 * `stream` (NULL: the context's stream); *n_invalid (host, may be NULL) receives
 * the number of bytes without a rank, which makes the call synchronous. */
pa_status pa_rank_map_device(pa_ctx *ctx, const uint8_t *symbols, uint32_t n_symbols,
                             const uint8_t *d_in, uint64_t n, int8_t *d_out, void *stream,
                             uint64_t *n_invalid);

/* 2-bit DNA packing (no counterpart in the reference).  Base i of a stream is
 * bits 2(i mod 16) .. 2(i mod 16)+1 of word i / 16; A/a = 0, C/c = 1, G/g = 2,
 * T/t = 3.  Any other byte is counted in *n_invalid and packed as
 * ((b >> 1) ^ (b >> 2)) & 3.  Unused bits of the last word are 0.
 * pa_pack_2bit_host runs on the calling thread (host buffers, the encoder for
 * files and callers that keep DNA packed); the _device forms run on `stream`
 * (NULL: the context's stream; synchronous when n_invalid is given).  Unpacking
 * writes bases [first_base, first_base + n) of the stream as the upper-case
 * letters ACGT. */
pa_status pa_pack_2bit_host(const uint8_t *in, uint64_t n, uint32_t *out_words, uint64_t *n_invalid);
pa_status pa_pack_2bit_device(pa_ctx *ctx, const uint8_t *d_in, uint64_t n, uint32_t *d_words,
                              void *stream, uint64_t *n_invalid);
pa_status pa_unpack_2bit_device(pa_ctx *ctx, const uint32_t *d_words, uint64_t first_base, uint64_t n,
                                uint8_t *d_out, void *stream);

/* pa_align_batch over 2-bit packed host sequences: pair k is bases
 * [off1[k], off1[k+1]) of the packed stream seq1_words against bases
 * [off2[k], off2[k+1]) of seq2_words.  Only the packed words cross to the
 * device (a quarter of the bytes); they are unpacked there into ACGT and
 * aligned exactly as pa_align_batch would align the letters. */
pa_status pa_align_batch_packed(pa_ctx *ctx, const pa_config *config,
                                const uint32_t *seq1_words, const uint64_t *off1,
                                const uint32_t *seq2_words, const uint64_t *off2,
                                uint64_t n_pairs, pa_result *out, pa_stats *stats);

/* FASTA / FASTQ reader (the record format of test/data/in.fastq; FASTA with
 * sequences over several lines).  The format is taken from the first
 * non-blank byte ('>' or '@').  Sequence bytes are kept as they are (no case
 * change); line ends may be LF or CRLF; a FASTQ record is '@name', sequence
 * line(s), '+' (optionally the name again), quality line(s) of the sequence's
 * length.  On a malformed file the status is PA_ERR_INVALID_ARGUMENT and `err`
 * (err_len bytes, may be NULL) holds the line number and the reason. */
typedef struct pa_seqfile pa_seqfile;
pa_status pa_seqfile_read(const char *path, pa_seqfile **out, char *err, size_t err_len);
pa_status pa_seqfile_parse(const char *text, uint64_t len, pa_seqfile **out, char *err, size_t err_len);
uint64_t pa_seqfile_count(const pa_seqfile *f);
/* concatenated sequence bytes, and count + 1 offsets into them */
const uint8_t *pa_seqfile_sequences(const pa_seqfile *f);
const uint64_t *pa_seqfile_offsets(const pa_seqfile *f);
/* FASTQ: the qualities, concatenated with the same offsets; FASTA: NULL */
const uint8_t *pa_seqfile_qualities(const pa_seqfile *f);
/* record i's name: the header line after '>' / '@', up to the line end */
const char *pa_seqfile_name(const pa_seqfile *f, uint64_t i);
void pa_seqfile_free(pa_seqfile *f);

const char *pa_status_string(pa_status status);
/* Message of the last error on this context (empty string if none). */
const char *pa_last_error(const pa_ctx *ctx);
int pa_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* PAIRWISE_ALIGNER_GB300_H */
