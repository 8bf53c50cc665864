// pa_common.cuh -- shared device-side types of the GB300 affine-gap DP.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/pairwise_aligner_gb300.h"

namespace pa {

// Score-model parameters, uniform over a launch.  Signs follow the reference:
// a gap of length k scores gap_open + k * gap_ext (affine_dp_algorithm.hpp:149-155).
struct DpParams {
    int32_t match, mismatch, gap_open, gap_ext;
    int32_t local;
    int32_t first_column_free, first_row_free, last_column_free, last_row_free;
    int32_t floor16;      // lower clamp of s16 global lanes
    int32_t smax;         // max(match, mismatch, 0): best gain of one diagonal step
    int32_t spad;         // score of a padded cell, <= 0 and <= every real score
    int32_t shift;        // global modes store H(i, j) - shift * i with shift = smax (local: 0)
};

// Work classes produced by the classifier; the class is the top field of the bucket key.
// Classes 4..6 are the long-pair versions of 0..2, computed by whole blocks (CTA mode);
// 8..10 the largest pairs, computed by thread-block clusters (cluster mode); 12..14 long
// pairs with few row passes, computed by teams of 4 warps (two pairs per block).
enum Klass : uint32_t {
    K_S16 = 0, K_S32 = 1, K_GEN = 2, K_NONE = 3, K_S16L = 4, K_S32L = 5, K_GENL = 6,
    K_S16H = 8, K_S32H = 9, K_GENH = 10, K_S16M = 12, K_S32M = 13, K_GENM = 14
};
constexpr int kClasses = 15;
constexpr uint32_t kLongOffset = 4;
constexpr uint32_t kHugeOffset = 8;
constexpr uint32_t kMediumOffset = 12;      // block-mode pairs with few passes: teams of 4 warps
constexpr int kClusterBlocks = 4;            // blocks per cluster in cluster mode

constexpr int kKeyBits = 20;                 // 4 class | 6 pass | 10 length bits
constexpr uint32_t kBuckets = 1u << kKeyBits;
constexpr int kClassShift = 16;

// Boundary row cell between passes of one group: H and the downward gap of the
// last held row of a pass, per streamed column (both lanes packed for s16x2).
struct __align__(8) Cell {
    uint32_t h, e;
};

// One streamed column of a short-pair unit (s16x2 lanes, pa_short.cuh): the score tables
// of both lanes for the column's base and the top input of the current pass (H and the
// downward gap of the row above the pass's first row).
struct __align__(16) Slot {
    uint32_t ta, tb, h, e;
};

// Band of one pair (band mode): the centre line runs through (0, 0), the 8
// checkpoints (i_c, i_c + diag[c]) with i_c = (c + 1) * m / 9, and (m, n); the
// half-width tapers linearly from w_start at column 0 to w_min at column m.
struct BandSpec {
    int32_t diag[8];
    int32_t w_start, w_min;
    int32_t pad[2];
};

// Per-launch description of a DP class.
struct DpLaunch {
    const uint8_t *seq1;          // streamed sequences (raw bytes)
    const uint64_t *off1;
    const uint8_t *seq2;          // held sequences (raw bytes)
    const uint64_t *off2;
    const uint32_t *qtab;         // per query base 4-byte score table (+1 pad entry per pair)
    const uint32_t *order;        // pair ids, bucket-sorted
    const uint32_t *begin_ptr;    // first entry of this class in `order`
    const uint32_t *count_ptr;    // number of pairs of this class
    uint32_t *unit_counter;       // persistent-queue head
    pa_result *out;
    Cell *boundary;               // pass-boundary scratch: (seq1_bytes + n_pairs) cells
    uint32_t *rerun_list;         // s16 global results that failed their exactness check
    uint32_t *rerun_count;
    unsigned long long *dp_cells; // statistics: cells computed (incl. padding), may be null
    int32_t G;                    // threads per group (1..32, power of two)
    int32_t rerun;                // this launch consumes a rerun list
    // label modes (training data of the band predictor): H at 8 checkpoint columns
    int32_t *dump;                // forward pass: dump[dump_off[p] + c * (n + 1) + j] = H(i_c, j)
    const uint64_t *dump_off;     // per pair offset into dump
    int32_t *labels;              // reverse pass: 8 optimal-path diagonals (j - i_c) per pair
    // band mode: per-pass column windows {first, last} (1-based) of every pair, at
    // slot (off2[id] - off2[0]) / band_rows + id; the outcome of list position k goes
    // to band_code[k]: 0 certified, 1 not certified (widen), 3 redo in s32 lanes
    const int2 *band_win;
    BandSpec *band;
    uint8_t *band_code;
    int32_t *band_ub;             // optional: the largest exit bound per pair
    int32_t band_rows;            // rows per pass of the window table (G * R)
    int32_t band_round;
    // CTA mode: an optional list taken before `order` (the largest pairs, largest first)
    const uint32_t *lead_order;
    const uint32_t *lead_begin_ptr;
    const uint32_t *lead_count_ptr;
    // CTA mode (long pairs): each block owns ring rows of ring_stride cells, one per group
    Cell *ring;
    uint64_t ring_stride;
    int32_t team;                 // band mode, CTA launches: warps per unit (1, 2, 4 or 8; 0 means 8)
    uint32_t *error;              // error bits (kErrWaitTimeout), may be null
    // substitution-matrix scoring (byte-compare kernels): symbol -> rank (-1 invalid) and the
    // dim x dim scores, row = sequence1 rank; null for the unitary model
    const int8_t *rank_map;
    const int32_t *matrix;
    int32_t mdim;
    // short-pair kernel (pa_short.cuh): (seq1_bytes + n_pairs) column slots, pair k's at off1[k] + k
    Slot *slots;
    // CTA / team / cluster modes: polls a progress wait makes after its first look before it
    // gives up (pa_set_wait_limit; default 2^24)
    uint32_t spin_limit;
};

__device__ __forceinline__ uint32_t prmt(uint32_t a, uint32_t b, uint32_t sel)
{
    uint32_t d;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(sel));
    return d;
}

// 2-bit code of an upper-case DNA byte: A=0 C=1 G=2 T=3; valid iff the byte is one of them.
__device__ __forceinline__ uint32_t dna_code(uint32_t b) { return ((b >> 1) ^ (b >> 2)) & 3u; }
__device__ __forceinline__ bool dna_valid(uint32_t b)
{
    return ((0x54474341u >> (8u * dna_code(b))) & 0xffu) == b;
}

// 4-byte score table of a streamed base: match in byte code(b), mismatch elsewhere;
// a byte outside A/C/G/T matches nothing.
__device__ __forceinline__ uint32_t score_table(uint32_t b, uint32_t match4, uint32_t mis4)
{
    if (!dna_valid(b)) return mis4;
    return prmt(match4, mis4, 0x4444u ^ (4u << (4u * dna_code(b))));
}

// Border cell of the first row / column (affine_initialisation_strategy.hpp:38-51):
// index 0 -> 0, penalised index k -> open + ext * k, free -> 0.  The matching gap
// value is border + (open + ext).
__device__ __forceinline__ int32_t border(const DpParams &p, int free_rule, int64_t k)
{
    return (free_rule || k == 0) ? 0 : (int32_t)(p.gap_open + (int64_t)p.gap_ext * k);
}

}  // namespace pa
