// pa_launch.h -- host-side entry points of the DP kernel instantiations.
// Each kernel variant lives in its own translation unit (pa_kern_v*.cu) so that
// the library builds in parallel.
#pragma once
#include "pa_common.cuh"

namespace pa {

// lanes16: s16x2 lanes (else s32); gen: byte-compare scoring; mode: Mode.
// Returns the resident blocks per SM of the selected kernel.
int dp_occupancy(int variant, bool lanes16, bool gen, int mode);
void dp_launch(int variant, bool lanes16, bool gen, int mode, int grid, cudaStream_t stream, const DpLaunch &L,
               const DpParams &P);

// Short-pair kernel in s16x2 lanes with unitary DNA scores (pa_short.cuh): G in {4, 8, 16,
// 32} lanes per group, form 0 (16 rows of sequence2 per thread) or 1 (32 rows); L.slots must
// hold seq1_bytes + n_pairs column slots.
constexpr int kShortFormCount = 2;
int dp_short_occupancy(int G, int form, int mode);
void dp_short_launch(int G, int form, int mode, int grid, cudaStream_t stream, const DpLaunch &L, const DpParams &P);
inline bool dp_short_supports(int G) { return G == 4 || G == 8 || G == 16 || G == 32; }

// CTA mode (long pairs): whole blocks per pair; L.ring must hold grid * 8 rows of
// L.ring_stride cells.
int dp_cta_occupancy(bool lanes16, bool gen, int mode);
void dp_cta_launch(bool lanes16, bool gen, int mode, int grid, cudaStream_t stream, const DpLaunch &L,
                   const DpParams &P);
// The same pairs on teams of 4 warps (two units per block, same ring rows as CTA mode).
int dp_team_occupancy(bool lanes16, bool gen, int mode);
void dp_team_launch(bool lanes16, bool gen, int mode, int grid, cudaStream_t stream, const DpLaunch &L,
                    const DpParams &P);

// Cluster mode (the largest pairs): clusters of kClusterBlocks blocks per pair; the grid is a
// multiple of the cluster size and L.ring holds grid * 8 rows.  mode may be M_BAND.
int dp_cluster_grid(bool lanes16, bool gen, int mode, int max_blocks);
cudaError_t dp_cluster_launch(bool lanes16, bool gen, int mode, int grid, cudaStream_t stream, const DpLaunch &L,
                              const DpParams &P);

// Traceback (pa_traceback.cu): one warp per pair, direction words of pair q at dir + dir_off[q],
// passes * (m + 31) * 32 words with passes = ceil(n / kTracebackPassRows).
constexpr int kTracebackPassRows = 256;
struct TbLaunch {
    const uint8_t *seq1, *seq2;
    const uint64_t *off1, *off2;
    uint32_t first, count;          // the chunk: pairs first .. first + count - 1
    const uint64_t *dir_off;        // per chunk pair: first direction word
    uint32_t *dir;
    Cell *bnd;                      // pass boundary: (H(i, last row of the pass), Q(i, next row))
    pa_result *out;
    pa_alignment *aln;
    uint8_t *ops;                   // pair k at (off1[k] - off1[0]) + (off2[k] - off2[0]), m + n bytes
    const int8_t *rank;             // substitution matrix (or null: match / mismatch)
    const int32_t *matrix;
    int32_t dim;
};
int traceback_grid(int sm_count);
void traceback_launch(int grid, cudaStream_t stream, const TbLaunch &L, const DpParams &P);

}  // namespace pa
