// pa_band_labels.cu -- training labels of the band predictor from the full GPU DP.
//
// For a global alignment the optimal path crosses column i_c = c*m/9 (c = 1..8)
// of sequence1 at some row j.  A forward DP keeps H(i_c, j) for all j; a
// second DP on the reversed pair gives the best suffix score from (i_c, j);
// their sum is the best score of a path through (i_c, j), and its argmax (the
// smallest j on ties) is the label: the diagonal j - i_c.  Both passes are the
// s32 byte-compare wavefront kernel (dp_kernel<L32, ..., GEN>) in its label
// modes.  This is the traceback-free labeller the band predictor is trained on;
// it has no counterpart in the reference, which never computes coordinates.
#include <algorithm>
#include <cstring>
#include <vector>

#include "pa_dp.cuh"

namespace pa {

void band_labels_launch(bool reverse, int grid, cudaStream_t st, const DpLaunch &L, const DpParams &P)
{
    if (reverse) dp_kernel<L32, 16, M_LABEL_REV, true, 0><<<grid, kBlock, 0, st>>>(L, P);
    else dp_kernel<L32, 16, M_LABEL_FWD, true, 0><<<grid, kBlock, 0, st>>>(L, P);
}

// Long pairs: whole blocks per pair (CTA mode), L.ring holding grid * 8 rows.
void band_labels_cta_launch(bool reverse, int grid, cudaStream_t st, const DpLaunch &L, const DpParams &P)
{
    if (reverse) dp_kernel_cta<L32, 16, M_LABEL_REV, true, 0><<<grid, kBlock, 0, st>>>(L, P);
    else dp_kernel_cta<L32, 16, M_LABEL_FWD, true, 0><<<grid, kBlock, 0, st>>>(L, P);
}

int band_labels_cta_occupancy()
{
    int a = 0, b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, dp_kernel_cta<L32, 16, M_LABEL_FWD, true, 0>, kBlock, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, dp_kernel_cta<L32, 16, M_LABEL_REV, true, 0>, kBlock, 0);
    return std::max(1, std::min(a, b));
}

int band_labels_occupancy()
{
    int a = 0, b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, dp_kernel<L32, 16, M_LABEL_FWD, true, 0>, kBlock, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, dp_kernel<L32, 16, M_LABEL_REV, true, 0>, kBlock, 0);
    return std::max(1, std::min(a, b));
}

}  // namespace pa
