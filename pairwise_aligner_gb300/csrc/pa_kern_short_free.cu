// pa_kern_short_free.cu -- instantiations of the short-pair s16x2 kernel, global mode with
// free end gaps (16 rows per thread only).
#include "pa_kern_short.cuh"

namespace pa {
int dp_short_occupancy_free(int G) { return occ_short_gb<M_GLOBAL_FREE>(G, 0); }
void dp_short_launch_free(int G, int grid, cudaStream_t st, const DpLaunch &L, const DpParams &P)
{
    go_short_gb<M_GLOBAL_FREE>(G, 0, grid, st, L, P);
}
}  // namespace pa
