// pa_kern_short_global.cu -- instantiations of the short-pair s16x2 kernel, global mode with
// penalised end gaps.
#include "pa_kern_short.cuh"

namespace pa {
int dp_short_occupancy_global(int G, int form) { return occ_short_gb<M_GLOBAL>(G, form); }
void dp_short_launch_global(int G, int form, int grid, cudaStream_t st, const DpLaunch &L, const DpParams &P)
{
    go_short_gb<M_GLOBAL>(G, form, grid, st, L, P);
}
}  // namespace pa
