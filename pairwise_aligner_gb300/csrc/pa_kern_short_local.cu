// pa_kern_short_local.cu -- instantiations of the short-pair s16x2 kernel, local mode.
#include "pa_kern_short.cuh"

namespace pa {
int dp_short_occupancy_local(int G, int form) { return occ_short_gb<M_LOCAL>(G, form); }
void dp_short_launch_local(int G, int form, int grid, cudaStream_t st, const DpLaunch &L, const DpParams &P)
{
    go_short_gb<M_LOCAL>(G, form, grid, st, L, P);
}
}  // namespace pa
