// pa_kern_short_global.cu -- instantiations of the short-pair s16x2 kernel, global modes
// (penalised end gaps; free end gaps).
#include "pa_kern_short.cuh"

namespace pa {
int dp_short_occupancy_global(int G, int form, bool free_ends)
{
    return free_ends ? occ_short_gb<M_GLOBAL_FREE>(G, form) : occ_short_gb<M_GLOBAL>(G, form);
}
void dp_short_launch_global(int G, int form, bool free_ends, int grid, cudaStream_t st, const DpLaunch &L,
                            const DpParams &P)
{
    if (free_ends) go_short_gb<M_GLOBAL_FREE>(G, form, grid, st, L, P);
    else go_short_gb<M_GLOBAL>(G, form, grid, st, L, P);
}
}  // namespace pa
