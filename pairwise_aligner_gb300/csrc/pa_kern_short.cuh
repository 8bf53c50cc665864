// pa_kern_short.cuh -- launcher body of the short-pair kernel for one mode, included by
// pa_kern_short_local.cu and pa_kern_short_global.cu with PA_SHORT_MODES defined.
#include "pa_short.cuh"
#include "pa_launch.h"

namespace pa {
namespace {

template <int MODE, int G, int MINB>
int occ_short()
{
    static int per_sm = -1;
    if (per_sm < 0) {
        int v = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, dp_short<MODE, G, MINB>, kBlock, 0);
        per_sm = v < 1 ? 1 : v;
    }
    return per_sm;
}

template <int MODE, int MINB>
int occ_short_g(int G)
{
    return G == 4 ? occ_short<MODE, 4, MINB>() : G == 8 ? occ_short<MODE, 8, MINB>()
                  : G == 16 ? occ_short<MODE, 16, MINB>() : occ_short<MODE, 32, MINB>();
}

template <int MODE>
int occ_short_gb(int G, int minb)
{
    return minb == 3 ? occ_short_g<MODE, 3>(G) : occ_short_g<MODE, 2>(G);
}

template <int MODE, int MINB>
void go_short_g(int G, int grid, cudaStream_t st, const DpLaunch &L, const DpParams &P)
{
    if (G == 4) dp_short<MODE, 4, MINB><<<grid, kBlock, 0, st>>>(L, P);
    else if (G == 8) dp_short<MODE, 8, MINB><<<grid, kBlock, 0, st>>>(L, P);
    else if (G == 16) dp_short<MODE, 16, MINB><<<grid, kBlock, 0, st>>>(L, P);
    else dp_short<MODE, 32, MINB><<<grid, kBlock, 0, st>>>(L, P);
}

template <int MODE>
void go_short_gb(int G, int minb, int grid, cudaStream_t st, const DpLaunch &L, const DpParams &P)
{
    if (minb == 3) go_short_g<MODE, 3>(G, grid, st, L, P);
    else go_short_g<MODE, 2>(G, grid, st, L, P);
}

}  // namespace
}  // namespace pa
