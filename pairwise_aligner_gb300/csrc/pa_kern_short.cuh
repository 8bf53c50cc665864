// pa_kern_short.cuh -- launcher body of the short-pair kernel, included by
// pa_kern_short_local.cu and pa_kern_short_global.cu.
#include "pa_short.cuh"
#include "pa_launch.h"

namespace pa {
namespace {

// Forms of the kernel: the rows of sequence2 a thread holds (0: 16, 1: 32).
template <int MODE, int G, int R>
int occ_short()
{
    static int per_sm = -1;
    if (per_sm < 0) {
        int v = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, dp_short<MODE, G, R>, kBlock, 0);
        per_sm = v < 1 ? 1 : v;
    }
    return per_sm;
}

template <int MODE, int R>
int occ_short_g(int G)
{
    return G == 4 ? occ_short<MODE, 4, R>() : G == 8 ? occ_short<MODE, 8, R>()
                  : G == 16 ? occ_short<MODE, 16, R>() : occ_short<MODE, 32, R>();
}

// The free-end-gap mode exists with 16 rows only (32 do not fit its registers).
template <int MODE>
int occ_short_gb(int G, int form)
{
    if constexpr (MODE != M_GLOBAL_FREE)
        if (form == 1) return occ_short_g<MODE, 32>(G);
    return occ_short_g<MODE, 16>(G);
}

template <int MODE, int R>
void go_short_g(int G, int grid, cudaStream_t st, const DpLaunch &L, const DpParams &P)
{
    if (G == 4) dp_short<MODE, 4, R><<<grid, kBlock, 0, st>>>(L, P);
    else if (G == 8) dp_short<MODE, 8, R><<<grid, kBlock, 0, st>>>(L, P);
    else if (G == 16) dp_short<MODE, 16, R><<<grid, kBlock, 0, st>>>(L, P);
    else dp_short<MODE, 32, R><<<grid, kBlock, 0, st>>>(L, P);
}

template <int MODE>
void go_short_gb(int G, int form, int grid, cudaStream_t st, const DpLaunch &L, const DpParams &P)
{
    if constexpr (MODE != M_GLOBAL_FREE)
        if (form == 1) return go_short_g<MODE, 32>(G, grid, st, L, P);
    go_short_g<MODE, 16>(G, grid, st, L, P);
}

}  // namespace
}  // namespace pa
