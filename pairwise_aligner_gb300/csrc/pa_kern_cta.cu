// pa_kern_cta.cu -- instantiations of the CTA-mode DP kernel (long pairs: the warps
// of a block pipeline the passes of one pair) and of the team kernel for long pairs with
// few passes (teams of 4 warps, two pairs per block).  Local mode uses the branch-free
// top input, global modes add the two-op vertical-gap chain; neither prefetches the
// score tables (measured 1-4 % faster without on GB300: the tables are loaded one
// column ahead and stay in L1).
#include "pa_dp.cuh"

namespace pa {
namespace {
constexpr int kRowsCta = 16;

template <class V, int MODE, bool GEN>
int occ_cta()
{
    static int per_sm = -1;
    if (per_sm < 0) {
        int v = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, dp_kernel_cta<V, kRowsCta, MODE, GEN, 36>,
                                                      kBlock, 0);
        per_sm = v < 1 ? 1 : v;
    }
    return per_sm;
}

template <class V, int MODE, bool GEN>
void go_cta(int grid, cudaStream_t st, const DpLaunch &L, const DpParams &P)
{
    dp_kernel_cta<V, kRowsCta, MODE, GEN, 36><<<grid, kBlock, 0, st>>>(L, P);
}

// Teams of kTeam warps per unit (two units per block) for block-mode pairs with few passes.
constexpr int kTeam = 4;

template <class V, int MODE, bool GEN>
int occ_team()
{
    static int per_sm = -1;
    if (per_sm < 0) {
        int v = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &v, dp_kernel_team<V, kRowsCta, MODE, GEN, 36, kTeam>, kBlock, 0);
        per_sm = v < 1 ? 1 : v;
    }
    return per_sm;
}

template <class V, int MODE, bool GEN>
void go_team(int grid, cudaStream_t st, const DpLaunch &L, const DpParams &P)
{
    dp_kernel_team<V, kRowsCta, MODE, GEN, 36, kTeam><<<grid, kBlock, 0, st>>>(L, P);
}

template <class V, bool GEN>
int occ_team_mode(int mode)
{
    return mode == M_LOCAL ? occ_team<V, M_LOCAL, GEN>() : mode == M_GLOBAL ? occ_team<V, M_GLOBAL, GEN>()
                                                                             : occ_team<V, M_GLOBAL_FREE, GEN>();
}

template <class V, bool GEN>
void go_team_mode(int mode, int grid, cudaStream_t st, const DpLaunch &L, const DpParams &P)
{
    if (mode == M_LOCAL) go_team<V, M_LOCAL, GEN>(grid, st, L, P);
    else if (mode == M_GLOBAL) go_team<V, M_GLOBAL, GEN>(grid, st, L, P);
    else go_team<V, M_GLOBAL_FREE, GEN>(grid, st, L, P);
}

template <class V, bool GEN>
int occ_cta_mode(int mode)
{
    return mode == M_LOCAL ? occ_cta<V, M_LOCAL, GEN>() : mode == M_GLOBAL ? occ_cta<V, M_GLOBAL, GEN>()
                                                                            : occ_cta<V, M_GLOBAL_FREE, GEN>();
}

template <class V, bool GEN>
void go_cta_mode(int mode, int grid, cudaStream_t st, const DpLaunch &L, const DpParams &P)
{
    if (mode == M_LOCAL) go_cta<V, M_LOCAL, GEN>(grid, st, L, P);
    else if (mode == M_GLOBAL) go_cta<V, M_GLOBAL, GEN>(grid, st, L, P);
    else go_cta<V, M_GLOBAL_FREE, GEN>(grid, st, L, P);
}
}  // namespace

int dp_cta_occupancy(bool lanes16, bool gen, int mode)
{
    if (lanes16) return occ_cta_mode<L16, false>(mode);
    return gen ? occ_cta_mode<L32, true>(mode) : occ_cta_mode<L32, false>(mode);
}

void dp_cta_launch(bool lanes16, bool gen, int mode, int grid, cudaStream_t st, const DpLaunch &L, const DpParams &P)
{
    if (lanes16) go_cta_mode<L16, false>(mode, grid, st, L, P);
    else if (gen) go_cta_mode<L32, true>(mode, grid, st, L, P);
    else go_cta_mode<L32, false>(mode, grid, st, L, P);
}

int dp_team_occupancy(bool lanes16, bool gen, int mode)
{
    if (lanes16) return occ_team_mode<L16, false>(mode);
    return gen ? occ_team_mode<L32, true>(mode) : occ_team_mode<L32, false>(mode);
}

void dp_team_launch(bool lanes16, bool gen, int mode, int grid, cudaStream_t st, const DpLaunch &L, const DpParams &P)
{
    if (lanes16) go_team_mode<L16, false>(mode, grid, st, L, P);
    else if (gen) go_team_mode<L32, true>(mode, grid, st, L, P);
    else go_team_mode<L32, false>(mode, grid, st, L, P);
}

}  // namespace pa
