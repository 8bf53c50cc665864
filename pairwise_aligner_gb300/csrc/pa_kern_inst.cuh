// pa_kern_inst.cuh -- per-variant launcher body, included once per pa_kern_v*.cu
// with PA_VARIANT defined.  Variant 0: three-operand H max, 2 blocks/SM;
// 1: short-chain H, 2 blocks/SM; 2: as 0 with at most 85 registers (3 blocks/SM);
// 3: as 0 with a branch-free top input and L1 prefetch of the score tables;
// 4: as 3 with the two-op vertical-gap chain; 5 and 6: as 3 and 4 with one prefetch per
// 8 columns that also covers the pass-boundary row; 7 and 8: as 3 and 4 without the
// score-table prefetch.
#ifndef PA_VARIANT
#error "define PA_VARIANT"
#endif

namespace {
constexpr int kVarMath = PA_VARIANT == 1   ? 1
                         : PA_VARIANT == 3 ? 4
                         : PA_VARIANT == 4 ? 12
                         : PA_VARIANT == 5 ? 20
                         : PA_VARIANT == 6 ? 28
                         : PA_VARIANT == 7 ? 36
                         : PA_VARIANT == 8 ? 44
                                           : 0;
constexpr int kVarMinB = PA_VARIANT == 2 ? 3 : 2;
constexpr int kRows = 16;

template <class V, int MODE, bool GEN>
int occ()
{
    static int per_sm = -1;
    if (per_sm < 0) {
        int v = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, dp_kernel<V, kRows, MODE, GEN, kVarMath, kVarMinB>, kBlock, 0);
        per_sm = v < 1 ? 1 : v;
    }
    return per_sm;
}

template <class V, int MODE, bool GEN>
void go(int grid, cudaStream_t st, const DpLaunch &L, const DpParams &P)
{
    dp_kernel<V, kRows, MODE, GEN, kVarMath, kVarMinB><<<grid, kBlock, 0, st>>>(L, P);
}

template <class V, bool GEN>
int occ_mode(int mode)
{
    return mode == M_LOCAL ? occ<V, M_LOCAL, GEN>() : mode == M_GLOBAL ? occ<V, M_GLOBAL, GEN>()
                                                                        : occ<V, M_GLOBAL_FREE, GEN>();
}

template <class V, bool GEN>
void go_mode(int mode, int grid, cudaStream_t st, const DpLaunch &L, const DpParams &P)
{
    if (mode == M_LOCAL) go<V, M_LOCAL, GEN>(grid, st, L, P);
    else if (mode == M_GLOBAL) go<V, M_GLOBAL, GEN>(grid, st, L, P);
    else go<V, M_GLOBAL_FREE, GEN>(grid, st, L, P);
}
}  // namespace

#define PA_CAT2(a, b) a##b
#define PA_CAT(a, b) PA_CAT2(a, b)

int PA_CAT(dp_occupancy_v, PA_VARIANT)(bool lanes16, bool gen, int mode)
{
    if (lanes16) return occ_mode<L16, false>(mode);
    return gen ? occ_mode<L32, true>(mode) : occ_mode<L32, false>(mode);
}

void PA_CAT(dp_launch_v, PA_VARIANT)(bool lanes16, bool gen, int mode, int grid, cudaStream_t st, const DpLaunch &L,
                                     const DpParams &P)
{
    if (lanes16) go_mode<L16, false>(mode, grid, st, L, P);
    else if (gen) go_mode<L32, true>(mode, grid, st, L, P);
    else go_mode<L32, false>(mode, grid, st, L, P);
}
