// pa_kern_cluster.cu -- instantiations and launchers of the cluster-mode DP kernel
// (the largest pairs: a cluster of kClusterBlocks co-scheduled blocks pipelines the
// row passes of one pair), for the plain modes and the band mode.
#include "pa_dp.cuh"

namespace pa {
namespace {
constexpr int kRowsCl = 16;

template <class V, int MODE, bool GEN>
void *cluster_fn()
{
    return (void *)dp_kernel_cluster<V, kRowsCl, MODE, GEN, 36, kClusterBlocks>;
}

void *pick(bool lanes16, bool gen, int mode)
{
    if (mode == M_BAND) return lanes16 ? cluster_fn<L16, M_BAND, false>() : cluster_fn<L32, M_BAND, false>();
    if (lanes16) {
        return mode == M_LOCAL ? cluster_fn<L16, M_LOCAL, false>()
                               : mode == M_GLOBAL ? cluster_fn<L16, M_GLOBAL, false>() : cluster_fn<L16, M_GLOBAL_FREE, false>();
    }
    if (gen) {
        return mode == M_LOCAL ? cluster_fn<L32, M_LOCAL, true>()
                               : mode == M_GLOBAL ? cluster_fn<L32, M_GLOBAL, true>() : cluster_fn<L32, M_GLOBAL_FREE, true>();
    }
    return mode == M_LOCAL ? cluster_fn<L32, M_LOCAL, false>()
                           : mode == M_GLOBAL ? cluster_fn<L32, M_GLOBAL, false>() : cluster_fn<L32, M_GLOBAL_FREE, false>();
}

cudaLaunchConfig_t config_of(int grid, cudaStream_t st, cudaLaunchAttribute *attr)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid, 1, 1);
    cfg.blockDim = dim3(kBlock, 1, 1);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kClusterBlocks;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cfg;
}
}  // namespace

// Blocks (a multiple of the cluster size) of a cluster-mode launch that are resident at once,
// at most `max_blocks`.
int dp_cluster_grid(bool lanes16, bool gen, int mode, int max_blocks)
{
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = config_of(max_blocks, nullptr, attr);
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, pick(lanes16, gen, mode), &cfg) != cudaSuccess || clusters < 1) {
        cudaGetLastError();
        clusters = 1;
    }
    const int grid = clusters * kClusterBlocks;
    const int cap = (max_blocks / kClusterBlocks) * kClusterBlocks;
    return grid < cap ? grid : (cap > 0 ? cap : kClusterBlocks);
}

cudaError_t dp_cluster_launch(bool lanes16, bool gen, int mode, int grid, cudaStream_t st, const DpLaunch &L,
                              const DpParams &P)
{
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = config_of(grid, st, attr);
    DpLaunch l = L;
    DpParams p = P;
    void *args[2] = {&l, &p};
    return cudaLaunchKernelExC(&cfg, pick(lanes16, gen, mode), args);
}

}  // namespace pa
