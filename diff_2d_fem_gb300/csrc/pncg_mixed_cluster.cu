// pncg_mixed_cluster.cu — the mixed-precision step kernel with several blocks per scene, for
// large scenes: one block cannot keep a scene of 10^5 nodes moving, while a thread-block cluster
// of 8, 12 or 16 blocks on as many SMs (pncg_mixed_kernel.cuh, CS > 1) splits every phase and
// combines its reductions through distributed shared memory, and the all-SM mode (CS == 0)
// spreads one scene over one block per SM, exchanging through global memory.
#include "pncg_mixed_kernel.cuh"

namespace d2f {

namespace {

template <int CS>
void cluster_config(cudaLaunchConfig_t &cfg, cudaLaunchAttribute &at, int grid, int smem, cudaStream_t st) {
    cfg = cudaLaunchConfig_t{};
    cfg.gridDim = dim3((unsigned)grid, 1, 1);
    cfg.blockDim = dim3(kClusterThreads, 1, 1);
    cfg.dynamicSmemBytes = (size_t)smem;
    cfg.stream = st;
    at = cudaLaunchAttribute{};
    at.id = cudaLaunchAttributeClusterDimension;
    at.val.clusterDim.x = CS;
    at.val.clusterDim.y = 1;
    at.val.clusterDim.z = 1;
    cfg.attrs = &at;
    cfg.numAttrs = 1;
}

template <int CS>
cudaError_t prepare(int smem) {
    auto k = pncg_mixed_kernel<kClusterThreads, 1, CS>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e == cudaSuccess && smem > 48 * 1024)
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    return e;
}

template <int CS>
cudaError_t launch_c(const d2f_scene_desc &d, int grid, int smem, cudaStream_t st) {
    cudaError_t e = prepare<CS>(smem);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute at;
    cluster_config<CS>(cfg, at, grid, smem, st);
    return cudaLaunchKernelEx(&cfg, pncg_mixed_kernel<kClusterThreads, 1, CS>, d, mixed_ptrs(d));
}

template <int CS>
int max_clusters_c(int smem) {
    if (prepare<CS>(smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute at;
    cluster_config<CS>(cfg, at, CS, smem, nullptr);
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, pncg_mixed_kernel<kClusterThreads, 1, CS>, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}
}  // namespace

// Every SM on one scene: a cooperative launch (all blocks co-resident, which the grid barrier
// needs) of one kClusterThreads block per SM. The blocks exchange through their part of the
// mixed scratch, whose barrier header starts at zero.
cudaError_t launch_mixed_grid(const d2f_scene_desc &d, int grid, int smem, cudaStream_t st) {
    if (grid > GX_MAX_BLOCKS) return cudaErrorInvalidConfiguration;
    auto k = pncg_mixed_kernel<kClusterThreads, 1, 0>;
    if (smem > 48 * 1024) {
        const cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
    }
    MixedPtrs mp = mixed_ptrs(d);
    cudaError_t e = cudaMemsetAsync(mp.gx, 0, 256, st);
    if (e != cudaSuccess) return e;
    d2f_scene_desc dd = d;
    void *args[2] = {&dd, &mp};
    return cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(k), dim3((unsigned)grid), dim3(kClusterThreads),
                                       args, (size_t)smem, st);
}

int grid_blocks_mixed(int smem) {
    int dev = 0, coop = 0, nsm = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || !coop) {
        cudaGetLastError();
        return 0;
    }
    auto k = pncg_mixed_kernel<kClusterThreads, 1, 0>;
    if (smem > 48 * 1024 && cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kClusterThreads, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return per_sm * nsm;
}

int grid_max_blocks() { return GX_MAX_BLOCKS; }

cudaError_t launch_mixed_cluster(int cs, const d2f_scene_desc &d, int grid, int smem, cudaStream_t st) {
    if (cs == 16) return launch_c<16>(d, grid, smem, st);
    if (cs == 12) return launch_c<12>(d, grid, smem, st);
    if (cs == 8) return launch_c<8>(d, grid, smem, st);
    return cudaErrorInvalidConfiguration;
}

int max_clusters_mixed(int cs, int smem) {
    if (cs == 16) return max_clusters_c<16>(smem);
    if (cs == 12) return max_clusters_c<12>(smem);
    if (cs == 8) return max_clusters_c<8>(smem);
    return 0;
}

}  // namespace d2f
