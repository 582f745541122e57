// pncg_mixed_feat.cu — the mixed step kernel (pncg_mixed_kernel.cuh) with reduced feature
// sets, instantiated for every launch shape: FEAT_IPC (elastic, colliders, friction, rigid
// modes, contact between bodies) and 0 (the same without contact between bodies).
#include "pncg_mixed_kernel.cuh"

namespace d2f {

template <int NT, int MINB, int FEAT>
static cudaError_t launch_f(const d2f_scene_desc &d, int grid, int smem, cudaStream_t st) {
    auto k = pncg_mixed_kernel<NT, MINB, 1, FEAT>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    k<<<grid, NT, smem, st>>>(d, mixed_ptrs(d));
    return cudaGetLastError();
}

template <int NT, int MINB, int FEAT>
static int occupancy_f(int smem) {
    int nb = 0;
    auto k = pncg_mixed_kernel<NT, MINB, 1, FEAT>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, NT, smem) != cudaSuccess) return 1;
    return nb > 0 ? nb : 1;
}

cudaError_t launch_mixed_feat(int feat, int nt, int minb, const d2f_scene_desc &d, int grid, int smem, cudaStream_t st) {
#define D2F_L(N, MB)                                                                                     \
    if (nt == N && minb == MB)                                                                           \
        return feat == FEAT_IPC ? launch_f<N, MB, FEAT_IPC>(d, grid, smem, st) : launch_f<N, MB, 0>(d, grid, smem, st);
    D2F_VARIANTS(D2F_L)
#undef D2F_L
    return cudaErrorInvalidConfiguration;
}

int occupancy_mixed_feat(int feat, int nt, int minb, int smem) {
#define D2F_O(N, MB) \
    if (nt == N && minb == MB) return feat == FEAT_IPC ? occupancy_f<N, MB, FEAT_IPC>(smem) : occupancy_f<N, MB, 0>(smem);
    D2F_VARIANTS(D2F_O)
#undef D2F_O
    return 1;
}

}  // namespace d2f
