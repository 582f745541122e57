// pncg_mixed.cu — the mixed FP32/FP64 step kernel (pncg_mixed_kernel.cuh) with every term,
// instantiated, and the launch entry points that pick a batch's feature set; the reduced
// feature sets are instantiated in pncg_mixed_feat.cu (compiled in parallel).
#include "pncg_mixed_kernel.cuh"

namespace d2f {

template <int NT, int MINB>
static cudaError_t launch_v(const d2f_scene_desc &d, int grid, int smem, cudaStream_t st) {
    auto k = pncg_mixed_kernel<NT, MINB, 1, FEAT_ALL>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    k<<<grid, NT, smem, st>>>(d, mixed_ptrs(d));
    return cudaGetLastError();
}

template <int NT, int MINB>
static int occupancy_v(int smem) {
    int nb = 0;
    auto k = pncg_mixed_kernel<NT, MINB, 1, FEAT_ALL>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, NT, smem) != cudaSuccess) return 1;
    return nb > 0 ? nb : 1;
}

cudaError_t launch_mixed(int nt, int minb, const d2f_scene_desc &d, int grid, int smem, cudaStream_t st) {
    const int feat = mixed_features(d);
    if (feat != FEAT_ALL) return launch_mixed_feat(feat, nt, minb, d, grid, smem, st);
#define D2F_L(N, MB) if (nt == N && minb == MB) return launch_v<N, MB>(d, grid, smem, st);
    D2F_VARIANTS(D2F_L)
#undef D2F_L
    return cudaErrorInvalidConfiguration;
}

int occupancy_mixed(int nt, int minb, int smem, int feat) {
    if (feat != FEAT_ALL) return occupancy_mixed_feat(feat, nt, minb, smem);
#define D2F_O(N, MB) if (nt == N && minb == MB) return occupancy_v<N, MB>(smem);
    D2F_VARIANTS(D2F_O)
#undef D2F_O
    return 1;
}

}  // namespace d2f

extern "C" size_t d2f_mixed_scratch_bytes(int32_t N, int32_t T, int32_t Nb, int32_t n_col, int32_t n_rig) {
    return d2f::mixed_layout(N, T, Nb, n_col, n_rig).total;
}
