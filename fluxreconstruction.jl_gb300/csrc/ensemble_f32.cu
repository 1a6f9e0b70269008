// ensemble_f32.cu -- FP32 instantiation of the persistent ensemble kernel.
#include "ensemble_kernels.cuh"

template <bool LEARNED> static int launch(const EnsArgs<float> &a, int grid, size_t smem, cudaStream_t st) {
    static fr_smem_optin optin; // raised per device whenever a launch needs more
    if (int rc = fr_raise_smem(k_ensemble<float, LEARNED>, smem, optin)) return rc;
    k_ensemble<float, LEARNED><<<grid, ENS_THREADS, smem, st>>>(a);
    FR_CUDA(cudaGetLastError());
    return FRGPU_OK;
}

int fr_ensemble_launch_f32(const void *args, int grid, size_t smem, cudaStream_t st) {
    const auto &a = *reinterpret_cast<const EnsArgs<float> *>(args);
    return a.mlp.P ? launch<true>(a, grid, smem, st) : launch<false>(a, grid, smem, st);
}

int fr_ensemble_occupancy_f32(size_t smem, bool learned, int *blocks) {
    if (learned) {
        FR_CUDA(cudaFuncSetAttribute(k_ensemble<float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        FR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_ensemble<float, true>, ENS_THREADS, smem));
    } else {
        FR_CUDA(cudaFuncSetAttribute(k_ensemble<float, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        FR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_ensemble<float, false>, ENS_THREADS, smem));
    }
    return FRGPU_OK;
}

int fr_ensemble_features_f32(const void *args, int n, const long *d_eoff, float *d_feat, int *d_labels,
                             cudaStream_t st) {
    const auto &a = *reinterpret_cast<const EnsArgs<float> *>(args);
    k_ens_features<float><<<n, 128, 0, st>>>(a, d_eoff, d_feat, d_labels);
    FR_CUDA(cudaGetLastError());
    return FRGPU_OK;
}
