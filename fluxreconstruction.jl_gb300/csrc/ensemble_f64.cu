// ensemble_f64.cu -- FP64 instantiation of the persistent ensemble kernel
// (compiled without implicit multiply-add contraction: bit-exact with the oracle).
#include "ensemble_kernels.cuh"

template <bool LEARNED> static int launch(const EnsArgs<double> &a, int grid, size_t smem, cudaStream_t st) {
    static fr_smem_optin optin; // raised per device whenever a launch needs more
    if (int rc = fr_raise_smem(k_ensemble<double, LEARNED>, smem, optin)) return rc;
    k_ensemble<double, LEARNED><<<grid, ENS_THREADS, smem, st>>>(a);
    FR_CUDA(cudaGetLastError());
    return FRGPU_OK;
}

int fr_ensemble_launch_f64(const void *args, int grid, size_t smem, cudaStream_t st) {
    const auto &a = *reinterpret_cast<const EnsArgs<double> *>(args);
    return a.mlp.P ? launch<true>(a, grid, smem, st) : launch<false>(a, grid, smem, st);
}

int fr_ensemble_occupancy_f64(size_t smem, bool learned, int *blocks) {
    if (learned) {
        FR_CUDA(cudaFuncSetAttribute(k_ensemble<double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        FR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_ensemble<double, true>, ENS_THREADS, smem));
    } else {
        FR_CUDA(cudaFuncSetAttribute(k_ensemble<double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        FR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_ensemble<double, false>, ENS_THREADS, smem));
    }
    return FRGPU_OK;
}

int fr_ensemble_features_f64(const void *args, int n, const long *d_eoff, float *d_feat, int *d_labels,
                             cudaStream_t st) {
    const auto &a = *reinterpret_cast<const EnsArgs<double> *>(args);
    k_ens_features<double><<<n, 128, 0, st>>>(a, d_eoff, d_feat, d_labels);
    FR_CUDA(cudaGetLastError());
    return FRGPU_OK;
}
