// Batched persistent kernel with 2 tile buffers per CTA.
#include "batch_kernel.cuh"

namespace falx {

int batch_occupancy_nb2(int &blocks, size_t &smem) {
    const void *fn = (const void *)batch_kernel<2>;
    smem = sizeof(BatchSmem<2>);
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, kThreads, smem) != cudaSuccess) {
        (void)cudaGetLastError();
        return FALX_ERR_CUDA;
    }
    return FALX_OK;
}

cudaError_t batch_launch_nb2(const cudaLaunchConfig_t &lc, void **args) {
    return cudaLaunchKernelExC(&lc, (const void *)batch_kernel<2>, args);
}

}  // namespace falx
