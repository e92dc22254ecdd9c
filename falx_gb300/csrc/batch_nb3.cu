// Batched persistent kernel with 3 tile buffers per CTA.
#include "batch_kernel.cuh"

namespace falx {

int batch_occupancy_nb3(int &blocks, size_t &smem) {
    const void *fn = (const void *)batch_kernel<3>;
    smem = sizeof(BatchSmem<3>);
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, kThreads, smem) != cudaSuccess) {
        (void)cudaGetLastError();
        return FALX_ERR_CUDA;
    }
    return FALX_OK;
}

cudaError_t batch_launch_nb3(const cudaLaunchConfig_t &lc, void **args) {
    return cudaLaunchKernelExC(&lc, (const void *)batch_kernel<3>, args);
}

}  // namespace falx
