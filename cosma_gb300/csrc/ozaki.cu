// FP64-accurate Ozaki-split GEMM (placeholder until the tcgen05 kernels land).
#include "common.cuh"
#include "runtime.hpp"

namespace cgb {
int ozaki_dgemm(const GemmDesc&, int, cudaStream_t, cosma_gpu_ozaki_info*) {
    return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "ozaki: not built yet");
}
}  // namespace cgb
