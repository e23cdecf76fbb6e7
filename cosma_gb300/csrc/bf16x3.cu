// 3xBF16 single-precision GEMM (placeholder until the tcgen05 kernels land).
#include "common.cuh"
#include "runtime.hpp"

namespace cgb {
int bf16x3_sgemm(const GemmDesc&, cudaStream_t) {
    return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "bf16x3: not built yet");
}
}  // namespace cgb
