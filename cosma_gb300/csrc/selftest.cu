// Self-test of the failure path that every tensor-core kernel relies on: a
// bounded wait that runs out.
//
// One thread waits on an mbarrier that nothing arrives on, through the same
// tc::mbar_wait the GEMM pipelines use, with a short limit.  The wait records
// its code in the device error word and the kernel returns; the host reads the
// word and reports COSMA_GPU_ERROR_DEVICE_TIMEOUT.  Nothing faults or traps and
// the CUDA context stays usable, which is what a real pipeline timeout
// (a lost TMA completion, a role that failed) must also guarantee.
#include "common.cuh"
#include "runtime.hpp"
#include "tc_common.cuh"

#include <string>

namespace cgb {

constexpr unsigned kDevSelfTestTimeout = 6;

__global__ void wait_timeout_kernel(unsigned* err, unsigned long long limit_ns) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar, 1);
        tc::fence_mbar_init();
        tc::mbar_wait(&bar, 0, err, kDevSelfTestTimeout, limit_ns);  // phase 0 never completes
    }
}

}  // namespace cgb

extern "C" int cosma_gpu_selftest_wait_timeout(unsigned long long limit_ns, void* stream) {
    using namespace cgb;
    clear_error();
    if (limit_ns < 1000000ull || limit_ns > 2000000000ull)
        return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "selftest: limit must be within [1 ms, 2 s]");
    cudaStream_t st = (cudaStream_t)stream;
    unsigned* err = nullptr;
    CGB_CUDA(cudaMalloc(&err, sizeof(unsigned)));
    unsigned host = 0;
    cudaError_t e = cudaMemsetAsync(err, 0, sizeof(unsigned), st);
    if (e == cudaSuccess) {
        wait_timeout_kernel<<<1, 32, 0, st>>>(err, limit_ns);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&host, err, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(err);
    if (e != cudaSuccess) return cuda_status(e, "selftest");
    if (host != kDevSelfTestTimeout)
        return set_error(COSMA_GPU_ERROR_INTERNAL, "selftest: the bounded wait did not report its timeout");
    return set_error(COSMA_GPU_ERROR_DEVICE_TIMEOUT,
                     "selftest: bounded wait gave up after " + std::to_string(limit_ns / 1000000ull) +
                         " ms as designed (device code " + std::to_string(host) + ")");
}
