// Method dispatch for device-pointer GEMMs and the *_device C-ABI entry points.
#include "common.cuh"
#include "runtime.hpp"

namespace cgb {

int DeviceBuffer::reserve(size_t need, cudaStream_t stream) {
    if (need <= bytes) return COSMA_GPU_SUCCESS;
    release();
    // 2 MiB granularity keeps small size changes from reallocating.
    size_t rounded = (need + (2u << 20) - 1) & ~size_t((2u << 20) - 1);
    (void)stream;
    const bool injected = inject_fault(kFaultDeviceAlloc);
    cudaError_t e = injected ? cudaErrorMemoryAllocation : cudaMalloc(&ptr, rounded);
    if (e != cudaSuccess) {
        ptr = nullptr;
        bytes = 0;
        return cuda_status(e, injected ? "cudaMalloc(workspace) [injected fault]" : "cudaMalloc(workspace)");
    }
    bytes = rounded;
    return COSMA_GPU_SUCCESS;
}

void DeviceBuffer::release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
}

static bool is_zero(const double* v, Scalar s) { return v[0] == 0.0 && (!scalar_complex(s) || v[1] == 0.0); }

int gemm_device(const GemmDesc& g, int method, int ozaki_slices, cudaStream_t stream, cosma_gpu_ozaki_info* info) {
    if (info) *info = cosma_gpu_ozaki_info{0, 0, 0, 0, 0.0, 0.0, 0.0, 0, 0};
    if (g.m < 0 || g.n < 0 || g.k < 0) return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "gemm: negative size");
    if (g.opa < 0 || g.opb < 0) return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "gemm: op must be N, T or C");
    if (g.m == 0 || g.n == 0) return COSMA_GPU_SUCCESS;
    const int64_t a_rows = g.opa == 0 ? g.m : g.k, b_rows = g.opb == 0 ? g.k : g.n;
    if (g.ldc < (g.m > 1 ? g.m : 1) || (g.k > 0 && (g.lda < (a_rows > 1 ? a_rows : 1) || g.ldb < (b_rows > 1 ? b_rows : 1))))
        return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "gemm: leading dimension too small");
    // k == 0 or alpha == 0: C <- beta * C (cosma_pxgemm.cpp:41-46 semantics)
    if (g.k == 0 || is_zero(g.alpha, g.scalar)) return scale_matrix_device(g.scalar, g.m, g.n, g.beta, g.C, g.ldc, stream);
    // AUTO: the reference's native arithmetic, except for real single precision,
    // which runs 3xBF16 on the tensor cores (FP32 accuracy; the FP64 pipe that the
    // native kernel uses for FP32 inputs is ~60x slower on GB300).
    if (method == COSMA_GPU_METHOD_AUTO)
        method = g.scalar == Scalar::S ? COSMA_GPU_METHOD_BF16X3 : COSMA_GPU_METHOD_NATIVE;
    if (method == COSMA_GPU_METHOD_OZAKI || method == COSMA_GPU_METHOD_OZAKI2) {
        const bool crt = method == COSMA_GPU_METHOD_OZAKI2;
        if (g.scalar == Scalar::D)
            return crt ? ozaki2_dgemm(g, ozaki_slices, stream, info) : ozaki_dgemm(g, ozaki_slices, stream, info);
        if (g.scalar == Scalar::Z)
            return crt ? ozaki2_zgemm(g, ozaki_slices, stream, info) : ozaki_zgemm(g, ozaki_slices, stream, info);
        // single precision: the tensor-core form accurate to FP32 (real), or
        // the native kernel (complex), so that a process-wide Ozaki default
        // also serves psgemm / pcgemm callers
        if (g.scalar == Scalar::S) return bf16x3_sgemm(g, stream);
        return native_gemm(g, stream);
    }
    if (method == COSMA_GPU_METHOD_BF16X3) {
        if (g.scalar == Scalar::S) return bf16x3_sgemm(g, stream);
        return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "gemm: the BF16x3 method is implemented for float");
    }
    if (method != COSMA_GPU_METHOD_NATIVE) return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "gemm: unknown method");
    return native_gemm(g, stream);
}

static GemmDesc make_desc(Scalar s, char ta, char tb, int64_t m, int64_t n, int64_t k, const double* alpha,
                          const void* A, int64_t lda, const void* B, int64_t ldb, const double* beta, void* C,
                          int64_t ldc) {
    GemmDesc g;
    g.scalar = s;
    g.opa = parse_op(ta);
    g.opb = parse_op(tb);
    g.m = m; g.n = n; g.k = k;
    g.alpha[0] = alpha[0]; g.alpha[1] = scalar_complex(s) ? alpha[1] : 0.0;
    g.beta[0] = beta[0]; g.beta[1] = scalar_complex(s) ? beta[1] : 0.0;
    g.A = A; g.lda = lda; g.B = B; g.ldb = ldb; g.C = C; g.ldc = ldc;
    return g;
}

GemmDesc make_gemm_desc(Scalar s, char ta, char tb, int64_t m, int64_t n, int64_t k, const double* alpha,
                        const void* A, int64_t lda, const void* B, int64_t ldb, const double* beta, void* C,
                        int64_t ldc) {
    return make_desc(s, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}

}  // namespace cgb

extern "C" {

int cosma_gpu_dgemm_device(int method, char ta, char tb, int64_t m, int64_t n, int64_t k, double alpha,
                           const double* A, int64_t lda, const double* B, int64_t ldb, double beta, double* C,
                           int64_t ldc, void* stream) {
    cgb::clear_error();
    double a[2] = {alpha, 0}, b[2] = {beta, 0};
    auto g = cgb::make_desc(cgb::Scalar::D, ta, tb, m, n, k, a, A, lda, B, ldb, b, C, ldc);
    return cgb::gemm_device(g, method, 0, (cudaStream_t)stream, nullptr);
}

int cosma_gpu_sgemm_device(int method, char ta, char tb, int64_t m, int64_t n, int64_t k, float alpha,
                           const float* A, int64_t lda, const float* B, int64_t ldb, float beta, float* C,
                           int64_t ldc, void* stream) {
    cgb::clear_error();
    double a[2] = {alpha, 0}, b[2] = {beta, 0};
    auto g = cgb::make_desc(cgb::Scalar::S, ta, tb, m, n, k, a, A, lda, B, ldb, b, C, ldc);
    return cgb::gemm_device(g, method, 0, (cudaStream_t)stream, nullptr);
}

int cosma_gpu_zgemm_device(int method, char ta, char tb, int64_t m, int64_t n, int64_t k, const double* alpha,
                           const double* A, int64_t lda, const double* B, int64_t ldb, const double* beta,
                           double* C, int64_t ldc, void* stream) {
    cgb::clear_error();
    auto g = cgb::make_desc(cgb::Scalar::Z, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    return cgb::gemm_device(g, method, 0, (cudaStream_t)stream, nullptr);
}

int cosma_gpu_cgemm_device(int method, char ta, char tb, int64_t m, int64_t n, int64_t k, const float* alpha,
                           const float* A, int64_t lda, const float* B, int64_t ldb, const float* beta, float* C,
                           int64_t ldc, void* stream) {
    cgb::clear_error();
    double a[2] = {alpha[0], alpha[1]}, b[2] = {beta[0], beta[1]};
    auto g = cgb::make_desc(cgb::Scalar::C, ta, tb, m, n, k, a, A, lda, B, ldb, b, C, ldc);
    return cgb::gemm_device(g, method, 0, (cudaStream_t)stream, nullptr);
}

int cosma_gpu_dgemm_ozaki_device(char ta, char tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
                                 int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc,
                                 int slices, void* stream, cosma_gpu_ozaki_info* info) {
    cgb::clear_error();
    double a[2] = {alpha, 0}, b[2] = {beta, 0};
    auto g = cgb::make_desc(cgb::Scalar::D, ta, tb, m, n, k, a, A, lda, B, ldb, b, C, ldc);
    return cgb::gemm_device(g, COSMA_GPU_METHOD_OZAKI, slices, (cudaStream_t)stream, info);
}

int cosma_gpu_release_workspaces(void* stream) {
    cgb::clear_error();
    cgb::ozaki_release_stream((cudaStream_t)stream);
    cgb::ozaki2_release_stream((cudaStream_t)stream);
    cgb::bf16x3_release_stream((cudaStream_t)stream);
    return COSMA_GPU_SUCCESS;
}

int cosma_gpu_dgemm_ozaki2_device(char ta, char tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
                                  int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc,
                                  int moduli, void* stream, cosma_gpu_ozaki_info* info) {
    cgb::clear_error();
    double a[2] = {alpha, 0}, b[2] = {beta, 0};
    auto g = cgb::make_desc(cgb::Scalar::D, ta, tb, m, n, k, a, A, lda, B, ldb, b, C, ldc);
    return cgb::gemm_device(g, COSMA_GPU_METHOD_OZAKI2, moduli, (cudaStream_t)stream, info);
}

int cosma_gpu_zgemm_ozaki2_device(char ta, char tb, int64_t m, int64_t n, int64_t k, const double* alpha,
                                  const double* A, int64_t lda, const double* B, int64_t ldb, const double* beta,
                                  double* C, int64_t ldc, int moduli, void* stream, cosma_gpu_ozaki_info* info) {
    cgb::clear_error();
    auto g = cgb::make_desc(cgb::Scalar::Z, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    return cgb::gemm_device(g, COSMA_GPU_METHOD_OZAKI2, moduli, (cudaStream_t)stream, info);
}

int cosma_gpu_zgemm_ozaki_device(char ta, char tb, int64_t m, int64_t n, int64_t k, const double* alpha,
                                 const double* A, int64_t lda, const double* B, int64_t ldb, const double* beta,
                                 double* C, int64_t ldc, int slices, void* stream, cosma_gpu_ozaki_info* info) {
    cgb::clear_error();
    auto g = cgb::make_desc(cgb::Scalar::Z, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    return cgb::gemm_device(g, COSMA_GPU_METHOD_OZAKI, slices, (cudaStream_t)stream, info);
}

}  // extern "C"
