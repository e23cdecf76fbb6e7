// C++ shims with the reference's names over the C ABI of cosma_gb300.h.
//
// They mirror the call shapes a COSMA maintainer already has:
//   gpu::make_context<T>(streams, tile_m, tile_n, tile_k)  (src/cosma/context.cpp:24-25,45)
//   gpu::gemm(ctx, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc,
//             pin_host_buffers, copy_c_back)               (src/cosma/local_multiply.cpp:245-260)
//   cosma::local_multiply(ctx, a, b, c, m, n, k, alpha, beta, copy_c_back)
//                                                           (src/cosma/local_multiply.hpp:6-49)
// and, like the reference, report errors by throwing (std::runtime_error
// carrying the library's message).  Header-only; link libcosma_gb300.so.
#pragma once

#include <complex>
#include <memory>
#include <stdexcept>
#include <string>

#include "cosma_gb300.h"

namespace cosma_gb300 {

inline void check(int status) {
    if (status != COSMA_GPU_SUCCESS)
        throw std::runtime_error(std::string("cosma_gb300: ") + cosma_gpu_last_error_string());
}

template <class T> struct scalar_tag;
template <> struct scalar_tag<float> { static constexpr char value = 's'; };
template <> struct scalar_tag<double> { static constexpr char value = 'd'; };
template <> struct scalar_tag<std::complex<float>> { static constexpr char value = 'c'; };
template <> struct scalar_tag<std::complex<double>> { static constexpr char value = 'z'; };

namespace gpu {

// Owns a cosma_gpu_mm_handle: device tile rings, streams, method.
template <class T>
class mm_handle {
public:
    mm_handle(int streams, int tile_m, int tile_n, int tile_k)
        : h_(cosma_gpu_tmm_make_context(scalar_tag<T>::value, streams, tile_m, tile_n, tile_k)) {
        if (!h_) check(cosma_gpu_last_error());
    }
    ~mm_handle() { cosma_gpu_tmm_destroy_context(h_); }
    mm_handle(const mm_handle&) = delete;
    mm_handle& operator=(const mm_handle&) = delete;

    cosma_gpu_mm_handle* get() const { return h_; }
    void set_method(int method, int ozaki_slices = 0) { check(cosma_gpu_tmm_set_method(h_, method, ozaki_slices)); }
    T* get_full_device_buffer_c() const { return static_cast<T*>(cosma_gpu_tmm_device_buffer_c(h_)); }

private:
    cosma_gpu_mm_handle* h_;
};

template <class T>
std::unique_ptr<mm_handle<T>> make_context(int streams = 0, int tile_m = 0, int tile_n = 0, int tile_k = 0) {
    return std::unique_ptr<mm_handle<T>>(new mm_handle<T>(streams, tile_m, tile_n, tile_k));
}

inline void gemm(mm_handle<float>& ctx, char ta, char tb, int m, int n, int k, float alpha, const float* A, int lda,
                 const float* B, int ldb, float beta, float* C, int ldc, bool pin_host_buffers = true,
                 bool copy_c_back = true) {
    check(cosma_gpu_tmm_gemm_s(ctx.get(), ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, pin_host_buffers,
                               copy_c_back));
}
inline void gemm(mm_handle<double>& ctx, char ta, char tb, int m, int n, int k, double alpha, const double* A,
                 int lda, const double* B, int ldb, double beta, double* C, int ldc, bool pin_host_buffers = true,
                 bool copy_c_back = true) {
    check(cosma_gpu_tmm_gemm_d(ctx.get(), ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, pin_host_buffers,
                               copy_c_back));
}
inline void gemm(mm_handle<std::complex<float>>& ctx, char ta, char tb, int m, int n, int k,
                 std::complex<float> alpha, const std::complex<float>* A, int lda, const std::complex<float>* B,
                 int ldb, std::complex<float> beta, std::complex<float>* C, int ldc, bool pin_host_buffers = true,
                 bool copy_c_back = true) {
    check(cosma_gpu_tmm_gemm_c(ctx.get(), ta, tb, m, n, k, reinterpret_cast<const float*>(&alpha),
                               reinterpret_cast<const float*>(A), lda, reinterpret_cast<const float*>(B), ldb,
                               reinterpret_cast<const float*>(&beta), reinterpret_cast<float*>(C), ldc,
                               pin_host_buffers, copy_c_back));
}
inline void gemm(mm_handle<std::complex<double>>& ctx, char ta, char tb, int m, int n, int k,
                 std::complex<double> alpha, const std::complex<double>* A, int lda,
                 const std::complex<double>* B, int ldb, std::complex<double> beta, std::complex<double>* C,
                 int ldc, bool pin_host_buffers = true, bool copy_c_back = true) {
    check(cosma_gpu_tmm_gemm_z(ctx.get(), ta, tb, m, n, k, reinterpret_cast<const double*>(&alpha),
                               reinterpret_cast<const double*>(A), lda, reinterpret_cast<const double*>(B), ldb,
                               reinterpret_cast<const double*>(&beta), reinterpret_cast<double*>(C), ldc,
                               pin_host_buffers, copy_c_back));
}

}  // namespace gpu

// cosma::local_multiply on a one-rank strategy: C = alpha*A*B + beta*C with
// A m x k, B k x n, C m x n, all column-major with ld = rows.  ctx == nullptr
// uses the per-type singleton context, as the reference's context-less
// overload does.
inline void local_multiply(gpu::mm_handle<float>* ctx, float* a, float* b, float* c, int m, int n, int k,
                           float alpha, float beta, bool copy_c_back = true) {
    check(cosma_gpu_local_multiply_s(ctx ? ctx->get() : nullptr, a, b, c, m, n, k, alpha, beta, copy_c_back));
}
inline void local_multiply(gpu::mm_handle<double>* ctx, double* a, double* b, double* c, int m, int n, int k,
                           double alpha, double beta, bool copy_c_back = true) {
    check(cosma_gpu_local_multiply_d(ctx ? ctx->get() : nullptr, a, b, c, m, n, k, alpha, beta, copy_c_back));
}
inline void local_multiply(gpu::mm_handle<std::complex<float>>* ctx, std::complex<float>* a, std::complex<float>* b,
                           std::complex<float>* c, int m, int n, int k, std::complex<float> alpha,
                           std::complex<float> beta, bool copy_c_back = true) {
    check(cosma_gpu_local_multiply_c(ctx ? ctx->get() : nullptr, reinterpret_cast<float*>(a),
                                     reinterpret_cast<float*>(b), reinterpret_cast<float*>(c), m, n, k,
                                     reinterpret_cast<const float*>(&alpha), reinterpret_cast<const float*>(&beta),
                                     copy_c_back));
}
inline void local_multiply(gpu::mm_handle<std::complex<double>>* ctx, std::complex<double>* a,
                           std::complex<double>* b, std::complex<double>* c, int m, int n, int k,
                           std::complex<double> alpha, std::complex<double> beta, bool copy_c_back = true) {
    check(cosma_gpu_local_multiply_z(ctx ? ctx->get() : nullptr, reinterpret_cast<double*>(a),
                                     reinterpret_cast<double*>(b), reinterpret_cast<double*>(c), m, n, k,
                                     reinterpret_cast<const double*>(&alpha), reinterpret_cast<const double*>(&beta),
                                     copy_c_back));
}

}  // namespace cosma_gb300
