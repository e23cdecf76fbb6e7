// C entry points over the reference's own CPU code, compiled from its sources
// into oracle/_ref/libcosma_ref.so (test infrastructure only):
//   ref_local_multiply_cpu_d  cosma::local_multiply_cpu<double>  (src/cosma/local_multiply.cpp:278-297)
//   ref_local_multiply_d      cosma::local_multiply<double> on a CPU build: cosma::gemm
//                             (src/cosma/local_multiply.cpp:300-381, src/cosma/blas.cpp:24-48)
//   ref_gemm_z                cosma::gemm for complex<double> (src/cosma/blas.cpp:50-75)
//   ref_numroc                cosma::scalapack::numroc (src/cosma/scalapack.cpp:49-88)
// The CBLAS functions the reference's blas.cpp calls are defined here on top
// of scipy's OpenBLAS (scipy_cblas_*), loaded at run time.
#include <cosma/blas.hpp>
#include <cosma/local_multiply.hpp>
#include <cosma/scalapack.hpp>

#include <cblas.h>
#include <dlfcn.h>

#include <complex>
#include <cstdio>
#include <cstdlib>

namespace cosma {
template <typename Scalar>
cosma_context<Scalar>* get_context_instance() {
    static cosma_context<Scalar> ctx;
    return &ctx;
}
template cosma_context<double>* get_context_instance<double>();
template cosma_context<float>* get_context_instance<float>();
template cosma_context<std::complex<double>>* get_context_instance<std::complex<double>>();
template cosma_context<std::complex<float>>* get_context_instance<std::complex<float>>();
namespace blacs {
// never reached on one rank without BLACS; present for the linker only
void Cblacs_pcoord(int, int, int* r, int* c) { *r = *c = 0; }
void Cblacs_get(int, int, int* v) { *v = 0; }
void Cblacs_gridinfo(int, int* a, int* b, int* c, int* d) { *a = *b = 1; *c = *d = 0; }
MPI_Comm Cblacs2sys_handle(int) { return 0; }
}  // namespace blacs
}  // namespace cosma

namespace {
void* openblas() {
    static void* h = [] {
        const char* path = std::getenv("COSMA_REF_OPENBLAS");
        void* p = path ? dlopen(path, RTLD_NOW | RTLD_LOCAL) : nullptr;
        if (!p) std::fprintf(stderr, "ref_shim: set COSMA_REF_OPENBLAS to scipy's OpenBLAS library\n");
        return p;
    }();
    return h;
}
template <class F>
F sym(const char* name) {
    void* h = openblas();
    void* f = h ? dlsym(h, name) : nullptr;
    if (!f) {
        std::fprintf(stderr, "ref_shim: %s not found\n", name);
        std::abort();
    }
    return reinterpret_cast<F>(f);
}
}  // namespace

extern "C" {
void cblas_dgemm(CBLAS_ORDER o, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb, int m, int n, int k, double alpha,
                 const double* a, int lda, const double* b, int ldb, double beta, double* c, int ldc) {
    using Fn = void (*)(int, int, int, int, int, int, double, const double*, int, const double*, int, double, double*,
                        int);
    static Fn f = sym<Fn>("scipy_cblas_dgemm");
    f(o, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}
void cblas_sgemm(CBLAS_ORDER o, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb, int m, int n, int k, float alpha,
                 const float* a, int lda, const float* b, int ldb, float beta, float* c, int ldc) {
    using Fn = void (*)(int, int, int, int, int, int, float, const float*, int, const float*, int, float, float*, int);
    static Fn f = sym<Fn>("scipy_cblas_sgemm");
    f(o, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}
void cblas_zgemm(CBLAS_ORDER o, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb, int m, int n, int k, const void* alpha,
                 const void* a, int lda, const void* b, int ldb, const void* beta, void* c, int ldc) {
    using Fn = void (*)(int, int, int, int, int, int, const void*, const void*, int, const void*, int, const void*,
                        void*, int);
    static Fn f = sym<Fn>("scipy_cblas_zgemm");
    f(o, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}
void cblas_cgemm(CBLAS_ORDER o, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb, int m, int n, int k, const void* alpha,
                 const void* a, int lda, const void* b, int ldb, const void* beta, void* c, int ldc) {
    using Fn = void (*)(int, int, int, int, int, int, const void*, const void*, int, const void*, int, const void*,
                        void*, int);
    static Fn f = sym<Fn>("scipy_cblas_cgemm");
    f(o, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}

void ref_local_multiply_cpu_d(double* a, double* b, double* c, int m, int n, int k, double alpha, double beta) {
    cosma::local_multiply_cpu<double>(a, b, c, m, n, k, alpha, beta);
}
void ref_local_multiply_d(double* a, double* b, double* c, int m, int n, int k, double alpha, double beta) {
    cosma::local_multiply<double>(a, b, c, m, n, k, alpha, beta, true);
}
void ref_gemm_z(int m, int n, int k, const double* alpha, const double* a, int lda, const double* b, int ldb,
                const double* beta, double* c, int ldc) {
    const std::complex<double> al(alpha[0], alpha[1]), be(beta[0], beta[1]);
    cosma::gemm(m, n, k, al, reinterpret_cast<const std::complex<double>*>(a), lda,
                reinterpret_cast<const std::complex<double>*>(b), ldb, be, reinterpret_cast<std::complex<double>*>(c),
                ldc);
}
int ref_numroc(int n, int nb, int iproc, int isrc, int nprocs) {
    return cosma::scalapack::numroc(n, nb, iproc, isrc, nprocs);
}
}
