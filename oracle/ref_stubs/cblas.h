/* Stand-in CBLAS declarations (the standard C interface to the BLAS) for
 * compiling the reference's src/cosma/blas.cpp; oracle/ref_shim.cpp defines
 * them on top of scipy's OpenBLAS. */
#pragma once
#ifdef __cplusplus
extern "C" {
#endif
enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
void cblas_dgemm(enum CBLAS_ORDER o, enum CBLAS_TRANSPOSE ta, enum CBLAS_TRANSPOSE tb, int m, int n, int k,
                 double alpha, const double* a, int lda, const double* b, int ldb, double beta, double* c, int ldc);
void cblas_sgemm(enum CBLAS_ORDER o, enum CBLAS_TRANSPOSE ta, enum CBLAS_TRANSPOSE tb, int m, int n, int k,
                 float alpha, const float* a, int lda, const float* b, int ldb, float beta, float* c, int ldc);
void cblas_zgemm(enum CBLAS_ORDER o, enum CBLAS_TRANSPOSE ta, enum CBLAS_TRANSPOSE tb, int m, int n, int k,
                 const void* alpha, const void* a, int lda, const void* b, int ldb, const void* beta, void* c,
                 int ldc);
void cblas_cgemm(enum CBLAS_ORDER o, enum CBLAS_TRANSPOSE ta, enum CBLAS_TRANSPOSE tb, int m, int n, int k,
                 const void* alpha, const void* a, int lda, const void* b, int ldb, const void* beta, void* c,
                 int ldc);
#ifdef __cplusplus
}
#endif
