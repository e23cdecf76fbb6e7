/*
 * oracle.c - CPU restatement of COSMA's one-rank GEMM path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the cosma_gb300 library links,
 * loads or calls this file; only tests/, the smoke check in
 * __graft_entry__.py and bench.py's CPU-baseline leg use it, as the checker.
 *
 * Parity status: the reference ships no golden vectors or known-answer files
 * (its tests compare two implementations on random inputs); this oracle is
 * pinned by (i) exact known-answer fixtures generated with rational
 * arithmetic (tests/golden/make_golden.py), (ii) the reference's own test
 * cases replayed with its own tolerance checker, and (iii) numpy/OpenBLAS,
 * the CPU BLAS the reference calls at P = 1.  The reference itself cannot be
 * built here (it needs MPI, ScaLAPACK and the COSTA / Tiled-MM sources,
 * which are not vendored).
 *
 * Build: cc -O2 -ffp-contract=off -fPIC -shared (oracle/build.py); the
 * explicit no-contraction flag keeps every a*b + c below rounded twice, as
 * written.
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <string.h>

typedef struct { double re, im; } zdouble;
typedef struct { float re, im; } cfloat;

static int op_code(char c) {
    switch (c) {
        case 'N': case 'n': return 0;
        case 'T': case 't': return 1;
        case 'C': case 'c': return 2;
    }
    return -1;
}

/* ------------------------------------------------------------------ GEMM */

/* Restates local_multiply_cpu (src/cosma/local_multiply.cpp:278-297):
 * for each (mi, ni): C *= beta; C += alpha * A * B over ki, column-major with
 * ld = m, k, m.  Note the reference multiplies C by beta even when beta == 0
 * (so a NaN in C survives); this restatement keeps that behaviour. */
void oracle_local_multiply_cpu_d(const double* a, const double* b, double* c, int m, int n, int k, double alpha,
                                 double beta) {
    for (int mi = 0; mi < m; ++mi)
        for (int ni = 0; ni < n; ++ni) {
            double cv = c[(int64_t)ni * m + mi];
            cv *= beta;
            for (int ki = 0; ki < k; ++ki) cv += alpha * a[(int64_t)ki * m + mi] * b[(int64_t)ni * k + ki];
            c[(int64_t)ni * m + mi] = cv;
        }
}

void oracle_local_multiply_cpu_z(const zdouble* a, const zdouble* b, zdouble* c, int m, int n, int k, zdouble alpha,
                                 zdouble beta) {
    for (int mi = 0; mi < m; ++mi)
        for (int ni = 0; ni < n; ++ni) {
            zdouble cv = c[(int64_t)ni * m + mi];
            zdouble t = {cv.re * beta.re - cv.im * beta.im, cv.re * beta.im + cv.im * beta.re};
            cv = t;
            for (int ki = 0; ki < k; ++ki) {
                zdouble x = a[(int64_t)ki * m + mi], y = b[(int64_t)ni * k + ki];
                zdouble ax = {alpha.re * x.re - alpha.im * x.im, alpha.re * x.im + alpha.im * x.re};
                cv.re += ax.re * y.re - ax.im * y.im;
                cv.im += ax.re * y.im + ax.im * y.re;
            }
            c[(int64_t)ni * m + mi] = cv;
        }
}

static double getd(const double* X, int op, int64_t ld, int64_t r, int64_t c) {
    return op == 0 ? X[r + c * ld] : X[c + r * ld];
}

/* BLAS dgemm semantics (cblas_dgemm ColMajor, src/cosma/blas.cpp:24-48):
 * C = alpha*op(A)*op(B) + beta*C; C is not read when beta == 0.
 * Accumulation: sequential over k in FP64. */
void oracle_gemm_d(char ta, char tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A, int64_t lda,
                   const double* B, int64_t ldb, double beta, double* C, int64_t ldc) {
    int oa = op_code(ta), ob = op_code(tb);
    for (int64_t j = 0; j < n; ++j)
        for (int64_t i = 0; i < m; ++i) {
            double s = 0.0;
            for (int64_t l = 0; l < k; ++l) s += getd(A, oa, lda, i, l) * getd(B, ob, ldb, l, j);
            double v = alpha * s;
            if (beta != 0.0) v += beta * C[i + j * ldc];
            C[i + j * ldc] = v;
        }
}

static zdouble getz(const zdouble* X, int op, int64_t ld, int64_t r, int64_t c) {
    zdouble v = op == 0 ? X[r + c * ld] : X[c + r * ld];
    if (op == 2) v.im = -v.im;
    return v;
}

void oracle_gemm_z(char ta, char tb, int64_t m, int64_t n, int64_t k, const double* alpha, const zdouble* A,
                   int64_t lda, const zdouble* B, int64_t ldb, const double* beta, zdouble* C, int64_t ldc) {
    int oa = op_code(ta), ob = op_code(tb);
    int beta_zero = beta[0] == 0.0 && beta[1] == 0.0;
    for (int64_t j = 0; j < n; ++j)
        for (int64_t i = 0; i < m; ++i) {
            double sr = 0.0, si = 0.0;
            for (int64_t l = 0; l < k; ++l) {
                zdouble x = getz(A, oa, lda, i, l), y = getz(B, ob, ldb, l, j);
                sr += x.re * y.re - x.im * y.im;
                si += x.re * y.im + x.im * y.re;
            }
            double vr = alpha[0] * sr - alpha[1] * si, vi = alpha[0] * si + alpha[1] * sr;
            if (!beta_zero) {
                zdouble c = C[i + j * ldc];
                vr += beta[0] * c.re - beta[1] * c.im;
                vi += beta[0] * c.im + beta[1] * c.re;
            }
            C[i + j * ldc].re = vr;
            C[i + j * ldc].im = vi;
        }
}

/* FP32 inputs, FP64 accumulation, one final rounding to FP32: a reference
 * more accurate than cblas_sgemm for checking FP32-accurate GPU paths. */
void oracle_gemm_s(char ta, char tb, int64_t m, int64_t n, int64_t k, float alpha, const float* A, int64_t lda,
                   const float* B, int64_t ldb, float beta, float* C, int64_t ldc) {
    int oa = op_code(ta), ob = op_code(tb);
    for (int64_t j = 0; j < n; ++j)
        for (int64_t i = 0; i < m; ++i) {
            double s = 0.0;
            for (int64_t l = 0; l < k; ++l) {
                float x = oa == 0 ? A[i + l * lda] : A[l + i * lda];
                float y = ob == 0 ? B[l + j * ldb] : B[j + l * ldb];
                s += (double)x * (double)y;
            }
            double v = (double)alpha * s;
            if (beta != 0.0f) v += (double)beta * (double)C[i + j * ldc];
            C[i + j * ldc] = (float)v;
        }
}

/* ----------------------------------------------------- double-double GEMM */
/* Error-free transformations: TwoSum (Knuth) and TwoProd via FMA.  The
 * accumulator (hi, lo) carries ~106 bits, so for the sizes used here the
 * result is the exactly rounded dot product to well below 1e-25 relative. */
static inline void two_sum(double a, double b, double* s, double* e) {
    double x = a + b;
    double bb = x - a;
    *e = (a - (x - bb)) + (b - bb);
    *s = x;
}
static inline void dd_add_prod(double* hi, double* lo, double a, double b) {
    double p = a * b;
    double pe = fma(a, b, -p);
    double s, e;
    two_sum(*hi, p, &s, &e);
    e += *lo + pe;
    double t = s + e;
    *lo = e - (t - s);
    *hi = t;
}

static void dd_dot(int oa, int ob, int64_t k, const double* A, int64_t lda, const double* B, int64_t ldb, int64_t i,
                   int64_t j, double* hi, double* lo, double* absum) {
    double h = 0.0, l = 0.0, ab = 0.0;
    for (int64_t q = 0; q < k; ++q) {
        double x = getd(A, oa, lda, i, q), y = getd(B, ob, ldb, q, j);
        dd_add_prod(&h, &l, x, y);
        ab += fabs(x) * fabs(y);
    }
    *hi = h;
    *lo = l;
    if (absum) *absum = ab;
}

/* Full double-double product op(A)*op(B) (alpha = 1, beta = 0): C_hi + C_lo,
 * and |op(A)||op(B)| in abs_ab (may be NULL). */
void oracle_gemm_dd(char ta, char tb, int64_t m, int64_t n, int64_t k, const double* A, int64_t lda, const double* B,
                    int64_t ldb, double* C_hi, double* C_lo, double* abs_ab, int64_t ldc) {
    int oa = op_code(ta), ob = op_code(tb);
    for (int64_t j = 0; j < n; ++j)
        for (int64_t i = 0; i < m; ++i)
            dd_dot(oa, ob, k, A, lda, B, ldb, i, j, &C_hi[i + j * ldc], &C_lo[i + j * ldc],
                   abs_ab ? &abs_ab[i + j * ldc] : NULL);
}

/* Double-double entries (rows[s], cols[s]) of op(A)*op(B) for s < nsamples. */
void oracle_gemm_dd_sampled(char ta, char tb, int64_t k, const double* A, int64_t lda, const double* B, int64_t ldb,
                            int64_t nsamples, const int64_t* rows, const int64_t* cols, double* hi, double* lo,
                            double* abs_ab) {
    int oa = op_code(ta), ob = op_code(tb);
    for (int64_t s = 0; s < nsamples; ++s)
        dd_dot(oa, ob, k, A, lda, B, ldb, rows[s], cols[s], &hi[s], &lo[s], abs_ab ? &abs_ab[s] : NULL);
}

/* -------------------------------------------- block-cyclic layout (COSTA) */

/* Restates scalapack::numroc (src/cosma/scalapack.cpp:49-88). */
int oracle_numroc(int n, int nb, int proc_coord, int proc_src, int n_procs) {
    int n_blocks = n / nb;
    int proc_offset = (n_procs + proc_coord - proc_src) % n_procs;
    int per = (n_blocks / n_procs) * nb;
    int rem = n_blocks % n_procs;
    int total = per;
    total += proc_offset < rem ? nb : 0;
    total += proc_offset == rem ? n % nb : 0;
    return total;
}

/* Owner process and local index of global index g (0-based) along one
 * dimension of a block-cyclic distribution with block nb over nprocs
 * processes starting at src: owner = (g/nb + src) % nprocs,
 * local = (g / (nb*nprocs))*nb + g % nb (utils/pxgemm_utils.hpp:71-87). */
void oracle_bc_coords(int64_t g, int nb, int nprocs, int src, int* owner, int64_t* local) {
    *owner = (int)((g / nb + src) % nprocs);
    *local = (g / ((int64_t)nb * nprocs)) * nb + g % nb;
}

/* Scatters a global column-major M x N matrix into the local buffer of
 * process (myrow, mycol) of a prow x pcol block-cyclic grid (lld = local
 * leading dimension).  Elements are copied bit-for-bit. */
void oracle_scatter_block_cyclic(int elem_bytes, const void* global, int64_t M, int64_t N, int64_t ldg, int mb, int nb,
                                 int prow, int pcol, int rsrc, int csrc, int myrow, int mycol, void* local,
                                 int64_t lld) {
    const char* G = (const char*)global;
    char* L = (char*)local;
    for (int64_t j = 0; j < N; ++j) {
        int oc;
        int64_t lc;
        oracle_bc_coords(j, nb, pcol, csrc, &oc, &lc);
        if (oc != mycol) continue;
        for (int64_t i = 0; i < M; ++i) {
            int orow;
            int64_t lr;
            oracle_bc_coords(i, mb, prow, rsrc, &orow, &lr);
            if (orow != myrow) continue;
            memcpy(L + (lr + lc * lld) * elem_bytes, G + (i + j * ldg) * elem_bytes, (size_t)elem_bytes);
        }
    }
}

/* The COSTA pack on one rank: dst(rows x cols, ldd) = op(src), bit-exact;
 * conjugation negates the imaginary part (sign-bit flip). */
void oracle_pack(char op, int is_complex, int elem_bytes, int64_t rows, int64_t cols, const void* src, int64_t lds,
                 void* dst, int64_t ldd) {
    int o = op_code(op);
    const unsigned char* S = (const unsigned char*)src;
    unsigned char* D = (unsigned char*)dst;
    for (int64_t j = 0; j < cols; ++j)
        for (int64_t i = 0; i < rows; ++i) {
            int64_t si = o == 0 ? i + j * lds : j + i * lds;
            unsigned char* d = D + (i + j * ldd) * elem_bytes;
            memcpy(d, S + si * elem_bytes, (size_t)elem_bytes);
            if (o == 2 && is_complex) d[elem_bytes - 1] ^= 0x80; /* sign of the imaginary part (little endian) */
        }
}

/* The COSTA back-transform of C on one rank: dst = alpha*src + beta*dst with
 * each product and the sum rounded separately; dst is not read when
 * beta == 0. */
void oracle_unpack_d(int64_t rows, int64_t cols, double alpha, const double* src, int64_t lds, double beta,
                     double* dst, int64_t ldd) {
    for (int64_t j = 0; j < cols; ++j)
        for (int64_t i = 0; i < rows; ++i) {
            double v = alpha * src[i + j * lds];
            if (beta != 0.0) {
                double w = beta * dst[i + j * ldd];
                v = v + w;
            }
            dst[i + j * ldd] = v;
        }
}

void oracle_unpack_z(int64_t rows, int64_t cols, const double* alpha, const zdouble* src, int64_t lds,
                     const double* beta, zdouble* dst, int64_t ldd) {
    int beta_zero = beta[0] == 0.0 && beta[1] == 0.0;
    for (int64_t j = 0; j < cols; ++j)
        for (int64_t i = 0; i < rows; ++i) {
            zdouble s = src[i + j * lds];
            double p1 = alpha[0] * s.re, p2 = alpha[1] * s.im, p3 = alpha[0] * s.im, p4 = alpha[1] * s.re;
            double vr = p1 - p2, vi = p3 + p4;
            if (!beta_zero) {
                zdouble d = dst[i + j * ldd];
                double q1 = beta[0] * d.re, q2 = beta[1] * d.im, q3 = beta[0] * d.im, q4 = beta[1] * d.re;
                double wr = q1 - q2, wi = q3 + q4;
                vr = vr + wr;
                vi = vi + wi;
            }
            dst[i + j * ldd].re = vr;
            dst[i + j * ldd].im = vi;
        }
}

/* C <- beta*C (scale_matrix, src/cosma/cosma_pxgemm.cpp:393-460); beta == 0
 * writes zeros. */
void oracle_scale_d(int64_t rows, int64_t cols, double beta, double* C, int64_t ldc) {
    if (beta == 1.0) return;
    for (int64_t j = 0; j < cols; ++j)
        for (int64_t i = 0; i < rows; ++i) C[i + j * ldc] = beta == 0.0 ? 0.0 : beta * C[i + j * ldc];
}
