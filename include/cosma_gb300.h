/*
 * cosma_gb300.h - C ABI of the GB300 (sm_103a) single-process GEMM path.
 *
 * This is the drop-in boundary for COSMA's one-rank GEMM path.  Every entry
 * point takes plain pointers and sizes; matrices are column-major.  Pointers
 * passed to the Tiled-MM / local_multiply / p?gemm entry points may be host
 * or device pointers (detected with cudaPointerGetAttributes); the *_device
 * entry points take device pointers and a cudaStream_t passed as void*.
 *
 * Complex scalars are passed as pointers to two consecutive reals (re, im),
 * exactly as the reference's ScaLAPACK ABI does (src/cosma/pxgemm.h:16-26).
 *
 * Errors: entry points that return int return COSMA_GPU_SUCCESS (0) or one
 * of the codes below and record a message for cosma_gpu_last_error_string().
 * The reference throws std::runtime_error on GPU errors
 * (src/cosma/gpu/utils.hpp:7-13); the ScaLAPACK entry points here are void
 * like the reference's, so their status is read via cosma_gpu_last_error().
 */
#ifndef COSMA_GB300_H
#define COSMA_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
#define COSMA_GPU_SUCCESS 0
#define COSMA_GPU_ERROR_INVALID_ARGUMENT 1
#define COSMA_GPU_ERROR_CUDA 2
#define COSMA_GPU_ERROR_OUT_OF_MEMORY 3
#define COSMA_GPU_ERROR_NOT_SUPPORTED 4
#define COSMA_GPU_ERROR_DEVICE_TIMEOUT 5
#define COSMA_GPU_ERROR_INTERNAL 6

/* Status of the last failing call on this thread (0 if none since the last
 * successful call). */
int cosma_gpu_last_error(void);
const char* cosma_gpu_last_error_string(void);
/* Library version string. */
const char* cosma_gpu_version(void);
/* Exercises the failure path of the tensor-core pipelines: a kernel waits on
 * a barrier nothing arrives on, through the bounded wait those pipelines use,
 * for limit_ns (1 ms .. 2 s).  Returns COSMA_GPU_ERROR_DEVICE_TIMEOUT when the
 * timeout was detected and reported (the expected outcome); the context stays
 * usable.  No reference counterpart. */
int cosma_gpu_selftest_wait_timeout(unsigned long long limit_ns, void* stream);

/* ------------------------------------------------------ arithmetic methods */
/* NATIVE: the operand type's own arithmetic on the FP64 pipe (the
 *         reference's semantics).
 * OZAKI : FP64-accurate GEMM from integer slices (|digit| <= 16) multiplied
 *         exactly on the FP8 tensor cores, summed exactly in 128-bit integers
 *         and rounded once (double and complex double).  On single-precision
 *         data it selects BF16X3 (float) or NATIVE (complex float).
 * BF16X3: single precision from three BF16 slices per operand, six slice
 *         products accumulated in FP32 on the BF16 tensor cores (float only).
 * AUTO  : BF16X3 for float, NATIVE for the other types. */
#define COSMA_GPU_METHOD_AUTO 0
#define COSMA_GPU_METHOD_NATIVE 1
#define COSMA_GPU_METHOD_OZAKI 2
#define COSMA_GPU_METHOD_BF16X3 3
/* FP64-accurate GEMM by the Chinese-remainder form of the Ozaki scheme
 * (Ozaki scheme II): one BF16 tensor-core GEMM per modulus.  Double and
 * complex double; float runs BF16x3 and complex float the native kernel, as
 * under COSMA_GPU_METHOD_OZAKI. */
#define COSMA_GPU_METHOD_OZAKI2 4

/* Statistics of one Ozaki-split GEMM (filled when a non-null pointer is
 * given). */
typedef struct cosma_gpu_ozaki_info {
    int slices;          /* digits per operand element                      */
    int products;        /* slice-pair GEMMs executed                       */
    int groups;          /* FP32 accumulator drains per output tile         */
    int fallback_native; /* 1 if non-finite input forced the native path    */
    double spread_bits;  /* exponent-spread estimate used to size slices    */
    double prep_ms;      /* scaling + slicing kernels (CUDA events)         */
    double gemm_ms;      /* slice-product GEMM kernel (CUDA events)         */
    int fraction_bits;   /* fixed-point fraction bits of the operands       */
    int exact_product;   /* 1: every input bit kept, the product is exact   */
} cosma_gpu_ozaki_info;

/* ----------------------------------------------------- Tiled-MM interface */
/* Replaces gpu::make_context<T>(streams, tile_m, tile_n, tile_k)
 * (called at src/cosma/context.cpp:24-25,45; Tiled-MM v2.3.2).
 * scalar: 's', 'd', 'c' or 'z'.  Non-positive sizes select the defaults
 * (COSMA_GPU_STREAMS / COSMA_GPU_MAX_TILE_{M,N,K} or the built-in values). */
typedef struct cosma_gpu_mm_handle cosma_gpu_mm_handle;
cosma_gpu_mm_handle* cosma_gpu_tmm_make_context(char scalar, int streams, int tile_m,
                                                int tile_n, int tile_k);
void cosma_gpu_tmm_destroy_context(cosma_gpu_mm_handle* handle);
/* Selects the arithmetic used by the handle's gemm calls.  ozaki_slices <= 0
 * lets the library size the slices from the inputs. */
int cosma_gpu_tmm_set_method(cosma_gpu_mm_handle* handle, int method, int ozaki_slices);
/* Device buffer holding the C of the last call made with copy_c_back == 0
 * (replaces mm_handle::get_full_device_buffer_c(), src/cosma/gpu/nccl_utils.cpp:200). */
void* cosma_gpu_tmm_device_buffer_c(cosma_gpu_mm_handle* handle);

/* 1 when the handle's last gemm call ran in an overlapped one-step form
 * (host A, B and C in one step: the Chinese-remainder method for double and
 * real-scaled complex, 3xBF16 for float), else 0.
 * New: a diagnostic of this library; the reference has no counterpart. */
int cosma_gpu_tmm_last_overlapped(cosma_gpu_mm_handle* h);
/* Bytes the handle's last gemm call moved host->device and device->host
 * (zero for operands that were already in device memory). */
int cosma_gpu_tmm_last_transfer_bytes(cosma_gpu_mm_handle* handle, int64_t* h2d_bytes,
                                      int64_t* d2h_bytes);
/* Ozaki statistics of the handle's last call. */
int cosma_gpu_tmm_last_ozaki_info(cosma_gpu_mm_handle* handle, cosma_gpu_ozaki_info* info);
/* Memory limit: the largest square tiles (multiple of 256) whose device
 * footprint (double-buffered A, B, C tile slots plus the method's worst-case
 * scratch) fits in `bytes`; the one-GPU counterpart of COSMA's sequential
 * splits under a memory limit (src/cosma/strategy.cpp:404-440).  The streamer
 * then runs problems of any size in steps of these tiles.
 * tiles_for_memory computes the tiles only; set_memory_limit applies them to
 * a handle (for its current method); tiles reads them back. */
int cosma_gpu_tmm_tiles_for_memory(char scalar, int method, int64_t bytes, int* tile_m, int* tile_n,
                                   int* tile_k);
int cosma_gpu_tmm_set_memory_limit(cosma_gpu_mm_handle* handle, int64_t bytes);
int cosma_gpu_tmm_tiles(cosma_gpu_mm_handle* handle, int* tile_m, int* tile_n, int* tile_k);

/* Replaces gpu::gemm(mm_handle<T>&, transa, transb, m, n, k, alpha, A, lda,
 * B, ldb, beta, C, ldc, pin_host_buffers, copy_c_back)
 * (call site src/cosma/local_multiply.cpp:245-260; Tiled-MM v2.3.2).
 * C = alpha * op(A) * op(B) + beta * C, op in {'N','T','C'} (case-insensitive).
 * With beta == 0, C is never read (it may hold NaN). */
int cosma_gpu_tmm_gemm_s(cosma_gpu_mm_handle* h, char transa, char transb, int m, int n, int k,
                         float alpha, const float* A, int lda, const float* B, int ldb,
                         float beta, float* C, int ldc, int pin_host_buffers, int copy_c_back);
int cosma_gpu_tmm_gemm_d(cosma_gpu_mm_handle* h, char transa, char transb, int m, int n, int k,
                         double alpha, const double* A, int lda, const double* B, int ldb,
                         double beta, double* C, int ldc, int pin_host_buffers, int copy_c_back);
int cosma_gpu_tmm_gemm_c(cosma_gpu_mm_handle* h, char transa, char transb, int m, int n, int k,
                         const float* alpha, const float* A, int lda, const float* B, int ldb,
                         const float* beta, float* C, int ldc, int pin_host_buffers,
                         int copy_c_back);
int cosma_gpu_tmm_gemm_z(cosma_gpu_mm_handle* h, char transa, char transb, int m, int n, int k,
                         const double* alpha, const double* A, int lda, const double* B,
                         int ldb, const double* beta, double* C, int ldc,
                         int pin_host_buffers, int copy_c_back);

/* --------------------------------------------------- COSMA local_multiply */
/* Replaces cosma::local_multiply(cosma_context<T>*, a, b, c, m, n, k, alpha,
 * beta, copy_c_back) (src/cosma/local_multiply.hpp:6-16,
 * src/cosma/local_multiply.cpp:300-381) and, with handle == NULL, the
 * context-less overload (src/cosma/local_multiply.hpp:40-49) that uses the
 * per-type singleton (src/cosma/context.cpp:155-158).  A is m x k (ld m),
 * B is k x n (ld k), C is m x n (ld m), no transposes: at P = 1
 * cosma::multiply reduces to exactly this call (src/cosma/multiply.cpp:369-394). */
int cosma_gpu_local_multiply_s(cosma_gpu_mm_handle* h, float* a, float* b, float* c, int m,
                               int n, int k, float alpha, float beta, int copy_c_back);
int cosma_gpu_local_multiply_d(cosma_gpu_mm_handle* h, double* a, double* b, double* c, int m,
                               int n, int k, double alpha, double beta, int copy_c_back);
int cosma_gpu_local_multiply_c(cosma_gpu_mm_handle* h, float* a, float* b, float* c, int m,
                               int n, int k, const float* alpha, const float* beta,
                               int copy_c_back);
int cosma_gpu_local_multiply_z(cosma_gpu_mm_handle* h, double* a, double* b, double* c, int m,
                               int n, int k, const double* alpha, const double* beta,
                               int copy_c_back);
/* The per-type singleton context (replaces get_context_instance<T>(),
 * src/cosma/context.cpp:155-158).  Owned by the library. */
cosma_gpu_mm_handle* cosma_gpu_context_instance(char scalar);

/* -------------------------------------------------- device-pointer GEMMs */
/* Stream-ordered GEMM on device pointers: no host synchronisation, no copies.
 * 64-bit sizes (the reference's int products m*k overflow at 65536^2,
 * src/cosma/local_multiply.cpp:343-346). */
int cosma_gpu_dgemm_device(int method, char transa, char transb, int64_t m, int64_t n,
                           int64_t k, double alpha, const double* A, int64_t lda,
                           const double* B, int64_t ldb, double beta, double* C, int64_t ldc,
                           void* stream);
int cosma_gpu_zgemm_device(int method, char transa, char transb, int64_t m, int64_t n,
                           int64_t k, const double* alpha, const double* A, int64_t lda,
                           const double* B, int64_t ldb, const double* beta, double* C,
                           int64_t ldc, void* stream);
int cosma_gpu_sgemm_device(int method, char transa, char transb, int64_t m, int64_t n,
                           int64_t k, float alpha, const float* A, int64_t lda,
                           const float* B, int64_t ldb, float beta, float* C, int64_t ldc,
                           void* stream);
int cosma_gpu_cgemm_device(int method, char transa, char transb, int64_t m, int64_t n,
                           int64_t k, const float* alpha, const float* A, int64_t lda,
                           const float* B, int64_t ldb, const float* beta, float* C,
                           int64_t ldc, void* stream);
/* FP64-accurate Ozaki-split DGEMM (no counterpart in the reference, which
 * runs native DGEMM).  slices <= 0 sizes the slice count from the inputs'
 * exponent spread; `info` may be NULL. */
int cosma_gpu_dgemm_ozaki_device(char transa, char transb, int64_t m, int64_t n, int64_t k,
                                 double alpha, const double* A, int64_t lda, const double* B,
                                 int64_t ldb, double beta, double* C, int64_t ldc, int slices,
                                 void* stream, cosma_gpu_ozaki_info* info);
/* The same for complex double (interleaved re/im, op N, T or C): the real
 * and imaginary parts come out of one slice-product GEMM over [Re | Im]
 * digit rows (four real products per complex one), each part summed exactly
 * and rounded once.  alpha/beta point to {re, im}. */
int cosma_gpu_zgemm_ozaki_device(char transa, char transb, int64_t m, int64_t n, int64_t k,
                                 const double* alpha, const double* A, int64_t lda,
                                 const double* B, int64_t ldb, const double* beta, double* C,
                                 int64_t ldc, int slices, void* stream, cosma_gpu_ozaki_info* info);

/* FP64-accurate DGEMM by the Chinese-remainder form of the Ozaki scheme
 * (Ozaki scheme II; new, no reference counterpart).  op(A) and op(B) are
 * scaled per row / column by powers of two and rounded to integers of P
 * fraction bits; their residues modulo `moduli` pairwise coprime moduli
 * <= 255 are multiplied exactly on the BF16 tensor cores (one GEMM per
 * modulus), and the exact integer product is rebuilt by the Chinese
 * remainder theorem and rounded once to FP64.  moduli <= 0 sizes the count
 * (and P) from the inputs' exponent spread; explicit counts run from 2 to
 * 28, and P is the largest the count allows for this k.  The automatic
 * count is the fewest moduli that either keep every bit of the inputs (the
 * product is then exact and C correctly rounded) or meet the accuracy rule
 * for the inputs' exponent spread.  In *info, `slices` and `products` report
 * the modulus count, `groups` the FP32 accumulator drains per output tile,
 * `fraction_bits` P and `exact_product` whether every input bit was kept.  Inf/NaN inputs
 * run the native kernel (fallback_native = 1).  k beyond 4,194,240 runs in
 * passes accumulated through C. */
int cosma_gpu_dgemm_ozaki2_device(char transa, char transb, int64_t m, int64_t n, int64_t k,
                                  double alpha, const double* A, int64_t lda, const double* B,
                                  int64_t ldb, double beta, double* C, int64_t ldc, int moduli,
                                  void* stream, cosma_gpu_ozaki_info* info);
/* Exact residual of a computed product (new; no reference counterpart): for
 * a candidate Ct (m x n, ld ldt) of op(A) * op(B) (op N or T), writes
 * E = op(A) op(B) - Ct, exact before its one rounding to FP64, and
 * Rx = op(A) op(B) rounded once, both m x n with leading dimension ldo.  The
 * product is the Chinese-remainder form's: exact for operands whose bits all
 * lie within P fraction bits of their row's / column's leading bit (moduli
 * = 28 gives P = 98 at k = 16384).  Used to state the error of a result over
 * every entry; an entry of Ct below ~2^-144 of its row and column scales
 * gives E = NaN.  k <= 4,194,240, one pass. */
int cosma_gpu_dgemm_ozaki2_residual(char transa, char transb, int64_t m, int64_t n, int64_t k,
                                    const double* A, int64_t lda, const double* B, int64_t ldb,
                                    const double* Ct, int64_t ldt, int moduli, double* E, double* Rx,
                                    int64_t ldo, void* stream, cosma_gpu_ozaki_info* info);
/* The modulus count and fraction bits P that cosma_gpu_dgemm_ozaki2_device
 * uses for depth k (2k for the complex form), the measured exponent spread
 * of the operands (the info record's spread_bits) and exact_bits, the
 * fraction bits that keep every input bit (max over rows and columns of the
 * scale exponent minus the weight of the lowest set bit; <= 0: unknown):
 * the fewer moduli of the two that meet the accuracy rule or keep every bit.
 * moduli > 0 fixes the count as in the GEMM call.  Host-only: touches no
 * device. */
int cosma_gpu_ozaki2_choose(int64_t k, double spread_bits, int exact_bits, int moduli, int* nmod,
                            int* fraction_bits);
/* The precision forms keep a workspace per (device, stream) that grows to
 * the largest problem run on that stream.  This frees the workspaces kept
 * for `stream` on the current device; call it before destroying a stream
 * that was passed to them (Tiled-MM handles do so for their own streams).
 * Work on the stream must be complete.  Always succeeds. */
int cosma_gpu_release_workspaces(void* stream);
/* The same for complex double (interleaved re/im, op N, T or C): both parts
 * of C come out of one modular GEMM of depth 2k per modulus (four real
 * products per complex one), each part exact before its one rounding.
 * alpha/beta point to {re, im}. */
int cosma_gpu_zgemm_ozaki2_device(char transa, char transb, int64_t m, int64_t n, int64_t k,
                                  const double* alpha, const double* A, int64_t lda,
                                  const double* B, int64_t ldb, const double* beta, double* C,
                                  int64_t ldc, int moduli, void* stream, cosma_gpu_ozaki_info* info);

/* Size of the static device array that cosma_gpu_dgemm_ozaki_noalloc draws
 * all of its scratch from (64 MiB, held on every GPU that loads the library). */
#define COSMA_GPU_OZAKI_NOALLOC_SCRATCH_BYTES (64ull << 20)

/* FP64-accurate Ozaki-split DGEMM that allocates nothing; it has no
 * counterpart in the reference.  It is meant for callers that cannot let a
 * library allocate device memory: applications whose device memory is all
 * owned by their own pool allocator, and code that must not trigger the
 * device-wide synchronisation cudaMalloc / cudaFree imply.  Arguments and
 * C are those of cosma_gpu_dgemm_ozaki_device (same kernels, same output
 * bits); the caller still provides A, B and C in device memory.  In *info
 * the slice fields and fallback_native are filled, prep_ms and gemm_ms stay
 * 0 (this entry point creates no timing events).
 * Scratch comes from one static device array of
 * COSMA_GPU_OZAKI_NOALLOC_SCRATCH_BYTES; problems needing more are rejected
 * with COSMA_GPU_ERROR_INVALID_ARGUMENT and a message giving the size (about
 * m = n = k = 1024 with 13 slices fits).  The first call on each device looks
 * up the array's device address (cudaGetSymbolAddress).  Each call waits for its stream twice per pass over K (k beyond 65536 takes
 * several passes): once to read the exponent statistics that fix the slice
 * count, once to read the kernels' error word.  All calls share the one
 * array: calls that overlap on the GPU (other streams, other threads) race
 * and must be serialised by the caller. */
int cosma_gpu_dgemm_ozaki_noalloc(char transa, char transb, int64_t m, int64_t n, int64_t k,
                                  double alpha, const double* A, int64_t lda, const double* B,
                                  int64_t ldb, double beta, double* C, int64_t ldc, int slices,
                                  void* stream, cosma_gpu_ozaki_info* info);

/* ----------------------------------------------------- fault injection */
/* Test hook (new; the reference has none): the next `count` calls at `site`
 * fail on the host as if CUDA had refused them, so that callers can check the
 * error paths without faulting a GPU.  Sites: 1 device workspace allocation
 * (cudaMalloc: the call returns COSMA_GPU_ERROR_OUT_OF_MEMORY with a message),
 * 2 page-locking of caller memory (cudaHostRegister: the streamer falls back
 * to its unregistered copy route, same result), 3 pinned staging allocations
 * (cudaMallocHost: an Ozaki / 3xBF16 call returns OUT_OF_MEMORY, the host
 * copies fall back to the driver's pageable copies), 4 a host copy issued by
 * the overlapped one-step form's copy thread (the call returns
 * COSMA_GPU_ERROR_CUDA with the copy's message; a refused operand-panel copy
 * comes before any write to C).  count 0 disarms the site.  Handles and
 * contexts stay usable after an injected failure. */
#define COSMA_GPU_FAULT_DEVICE_ALLOC 1
#define COSMA_GPU_FAULT_HOST_REGISTER 2
#define COSMA_GPU_FAULT_PINNED_ALLOC 3
#define COSMA_GPU_FAULT_HOST_COPY 4
int cosma_gpu_test_fail_next(int site, int count);
/* Faults still armed at `site` (-1 for an unknown site). */
int cosma_gpu_test_faults_pending(int site);

/* ------------------------------------------------- grouped (batched) GEMM */
/* One problem of a batch: C = alpha * op(A) * op(B) + beta * C on device
 * pointers (column-major).  Layout is part of the ABI (80 bytes). */
typedef struct cosma_gpu_gemm_problem {
    char transa, transb; /* 'N', 'T' or 'C' */
    int32_t m, n, k;
    double alpha, beta;
    const double* A;
    int64_t lda;
    const double* B;
    int64_t ldb;
    double* C;
    int64_t ldc;
} cosma_gpu_gemm_problem;

typedef struct cosma_gpu_grouped_info {
    int tiles;            /* tiles in the persistent launch                  */
    int tile_policy;      /* 0 all 32x32, 1 per-problem shapes, 2 16-row tiles for small m/n */
    int dynamic_schedule; /* 1: warps fetch tiles through an atomic counter  */
    int warps_per_cta;
    double useful_flops;  /* sum of 2 m n k                                  */
    double padded_flops;  /* work the tiles actually issue                   */
    double tuned_ms;      /* time of the chosen configuration while tuning   */
} cosma_gpu_grouped_info;

/* A grouped GEMM of `count` independent FP64 problems in one persistent
 * launch, captured in a CUDA graph.  The reference runs such batches as a loop
 * of local_multiply calls (src/cosma/multiply.cpp:476-587); there is no
 * grouped entry point in the reference.  With autotune != 0 the tile policy,
 * schedule and CTA size are chosen by timing candidates on the batch (the
 * choice is cached per batch signature); tuning runs the batch several times
 * and restores the C of problems with beta != 0.  The problem array is copied;
 * the device buffers must stay valid while the plan is used.
 *
 * method COSMA_GPU_METHOD_OZAKI gives the FP64-accurate form: the graph
 * scales, slices and multiplies every problem on the FP8 tensor cores (one
 * launch per step over the whole batch).  Slice counts are planned from the
 * data present at creation and re-checked on the device at every run; a
 * problem whose data then needs more slices, or holds Inf/NaN, is left to the
 * single-problem path.  Runs of an Ozaki plan synchronise `stream` (the host
 * reads the check), and tuning (tile order) runs only for beta == 0 batches.
 *
 * method COSMA_GPU_METHOD_OZAKI2 gives the Chinese-remainder form: one
 * modulus count N for the batch (the most any problem's data needs, from the
 * same rule as cosma_gpu_dgemm_ozaki2_device), each problem's fraction bits
 * the most N admits at its k; the graph scales, splits into residues,
 * multiplies every 128 x 128 tile's N modular products on the BF16 tensor
 * cores and reconstructs each entry with one rounding.  The same re-check
 * and single-problem fall-back apply; problems with k > 65536 always take
 * the single-problem path. */
typedef struct cosma_gpu_grouped_plan cosma_gpu_grouped_plan;
cosma_gpu_grouped_plan* cosma_gpu_grouped_plan_create(int method, int count,
                                                      const cosma_gpu_gemm_problem* problems,
                                                      int autotune, void* stream);
/* Replays the plan's CUDA graph on `stream` (asynchronous for native plans). */
int cosma_gpu_grouped_plan_run(cosma_gpu_grouped_plan* plan, void* stream);
int cosma_gpu_grouped_plan_info(cosma_gpu_grouped_plan* plan, cosma_gpu_grouped_info* info);
/* Slice count planned for each problem of an Ozaki plan, or the modulus count
 * of the batch for each problem of a Chinese-remainder plan (`count` ints; 0
 * for problems the plan does not take, and for every problem of a native plan). */
int cosma_gpu_grouped_plan_slices(cosma_gpu_grouped_plan* plan, int* slices);
void cosma_gpu_grouped_plan_destroy(cosma_gpu_grouped_plan* plan);
/* One-shot grouped GEMM (plan without tuning, run, synchronise, destroy). */
int cosma_gpu_dgemm_grouped_device(int method, int count, const cosma_gpu_gemm_problem* problems,
                                   void* stream);

/* ------------------------------------------- multiply_using_layout (C API) */
/* Replaces the reference's C interface for arbitrary block layouts
 * (src/cosma/cinterface.hpp:9-40, cinterface.cpp:55-147; multiply.cpp:78-213)
 * on one rank.  The two structs have the reference's `block` / `layout`
 * memory layout, so existing descriptions can be passed by pointer.
 *   rowsplit[rowblocks + 1], colsplit[colblocks + 1]: block boundaries;
 *   owners[rowblocks * colblocks]: must all be 0 (one rank);
 *   localblocks[nlocalblocks]: every block (row, col) exactly once, column-major
 *   with leading dimension ld, in host or device memory.
 * The layouts describe the matrices as stored: op(A) is m x k, so A is m x k
 * for 'N' and k x m for 'T' / 'C' (the reference derives m and k from the
 * stored shape, which coincide for 'N').  Computes
 * C = alpha * op(A) * op(B) + beta * C with the process-wide method
 * (cosma_gpu_pxgemm_set_method / COSMA_GPU_GEMM_METHOD). */
typedef struct cosma_gpu_block {
    void* data;
    const int ld;
    const int row;
    const int col;
} cosma_gpu_block;
typedef struct cosma_gpu_layout {
    int rowblocks;
    int colblocks;
    const int* rowsplit;
    const int* colsplit;
    const int* owners;
    int nlocalblocks;
    cosma_gpu_block* localblocks;
} cosma_gpu_layout;
int cosma_gpu_smultiply_using_layout(const char* transa, const char* transb, const float* alpha,
                                     const cosma_gpu_layout* a, const cosma_gpu_layout* b,
                                     const float* beta, const cosma_gpu_layout* c);
int cosma_gpu_dmultiply_using_layout(const char* transa, const char* transb, const double* alpha,
                                     const cosma_gpu_layout* a, const cosma_gpu_layout* b,
                                     const double* beta, const cosma_gpu_layout* c);
int cosma_gpu_cmultiply_using_layout(const char* transa, const char* transb, const float* alpha,
                                     const cosma_gpu_layout* a, const cosma_gpu_layout* b,
                                     const float* beta, const cosma_gpu_layout* c);
int cosma_gpu_zmultiply_using_layout(const char* transa, const char* transb, const double* alpha,
                                     const cosma_gpu_layout* a, const cosma_gpu_layout* b,
                                     const double* beta, const cosma_gpu_layout* c);

/* ------------------------------------- COSTA 1x1-grid layout transforms */
/* dst(rows x cols) = op(src) where op in {'N','T','C'}: the block-cyclic ->
 * COSMA-blocked pack that costa::transformer::schedule(scalapack -> cosma,
 * trans, 1, 0) + transform() performs on one rank
 * (src/cosma/cosma_pxgemm.cpp:338-343).  Bit-exact copy.  elem_bytes is 4
 * (s), 8 (d or c) or 16 (z); conjugation flips the sign bit of imaginary
 * parts (elem_bytes 8 with is_complex=1 means complex float). */
int costa_gpu_pack(char op, int is_complex, int elem_bytes, int64_t rows, int64_t cols,
                   const void* src, int64_t ld_src, void* dst, int64_t ld_dst, void* stream);
/* dst = alpha * src + beta * dst (dst is not read when beta == 0): the
 * COSMA -> ScaLAPACK back-transform of C with alpha/beta
 * (src/cosma/cosma_pxgemm.cpp:362-364).  Real: products rounded as
 * fl(fl(alpha*s) + fl(beta*d)) without contraction. */
int costa_gpu_unpack_d(int64_t rows, int64_t cols, double alpha, const double* src,
                       int64_t ld_src, double beta, double* dst, int64_t ld_dst, void* stream);
int costa_gpu_unpack_z(int64_t rows, int64_t cols, const double* alpha, const double* src,
                       int64_t ld_src, const double* beta, double* dst, int64_t ld_dst,
                       void* stream);
int costa_gpu_unpack_s(int64_t rows, int64_t cols, float alpha, const float* src,
                       int64_t ld_src, float beta, float* dst, int64_t ld_dst, void* stream);
int costa_gpu_unpack_c(int64_t rows, int64_t cols, const float* alpha, const float* src,
                       int64_t ld_src, const float* beta, float* dst, int64_t ld_dst,
                       void* stream);

/* ------------------------------------------- ScaLAPACK p?gemm (1x1 grid) */
/* Replace the reference's interposed ScaLAPACK symbols (src/cosma/pxgemm.h:6-107,
 * src/cosma/pxgemm.cpp:8-...) and the prefixed cosma_p?gemm family
 * (src/cosma/prefixed_pxgemm.h:6-54).  Only a 1x1 process grid is accepted:
 * if BLACS' Cblacs_gridinfo is linked it is asked for the grid, otherwise the
 * grid is taken to be 1x1.  Descriptors: desc[1] ctxt, desc[2..3] M,N,
 * desc[4..5] MB,NB, desc[6..7] RSRC,CSRC, desc[8] LLD (src/cosma/scalapack.hpp:11-47). */
#define COSMA_GPU_PXGEMM_ARGS(T)                                                              \
    const char *transa, const char *transb, const int *m, const int *n, const int *k,        \
        const T *alpha, const T *a, const int *ia, const int *ja, const int *desca,          \
        const T *b, const int *ib, const int *jb, const int *descb, const T *beta, T *c,     \
        const int *ic, const int *jc, const int *descc

void psgemm(COSMA_GPU_PXGEMM_ARGS(float));
void pdgemm(COSMA_GPU_PXGEMM_ARGS(double));
void pcgemm(COSMA_GPU_PXGEMM_ARGS(float));
void pzgemm(COSMA_GPU_PXGEMM_ARGS(double));
void psgemm_(COSMA_GPU_PXGEMM_ARGS(float));
void pdgemm_(COSMA_GPU_PXGEMM_ARGS(double));
void pcgemm_(COSMA_GPU_PXGEMM_ARGS(float));
void pzgemm_(COSMA_GPU_PXGEMM_ARGS(double));
void PSGEMM(COSMA_GPU_PXGEMM_ARGS(float));
void PDGEMM(COSMA_GPU_PXGEMM_ARGS(double));
void PCGEMM(COSMA_GPU_PXGEMM_ARGS(float));
void PZGEMM(COSMA_GPU_PXGEMM_ARGS(double));
void PSGEMM_(COSMA_GPU_PXGEMM_ARGS(float));
void PDGEMM_(COSMA_GPU_PXGEMM_ARGS(double));
void PCGEMM_(COSMA_GPU_PXGEMM_ARGS(float));
void PZGEMM_(COSMA_GPU_PXGEMM_ARGS(double));
void cosma_psgemm(COSMA_GPU_PXGEMM_ARGS(float));
void cosma_pdgemm(COSMA_GPU_PXGEMM_ARGS(double));
void cosma_pcgemm(COSMA_GPU_PXGEMM_ARGS(float));
void cosma_pzgemm(COSMA_GPU_PXGEMM_ARGS(double));
void cosma_psgemm_(COSMA_GPU_PXGEMM_ARGS(float));
void cosma_pdgemm_(COSMA_GPU_PXGEMM_ARGS(double));
void cosma_pcgemm_(COSMA_GPU_PXGEMM_ARGS(float));
void cosma_pzgemm_(COSMA_GPU_PXGEMM_ARGS(double));
void COSMA_PSGEMM(COSMA_GPU_PXGEMM_ARGS(float));
void COSMA_PDGEMM(COSMA_GPU_PXGEMM_ARGS(double));
void COSMA_PCGEMM(COSMA_GPU_PXGEMM_ARGS(float));
void COSMA_PZGEMM(COSMA_GPU_PXGEMM_ARGS(double));
void COSMA_PSGEMM_(COSMA_GPU_PXGEMM_ARGS(float));
void COSMA_PDGEMM_(COSMA_GPU_PXGEMM_ARGS(double));
void COSMA_PCGEMM_(COSMA_GPU_PXGEMM_ARGS(float));
void COSMA_PZGEMM_(COSMA_GPU_PXGEMM_ARGS(double));

/* Method used by the p?gemm entry points (default NATIVE; the
 * COSMA_GPU_GEMM_METHOD environment variable "native"/"ozaki"/"bf16x3"/
 * "ozaki2" sets the initial value).  With OZAKI2, a real double call on host
 * A, B and C runs in the overlapped one-step form (panel copies, modular
 * GEMMs and C copies overlapped; the same bits as the staged form) unless
 * COSMA_GPU_OZAKI2_OVERLAP=OFF. */
int cosma_gpu_pxgemm_set_method(int method);

/* The last p?gemm call's host-to-device and device-to-host bytes (the
 * copies of host arrays; 0 for device arrays) and whether the overlapped
 * form ran it (1) or the staged one (0).
 * New: a diagnostic of this library; the reference has no counterpart. */
int cosma_gpu_pxgemm_last_transfers(int64_t* h2d_bytes, int64_t* d2h_bytes, int* overlapped);

/* Route a host <-> HBM copy of the array at `ptr` takes inside the
 * host-pointer entry points (p?gemm, multiply_using_layout):
 *   0  cudaMemcpy (device, pinned or registered memory);
 *   1  pageable memory through pinned staging buffers filled by host threads;
 *   2  a device copy kernel reading / writing the host array in place, for
 *      pageable and for mapped pinned memory, where the GPU reaches host
 *      memory through the host's page tables, as on a Grace host
 *      (COSMA_GPU_HOST_DIRECT=OFF selects routes 1 and 0 instead).
 * New: COSMA stages through its own pinned buffers (src/cosma/pinned_buffers.cpp). */
int cosma_gpu_host_copy_route(const void* ptr);

#ifdef __cplusplus
}
#endif

#endif /* COSMA_GB300_H */
