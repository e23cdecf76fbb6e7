// Native FP64 / complex-FP64 / FP32 GEMM on sm_103a: the plain drop-in form.
//
// C = alpha * op(A) * op(B) + beta * C, column-major, op in {N, T, C}.
// This replaces the cuBLAS ?gemm that Tiled-MM's gpu::gemm issues per tile
// (call site src/cosma/local_multiply.cpp:245-260).
//
// sm_103a has no tcgen05 FP64 kind, so the FP64 tensor path is the warp-level
// DMMA (mma.sync m16n8k4 .f64).  Measured on GB300 the FP64 pipe delivers
// ~1.05 TFLOP/s through DMMA and ~1.0 through DFMA, i.e. only a few flops per
// clock per SM, so this kernel is compute-bound at any reasonable tiling: a
// 64x64x16 block tile, 4 warps (2x2, 32x32 each), a 3-stage cp.async ring
// and bank-conflict-free fragment reads are enough to keep the pipe fed.
// The same kernel serves FP32 (converted to FP64 in shared memory reads,
// i.e. FP32 inputs multiplied exactly and accumulated in FP64) and complex
// data (four real DMMAs per complex fragment product).
#include "common.cuh"
#include "runtime.hpp"

#include <cuComplex.h>

namespace cgb {
namespace {

constexpr int BM = 64, BN = 64, BK = 16, STAGES = 3, THREADS = 128;
constexpr int PAD = 4;  // doubles of padding per smem row (see bank analysis below)

// Element traits: FP64 real, FP32 real (loaded as float, multiplied in FP64),
// complex double, complex float.
template <class E> struct Elem;
template <> struct Elem<double> { static constexpr bool cplx = false; static constexpr int bytes = 8; };
template <> struct Elem<float> { static constexpr bool cplx = false; static constexpr int bytes = 4; };
template <> struct Elem<double2> { static constexpr bool cplx = true; static constexpr int bytes = 16; };
template <> struct Elem<float2> { static constexpr bool cplx = true; static constexpr int bytes = 8; };

struct Args {
    int64_t m, n, k;
    const void* A; int64_t lda;
    const void* B; int64_t ldb;
    void* C; int64_t ldc;
    double alpha_re, alpha_im, beta_re, beta_im;
    int conj_a, conj_b;
};

__device__ __forceinline__ void cp_async(void* smem, const void* gmem, int bytes_valid, int size) {
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    if (size == 16)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(bytes_valid));
    else if (size == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gmem), "r"(bytes_valid));
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s), "l"(gmem), "r"(bytes_valid));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N> __device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

__device__ __forceinline__ void dmma(double (&c)[4], double a0, double a1, double b0) {
    asm volatile("mma.sync.aligned.m16n8k4.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5}, {%6}, {%0,%1,%2,%3};\n"
                 : "+d"(c[0]), "+d"(c[1]), "+d"(c[2]), "+d"(c[3])
                 : "d"(a0), "d"(a1), "d"(b0));
}

__device__ __forceinline__ double neg_bits(double x) {  // sign flip without an FP64 op
    return __longlong_as_double(__double_as_longlong(x) ^ (long long)0x8000000000000000ull);
}

// Shared-memory layout: each operand tile is stored with the global
// contiguous dimension contiguous in shared memory, so global reads coalesce:
//   A, op N : sA[l][i] (row stride BM+PAD)   A, op T/C : sA[i][l] (stride BK+PAD)
//   B, op N : sB[j][l] (stride BK+PAD)       B, op T/C : sB[l][j] (stride BN+PAD)
// Fragment reads touch 4 rows x 8 consecutive doubles (or 8 rows x 4); with
// the +4 padding every bank is hit exactly twice per 32 doubles = the minimum
// two wavefronts for 256 bytes.  Complex elements are stored interleaved.
template <class E, bool TA, bool TB>
struct Tile {
    static constexpr int SA = TA ? (BK + PAD) : (BM + PAD);
    static constexpr int SB = TB ? (BN + PAD) : (BK + PAD);
    static constexpr int A_ELEMS = TA ? BM * SA : BK * SA;
    static constexpr int B_ELEMS = TB ? BK * SB : BN * SB;
    static constexpr int STAGE_BYTES = (A_ELEMS + B_ELEMS) * Elem<E>::bytes;
    __device__ static int a_idx(int i, int l) { return TA ? i * SA + l : l * SA + i; }
    __device__ static int b_idx(int l, int j) { return TB ? l * SB + j : j * SB + l; }
};

template <class E, bool TA, bool TB>
__device__ __forceinline__ void load_stage(const Args& g, unsigned char* stage, int64_t m0, int64_t n0,
                                           int64_t k0) {
    using T = Tile<E, TA, TB>;
    constexpr int EB = Elem<E>::bytes;
    E* sA = reinterpret_cast<E*>(stage);
    E* sB = reinterpret_cast<E*>(stage + T::A_ELEMS * EB);
    const E* A = reinterpret_cast<const E*>(g.A);
    const E* B = reinterpret_cast<const E*>(g.B);
    const int tid = threadIdx.x;
    // A tile: BM x BK elements of op(A).
#pragma unroll
    for (int r = 0; r < (BM * BK) / THREADS; ++r) {
        int e = tid + r * THREADS;
        int i, l;
        if (!TA) { i = e % BM; l = e / BM; } else { l = e % BK; i = e / BK; }
        int64_t gi = m0 + i, gl = k0 + l;
        bool ok = gi < g.m && gl < g.k;
        const E* src = ok ? (TA ? A + gl + gi * g.lda : A + gi + gl * g.lda) : A;
        cp_async(sA + T::a_idx(i, l), src, ok ? EB : 0, EB);
    }
    // B tile: BK x BN elements of op(B).
#pragma unroll
    for (int r = 0; r < (BN * BK) / THREADS; ++r) {
        int e = tid + r * THREADS;
        int l, j;
        if (!TB) { l = e % BK; j = e / BK; } else { j = e % BN; l = e / BN; }
        int64_t gl = k0 + l, gj = n0 + j;
        bool ok = gl < g.k && gj < g.n;
        const E* src = ok ? (TB ? B + gj + gl * g.ldb : B + gl + gj * g.ldb) : B;
        cp_async(sB + T::b_idx(l, j), src, ok ? EB : 0, EB);
    }
}

template <class E> __device__ __forceinline__ void ld_elem(const E* p, double& re, double& im);
template <> __device__ __forceinline__ void ld_elem<double>(const double* p, double& re, double& im) { re = *p; im = 0; }
template <> __device__ __forceinline__ void ld_elem<float>(const float* p, double& re, double& im) { re = (double)*p; im = 0; }
template <> __device__ __forceinline__ void ld_elem<double2>(const double2* p, double& re, double& im) { double2 v = *p; re = v.x; im = v.y; }
template <> __device__ __forceinline__ void ld_elem<float2>(const float2* p, double& re, double& im) { float2 v = *p; re = v.x; im = v.y; }

template <class E, bool TA, bool TB>
__global__ void __launch_bounds__(THREADS) dmma_gemm_kernel(Args g) {
    using T = Tile<E, TA, TB>;
    constexpr bool CPLX = Elem<E>::cplx;
    constexpr int EB = Elem<E>::bytes;
    extern __shared__ __align__(16) unsigned char smem[];

    const int64_t m0 = (int64_t)blockIdx.x * BM;
    const int64_t n0 = (int64_t)blockIdx.y * BN;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wm = (warp & 1) * 32, wn = (warp >> 1) * 32;
    const int gq = lane >> 2, tq = lane & 3;

    // accumulators: 2 (m16) x 4 (n8) fragments x 4 doubles (x2 for complex)
    double acc_re[2][4][4] = {};
    double acc_im[CPLX ? 2 : 1][CPLX ? 4 : 1][4] = {};

    const int64_t ktiles = (g.k + BK - 1) / BK;
#pragma unroll
    for (int s = 0; s < STAGES - 1; ++s) {
        if (s < ktiles) load_stage<E, TA, TB>(g, smem + s * T::STAGE_BYTES, m0, n0, (int64_t)s * BK);
        cp_commit();
    }
    for (int64_t kt = 0; kt < ktiles; ++kt) {
        cp_wait<STAGES - 2>();
        __syncthreads();
        {   // prefetch tile kt + STAGES - 1 into the slot freed at kt - 1
            int64_t nk = kt + STAGES - 1;
            if (nk < ktiles) load_stage<E, TA, TB>(g, smem + (nk % STAGES) * T::STAGE_BYTES, m0, n0, nk * BK);
            cp_commit();
        }
        const unsigned char* stage = smem + (kt % STAGES) * T::STAGE_BYTES;
        const E* sA = reinterpret_cast<const E*>(stage);
        const E* sB = reinterpret_cast<const E*>(stage + T::A_ELEMS * EB);
#pragma unroll
        for (int kk = 0; kk < BK; kk += 4) {
            double ar[2][2], ai[2][2], br[4], bi[4];
#pragma unroll
            for (int mi = 0; mi < 2; ++mi)
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    ld_elem<E>(sA + T::a_idx(wm + mi * 16 + gq + 8 * h, kk + tq), ar[mi][h], ai[mi][h]);
                    if (CPLX && g.conj_a) ai[mi][h] = neg_bits(ai[mi][h]);
                }
#pragma unroll
            for (int ni = 0; ni < 4; ++ni) {
                ld_elem<E>(sB + T::b_idx(kk + tq, wn + ni * 8 + gq), br[ni], bi[ni]);
                if (CPLX && g.conj_b) bi[ni] = neg_bits(bi[ni]);
            }
#pragma unroll
            for (int mi = 0; mi < 2; ++mi)
#pragma unroll
                for (int ni = 0; ni < 4; ++ni) {
                    dmma(acc_re[mi][ni], ar[mi][0], ar[mi][1], br[ni]);
                    if constexpr (CPLX) {
                        dmma(acc_re[mi][ni], neg_bits(ai[mi][0]), neg_bits(ai[mi][1]), bi[ni]);
                        dmma(acc_im[mi][ni], ar[mi][0], ar[mi][1], bi[ni]);
                        dmma(acc_im[mi][ni], ai[mi][0], ai[mi][1], br[ni]);
                    }
                }
        }
    }
    cp_wait<0>();

    // Epilogue: C = alpha*acc + beta*C; C is not read when beta == 0.
    const bool beta_zero = (g.beta_re == 0.0 && g.beta_im == 0.0);
    E* C = reinterpret_cast<E*>(g.C);
#pragma unroll
    for (int mi = 0; mi < 2; ++mi)
#pragma unroll
        for (int ni = 0; ni < 4; ++ni)
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                int64_t i = m0 + wm + mi * 16 + gq + 8 * (r >> 1);
                int64_t j = n0 + wn + ni * 8 + 2 * tq + (r & 1);
                if (i >= g.m || j >= g.n) continue;
                E* p = C + i + j * g.ldc;
                if constexpr (!CPLX) {
                    double v = g.alpha_re * acc_re[mi][ni][r];
                    if (!beta_zero) v += g.beta_re * (double)(*p);
                    *p = (E)v;
                } else {
                    double xr = acc_re[mi][ni][r], xi = acc_im[mi][ni][r];
                    double vr = g.alpha_re * xr - g.alpha_im * xi;
                    double vi = g.alpha_re * xi + g.alpha_im * xr;
                    if (!beta_zero) {
                        double cr, ci;
                        ld_elem<E>(p, cr, ci);
                        vr += g.beta_re * cr - g.beta_im * ci;
                        vi += g.beta_re * ci + g.beta_im * cr;
                    }
                    E out;
                    out.x = vr; out.y = vi;
                    *p = out;
                }
            }
}

template <class E, bool TA, bool TB>
int launch_typed(const Args& a, cudaStream_t stream) {
    using T = Tile<E, TA, TB>;
    constexpr int smem = STAGES * T::STAGE_BYTES;
    auto kern = dmma_gemm_kernel<E, TA, TB>;
    static PerDevice<bool> configured;  // the attribute is set once per device
    bool done = false;
    CGB_CHECK(configured.get(
        [&](bool& v) {
            CGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
            v = true;
            return COSMA_GPU_SUCCESS;
        },
        &done));
    dim3 grid((unsigned)ceil_div(a.m, BM), (unsigned)ceil_div(a.n, BN));
    if (grid.y > 65535) return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "native gemm: n too large");
    kern<<<grid, THREADS, smem, stream>>>(a);
    CGB_CUDA(cudaGetLastError());
    return COSMA_GPU_SUCCESS;
}

template <class E>
int launch(const Args& a, bool ta, bool tb, cudaStream_t s) {
    if (!ta && !tb) return launch_typed<E, false, false>(a, s);
    if (!ta && tb) return launch_typed<E, false, true>(a, s);
    if (ta && !tb) return launch_typed<E, true, false>(a, s);
    return launch_typed<E, true, true>(a, s);
}

}  // namespace

int native_gemm(const GemmDesc& gd, cudaStream_t stream) {
    if (gd.m == 0 || gd.n == 0) return COSMA_GPU_SUCCESS;
    Args a;
    a.m = gd.m; a.n = gd.n; a.k = gd.k;
    a.A = gd.A; a.lda = gd.lda; a.B = gd.B; a.ldb = gd.ldb; a.C = gd.C; a.ldc = gd.ldc;
    a.alpha_re = gd.alpha[0]; a.alpha_im = gd.alpha[1];
    a.beta_re = gd.beta[0]; a.beta_im = gd.beta[1];
    a.conj_a = gd.opa == 2; a.conj_b = gd.opb == 2;
    const bool ta = gd.opa != 0, tb = gd.opb != 0;
    // Vector loads/stores of whole elements need element-aligned addresses
    // (16 bytes for complex double); reject misaligned buffers up front.
    const uintptr_t align = gd.scalar == Scalar::Z ? 16 : (gd.scalar == Scalar::S ? 4 : 8);
    if (((uintptr_t)gd.A | (uintptr_t)gd.B | (uintptr_t)gd.C) % align)
        return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "native gemm: buffers must be aligned to the element size");
    switch (gd.scalar) {
        case Scalar::D: return launch<double>(a, ta, tb, stream);
        case Scalar::S: return launch<float>(a, ta, tb, stream);
        case Scalar::Z: return launch<double2>(a, ta, tb, stream);
        case Scalar::C: return launch<float2>(a, ta, tb, stream);
    }
    return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "native gemm: bad scalar");
}

}  // namespace cgb
