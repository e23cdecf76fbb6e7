// COSTA layout transforms on a 1x1 process grid, as GPU kernels.
//
// On one rank a ScaLAPACK block-cyclic matrix is a single column-major
// buffer with leading dimension LLD (block-cyclic owner (i/mb) % 1 == 0 and
// local index (i/(mb*1))*mb + i%mb == i, the map restated in
// utils/pxgemm_utils.hpp:66-90), so costa::transformer's pack of a
// sub-matrix into COSMA's blocked layout (src/cosma/cosma_pxgemm.cpp:212-249,
// 338-343) is   dst(rows x cols, ld = rows) = op(src(ia:, ja:))   with op in
// {N, T, C}, and the back-transform of C (cosma_pxgemm.cpp:362-364) is
// dst = alpha*src + beta*dst.
//
// * pack: pure data movement, bit-exact (conjugation flips the sign bit of
//   the imaginary part, which is IEEE negation).  Transposing packs stage a
//   64x64-element tile (32x32 for 16-byte elements) through padded shared
//   memory so that both the HBM read and the HBM write are full-line
//   coalesced; non-transposing packs are a 16-byte-vectorised 2-D copy.
// * unpack: dst = fl(fl(alpha*src) + fl(beta*dst)) without FMA contraction;
//   dst is never read when beta == 0 (the reference's test pre-fills C with
//   NaN in that case, utils/pxgemm_utils.hpp:604-614).
#include "common.cuh"
#include "runtime.hpp"

#include <cmath>

namespace cgb {
namespace {

// 16-byte element carrier (complex double)
struct alignas(16) U128 { unsigned long long lo, hi; };

template <class U> __device__ __forceinline__ U conj_bits(U v);
template <> __device__ __forceinline__ unsigned long long conj_bits(unsigned long long v) {
    return v ^ 0x8000000000000000ull;  // complex float: imaginary float in the high word
}
template <> __device__ __forceinline__ U128 conj_bits(U128 v) {
    v.hi ^= 0x8000000000000000ull;
    return v;
}
template <> __device__ __forceinline__ unsigned conj_bits(unsigned v) { return v; }

// Transpose tile edge in elements: 64 for 4/8-byte elements (33 KB of
// static shared memory), 32 for 16-byte elements.  Rows are padded by one
// element, which makes the column-wise shared reads conflict-free for 4-byte
// elements and minimal-wavefront for 8/16-byte elements.
template <class U> struct TileEdge { static constexpr int value = sizeof(U) == 16 ? 32 : 64; };
constexpr int kTransposeThreads = 256;

// dst[i + j*ldd] = op(src)[i, j] = src[j + i*lds]   (op = T or C)
// Reads run along src's contiguous dimension, writes along dst's.
template <class U, bool CONJ>
__global__ void __launch_bounds__(kTransposeThreads) transpose_kernel(int64_t rows, int64_t cols,
                                                                      const U* __restrict__ src, int64_t lds,
                                                                      U* __restrict__ dst, int64_t ldd) {
    constexpr int TT = TileEdge<U>::value;
    constexpr int NY = kTransposeThreads / TT;
    __shared__ U tile[TT][TT + 1];
    const int64_t i0 = (int64_t)blockIdx.x * TT;  // dst rows = src cols
    const int64_t j0 = (int64_t)blockIdx.y * TT;  // dst cols = src rows
    const int tx = threadIdx.x % TT, ty = threadIdx.x / TT;
#pragma unroll 4
    for (int r = ty; r < TT; r += NY) {
        int64_t j = j0 + tx, i = i0 + r;
        if (j < cols && i < rows) tile[r][tx] = src[j + i * lds];
    }
    __syncthreads();
#pragma unroll 4
    for (int r = ty; r < TT; r += NY) {
        int64_t i = i0 + tx, j = j0 + r;
        if (i < rows && j < cols) {
            U v = tile[tx][r];
            if (CONJ) v = conj_bits(v);
            dst[i + j * ldd] = v;
        }
    }
}

// dst[i + j*ldd] = src[i + j*lds]   (op = N), column-per-warp vectorised copy.
template <class U>
__global__ void copy2d_kernel(int64_t rows, int64_t cols, const U* __restrict__ src, int64_t lds,
                              U* __restrict__ dst, int64_t ldd) {
    const int64_t total_cols = cols;
    for (int64_t j = blockIdx.y; j < total_cols; j += gridDim.y) {
        const U* s = src + j * lds;
        U* d = dst + j * ldd;
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (int64_t)gridDim.x * blockDim.x)
            d[i] = s[i];
    }
}

// 16-byte vectorised column copy when both columns are 16-byte aligned.
__global__ void copy2d_vec16_kernel(int64_t rows_bytes16, int64_t cols, const uint4* __restrict__ src,
                                    int64_t lds16, uint4* __restrict__ dst, int64_t ldd16) {
    for (int64_t j = blockIdx.y; j < cols; j += gridDim.y) {
        const uint4* s = src + j * lds16;
        uint4* d = dst + j * ldd16;
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows_bytes16;
             i += (int64_t)gridDim.x * blockDim.x)
            d[i] = s[i];
    }
}

template <class U>
__global__ void conj_copy2d_kernel(int64_t rows, int64_t cols, const U* __restrict__ src, int64_t lds,
                                   U* __restrict__ dst, int64_t ldd) {
    for (int64_t j = blockIdx.y; j < cols; j += gridDim.y)
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (int64_t)gridDim.x * blockDim.x)
            dst[i + j * ldd] = conj_bits(src[i + j * lds]);
}

// ---------------------------------------------------------------- unpack
template <class R>
__device__ __forceinline__ R mul_rn(R a, R b);
template <> __device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
template <> __device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
template <class R>
__device__ __forceinline__ R add_rn(R a, R b);
template <> __device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
template <> __device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
template <class R>
__device__ __forceinline__ R sub_rn(R a, R b);
template <> __device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
template <> __device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }

// fl(s * x) for a scale s = 2^e.  A normal x whose scaled exponent stays
// normal is scaled exactly by moving its exponent field - integer work
// instead of an FP64 multiply (GB300's FP64 pipe, not HBM, bounds the
// unpack otherwise); zeros, subnormals, Inf/NaN and results that leave the
// normal range take the multiply, so the result is fl(s*x) bit for bit.
// The rare multiply is a call, so that the compiler branches around it
// instead of issuing it predicated on every element.
__device__ __noinline__ double mul_rare(double s, double x) { return __dmul_rn(s, x); }
__device__ __noinline__ float mul_rare(float s, float x) { return __fmul_rn(s, x); }
__device__ __forceinline__ double mul_pow2(double s, int e, double x) {
    const long long b = __double_as_longlong(x);
    const int ex = (int)((b >> 52) & 0x7FF), ne = ex + e;
    if (ex == 0 || ex == 0x7FF || ne <= 0 || ne >= 0x7FF) return mul_rare(s, x);
    return __longlong_as_double(b + ((long long)e << 52));
}
__device__ __forceinline__ float mul_pow2(float s, int e, float x) {
    const int b = __float_as_int(x);
    const int ex = (b >> 23) & 0xFF, ne = ex + e;
    if (ex == 0 || ex == 0xFF || ne <= 0 || ne >= 0xFF) return mul_rare(s, x);
    return __int_as_float(b + (e << 23));
}

// fl(s * x) for a double s = +-m 2^e with an odd significand m of at most 11
// bits (1.5, 3, 0.75, ...): the 53-bit significand of x times m fits 64 bits,
// and its round-to-nearest-even to 53 bits with the exponents added is the
// IEEE product whenever that product is a normal number.  A zero x gives the
// signed zero; subnormal x, Inf/NaN and products outside the normal range
// take the multiply (rare: a call).  Integer work only, so that the unpack
// issues one FP64 instruction per element (the add) instead of two.
// With k = floor(log2 m), the product P = (2^52 + frac) m has its top bit at
// 52 + k or 53 + k, so one shift finds how many bits (sh) fall below the kept
// 53, and P + 2^(sh-1) - 1 + (bit sh of P), shifted by sh, is P rounded to
// nearest even.
__device__ __forceinline__ double mul_short(double s, uint32_t m, int e, int k, double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned long long sign = (b ^ (unsigned long long)__double_as_longlong(s)) & 0x8000000000000000ull;
    const int ex = (int)((b >> 52) & 0x7FF);
    if ((unsigned)(ex - 1) >= 0x7FEu) {  // zero, subnormal, Inf or NaN
        if ((b << 1) == 0) return __longlong_as_double((long long)sign);
        return mul_rare(s, x);
    }
    const unsigned long long P = ((b & 0xFFFFFFFFFFFFFull) | (1ull << 52)) * m;  // < 2^(54 + k)
    const int sh = k + (int)(P >> (53 + k));                                      // 0..11
    const unsigned long long lsb = (P >> sh) & 1ull;
    const unsigned long long bias = sh ? (1ull << (sh - 1)) - 1ull + lsb : 0ull;
    unsigned long long q = (P + bias) >> sh;
    int ne = ex + e + sh;
    const int carry = (int)(q >> 53);  // rounding carried into a new bit
    q >>= carry;
    ne += carry;
    if ((unsigned)(ne - 1) >= 0x7FEu) return mul_rare(s, x);  // product outside the normal range
    return __longlong_as_double((long long)(sign | ((unsigned long long)ne << 52) | (q & 0xFFFFFFFFFFFFFull)));
}

// How a real scale is applied: 0 = identity (s == 1), 1 = exponent shift
// (s a power of two, exponent e), 2 = multiply, 3 = short-significand
// product (double only: s = +-m 2^e, m odd, at most 11 bits).
template <class R>
struct ScaleMode {
    int mode, e;
    uint32_t m;
    int k;  // floor(log2 m)
};
template <class R>
__host__ ScaleMode<R> scale_mode(double s) {
    int e = 0;
    const double f = std::frexp(s, &e);  // s = f * 2^e, f in [0.5, 1)
    if (s == 1.0) return {0, 0, 1, 0};
    if (f == 0.5 && std::isfinite(s)) return {1, e - 1, 1, 0};
    if (sizeof(R) == 8 && std::isfinite(s) && s != 0.0) {
        double a = std::fabs(f);
        int ae = e;
        for (int i = 0; i < 11 && a != std::floor(a); ++i) {  // a * 2^ae == |s|; make a an integer
            a *= 2.0;
            --ae;
        }
        if (a == std::floor(a) && a < 2048.0) {
            int k = 0;
            while ((2u << k) <= (uint32_t)a) ++k;
            return {3, ae, (uint32_t)a, k};
        }
    }
    return {2, 0, 1, 0};
}
template <int MODE, class R>
__device__ __forceinline__ R apply_scale(R s, const ScaleMode<R>& md, R x) {
    if constexpr (MODE == 0) return x;
    else if constexpr (MODE == 1) return mul_pow2(s, md.e, x);
    else if constexpr (MODE == 3) {
        if constexpr (sizeof(R) == 8) return mul_short(s, md.m, md.e, md.k, x);
        else return mul_rn(s, x);  // not chosen for float
    }
    else return mul_rn(s, x);
}

// real: d = fl(fl(alpha*s) + fl(beta*d)); beta == 0 -> d = fl(alpha*s).  The
// modes only choose how each (exact or rounded) product is formed, never the
// result: a multiply by 1 or by a power of two is exact unless it leaves the
// normal range, where mul_pow2 multiplies.
//
// Each thread takes four elements of a column, a block stride apart, and
// issues all their loads before any arithmetic: GB300's FP64 pipe is narrow
// (the multiply and add of one element cost about what its 24 bytes of HBM
// traffic do), so the loads of the next elements must be in flight while the
// FP64 work of the current ones runs.  The modes are template parameters:
// with runtime modes the compiler issues every mode's FP64 multiply,
// predicated, for every element.
template <class R, int AM, int BM, bool READ>
__global__ void unpack_real_kernel(int64_t rows, int64_t cols, R alpha, ScaleMode<R> am, const R* __restrict__ src,
                                   int64_t lds, R beta, ScaleMode<R> bm, R* __restrict__ dst, int64_t ldd) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t j = blockIdx.y; j < cols; j += gridDim.y) {
        const R* s = src + j * lds;
        R* d = dst + j * ldd;
        for (int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i0 < rows; i0 += 4 * stride) {
            R x[4], y[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int64_t i = i0 + q * stride;
                x[q] = i < rows ? s[i] : R(0);
                y[q] = (READ && i < rows) ? d[i] : R(0);
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int64_t i = i0 + q * stride;
                if (i >= rows) break;
                R v = apply_scale<AM>(alpha, am, x[q]);
                if constexpr (READ) v = add_rn(v, apply_scale<BM>(beta, bm, y[q]));
                d[i] = v;
            }
        }
    }
}

// The same on 16-byte pairs of doubles (rows, leading dimensions even and
// both arrays 16-byte aligned): a warp moves 512 bytes per load instead of
// 256, which the unpack needs to keep HBM busy once its FP64 work is one
// instruction per element.
template <int AM, int BM, bool READ>
__global__ void unpack_real2_kernel(int64_t rows2, int64_t cols, double alpha, ScaleMode<double> am,
                                    const double2* __restrict__ src, int64_t lds2, double beta, ScaleMode<double> bm,
                                    double2* __restrict__ dst, int64_t ldd2) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t j = blockIdx.y; j < cols; j += gridDim.y) {
        const double2* s = src + j * lds2;
        double2* d = dst + j * ldd2;
        for (int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i0 < rows2; i0 += 4 * stride) {
            double2 x[4], y[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int64_t i = i0 + q * stride;
                x[q] = i < rows2 ? s[i] : make_double2(0.0, 0.0);
                y[q] = (READ && i < rows2) ? d[i] : make_double2(0.0, 0.0);
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int64_t i = i0 + q * stride;
                if (i >= rows2) break;
                double2 v;
                v.x = apply_scale<AM>(alpha, am, x[q].x);
                v.y = apply_scale<AM>(alpha, am, x[q].y);
                if constexpr (READ) {
                    v.x = add_rn(v.x, apply_scale<BM>(beta, bm, y[q].x));
                    v.y = add_rn(v.y, apply_scale<BM>(beta, bm, y[q].y));
                }
                d[i] = v;
            }
        }
    }
}

// complex: x*y = (xr*yr - xi*yi) + (xr*yi + xi*yr) i, every product and sum
// rounded separately (no contraction); d = fl(alpha*s + beta*d) componentwise.
template <class R, class V>
__device__ __forceinline__ V cmul_rn(R ar, R ai, V s) {
    V out;
    out.x = sub_rn(mul_rn(ar, s.x), mul_rn(ai, s.y));
    out.y = add_rn(mul_rn(ar, s.y), mul_rn(ai, s.x));
    return out;
}
template <class R, class V>
__global__ void unpack_cplx_kernel(int64_t rows, int64_t cols, R ar, R ai, const V* __restrict__ src, int64_t lds,
                                   R br, R bi, V* __restrict__ dst, int64_t ldd, int read_dst) {
    for (int64_t j = blockIdx.y; j < cols; j += gridDim.y)
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (int64_t)gridDim.x * blockDim.x) {
            V v = cmul_rn<R, V>(ar, ai, src[i + j * lds]);
            if (read_dst) {
                V w = cmul_rn<R, V>(br, bi, dst[i + j * ldd]);
                v.x = add_rn(v.x, w.x);
                v.y = add_rn(v.y, w.y);
            }
            dst[i + j * ldd] = v;
        }
}

// C <- beta * C (k == 0 or alpha == 0 corner case of p?gemm / gemm).
// beta == 0 writes zeros without reading C.
template <class R>
__global__ void scale_real_kernel(int64_t rows, int64_t cols, R beta, R* C, int64_t ldc) {
    for (int64_t j = blockIdx.y; j < cols; j += gridDim.y)
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (int64_t)gridDim.x * blockDim.x)
            C[i + j * ldc] = (beta == R(0)) ? R(0) : mul_rn(beta, C[i + j * ldc]);
}
template <class R, class V>
__global__ void scale_cplx_kernel(int64_t rows, int64_t cols, R br, R bi, V* C, int64_t ldc) {
    for (int64_t j = blockIdx.y; j < cols; j += gridDim.y)
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (int64_t)gridDim.x * blockDim.x) {
            V v;
            if (br == R(0) && bi == R(0)) { v.x = R(0); v.y = R(0); }
            else v = cmul_rn<R, V>(br, bi, C[i + j * ldc]);
            C[i + j * ldc] = v;
        }
}

dim3 grid2d(int64_t rows, int64_t cols, int threads) {
    int64_t bx = ceil_div(rows, threads);
    if (bx > 64) bx = 64;  // columns beyond the grid's height are strided; rows beyond 64 blocks too
    int64_t by = cols < 65535 ? cols : 65535;
    if (by < 1) by = 1;
    if (bx < 1) bx = 1;
    return dim3((unsigned)bx, (unsigned)by);
}

template <class U>
int pack_typed(int op, int64_t rows, int64_t cols, const void* src, int64_t lds, void* dst, int64_t ldd,
               cudaStream_t s) {
    if (op == 0) {
        const size_t eb = sizeof(U);
        if (((uintptr_t)src % 16 == 0) && ((uintptr_t)dst % 16 == 0) && ((lds * eb) % 16 == 0) &&
            ((ldd * eb) % 16 == 0) && ((rows * eb) % 16 == 0)) {
            int64_t r16 = rows * eb / 16;
            copy2d_vec16_kernel<<<grid2d(r16, cols, 256), 256, 0, s>>>(r16, cols, (const uint4*)src, lds * eb / 16,
                                                                         (uint4*)dst, ldd * eb / 16);
        } else {
            copy2d_kernel<U><<<grid2d(rows, cols, 256), 256, 0, s>>>(rows, cols, (const U*)src, lds, (U*)dst, ldd);
        }
    } else if (op == 3) {  // conjugate without transpose (internal use)
        conj_copy2d_kernel<U><<<grid2d(rows, cols, 256), 256, 0, s>>>(rows, cols, (const U*)src, lds, (U*)dst, ldd);
    } else {
        constexpr int TT = TileEdge<U>::value;
        dim3 grid((unsigned)ceil_div(rows, TT), (unsigned)ceil_div(cols, TT));
        if (grid.y > 65535) return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "pack: too many columns");
        if (op == 2)
            transpose_kernel<U, true><<<grid, kTransposeThreads, 0, s>>>(rows, cols, (const U*)src, lds, (U*)dst, ldd);
        else
            transpose_kernel<U, false><<<grid, kTransposeThreads, 0, s>>>(rows, cols, (const U*)src, lds, (U*)dst, ldd);
    }
    CGB_CUDA(cudaGetLastError());
    return COSMA_GPU_SUCCESS;
}

}  // namespace

int pack_device(int op, bool is_complex, int elem_bytes, int64_t rows, int64_t cols, const void* src, int64_t lds,
                void* dst, int64_t ldd, cudaStream_t s) {
    if (rows == 0 || cols == 0) return COSMA_GPU_SUCCESS;
    if (op == 2 && !is_complex) op = 1;  // conjugate transpose of real data is a transpose
    if (elem_bytes == 4 || elem_bytes == 8 || elem_bytes == 16) {
        if (((uintptr_t)src | (uintptr_t)dst) % (uintptr_t)elem_bytes)
            return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "pack: buffers must be aligned to the element size");
    }
    switch (elem_bytes) {
        case 4: return pack_typed<unsigned>(op, rows, cols, src, lds, dst, ldd, s);
        case 8: return pack_typed<unsigned long long>(op, rows, cols, src, lds, dst, ldd, s);
        case 16: return pack_typed<U128>(op, rows, cols, src, lds, dst, ldd, s);
    }
    return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "pack: elem_bytes must be 4, 8 or 16");
}

// One instantiation of the real unpack: 16-byte pairs when `pairs`.
template <class R, int A, int B, bool RD>
void launch_unpack_one(dim3 g, dim3 g2, bool pairs, cudaStream_t st, int64_t rows, int64_t cols, R alpha,
                       ScaleMode<R> am, const R* src, int64_t lds, R beta, ScaleMode<R> bm, R* dst, int64_t ldd) {
    if constexpr (sizeof(R) == 8) {
        if (pairs) {
            unpack_real2_kernel<A, B, RD><<<g2, 256, 0, st>>>(rows / 2, cols, alpha, am, (const double2*)src, lds / 2,
                                                              beta, bm, (double2*)dst, ldd / 2);
            return;
        }
    }
    unpack_real_kernel<R, A, B, RD><<<g, 256, 0, st>>>(rows, cols, alpha, am, src, lds, beta, bm, dst, ldd);
}

// The real unpack for the scale modes of alpha and beta (beta's only when C
// is read); 16-byte pairs of doubles where the layout allows.
template <class R>
void launch_unpack_real(dim3 g, cudaStream_t st, int64_t rows, int64_t cols, R alpha, ScaleMode<R> am, const R* src,
                        int64_t lds, R beta, ScaleMode<R> bm, R* dst, int64_t ldd, bool read_dst) {
    const bool pairs = sizeof(R) == 8 && rows % 2 == 0 && lds % 2 == 0 && ldd % 2 == 0 &&
                       ((uintptr_t)src | (uintptr_t)dst) % 16 == 0;
    const dim3 g2 = grid2d(ceil_div(rows / 2, 4), cols, 256);
#define CGB_UNPACK(A, B, RD) \
    launch_unpack_one<R, A, B, RD>(g, g2, pairs, st, rows, cols, alpha, am, src, lds, beta, bm, dst, ldd)
#define CGB_UNPACK_B(A)                              \
    if (!read_dst) CGB_UNPACK(A, 0, false);          \
    else if (bm.mode == 0) CGB_UNPACK(A, 0, true);   \
    else if (bm.mode == 1) CGB_UNPACK(A, 1, true);   \
    else if (bm.mode == 3) CGB_UNPACK(A, 3, true);   \
    else CGB_UNPACK(A, 2, true);
    if (am.mode == 0) { CGB_UNPACK_B(0) }
    else if (am.mode == 1) { CGB_UNPACK_B(1) }
    else if (am.mode == 3) { CGB_UNPACK_B(3) }
    else { CGB_UNPACK_B(2) }
#undef CGB_UNPACK_B
#undef CGB_UNPACK
}

int unpack_device(Scalar sc, int64_t rows, int64_t cols, const double* alpha, const void* src, int64_t lds,
                  const double* beta, void* dst, int64_t ldd, cudaStream_t s) {
    if (rows == 0 || cols == 0) return COSMA_GPU_SUCCESS;
    const uintptr_t align = sc == Scalar::Z ? 16 : (sc == Scalar::S ? 4 : 8);
    if (((uintptr_t)src | (uintptr_t)dst) % align)
        return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "unpack: buffers must be aligned to the element size");
    const int read_dst = !(beta[0] == 0.0 && (!scalar_complex(sc) || beta[1] == 0.0));
    dim3 g = grid2d(rows, cols, 256);
    dim3 g4 = grid2d(ceil_div(rows, 4), cols, 256);  // the real kernels take four elements per thread
    switch (sc) {
        case Scalar::D:
            launch_unpack_real<double>(g4, s, rows, cols, alpha[0], scale_mode<double>(alpha[0]), (const double*)src,
                                       lds, beta[0], scale_mode<double>(beta[0]), (double*)dst, ldd, read_dst);
            break;
        case Scalar::S:
            launch_unpack_real<float>(g4, s, rows, cols, (float)alpha[0], scale_mode<float>((float)alpha[0]),
                                      (const float*)src, lds, (float)beta[0], scale_mode<float>((float)beta[0]),
                                      (float*)dst, ldd, read_dst);
            break;
        case Scalar::Z:
            unpack_cplx_kernel<double, double2><<<g, 256, 0, s>>>(rows, cols, alpha[0], alpha[1],
                                                                  (const double2*)src, lds, beta[0], beta[1],
                                                                  (double2*)dst, ldd, read_dst);
            break;
        case Scalar::C:
            unpack_cplx_kernel<float, float2><<<g, 256, 0, s>>>(rows, cols, (float)alpha[0], (float)alpha[1],
                                                                (const float2*)src, lds, (float)beta[0],
                                                                (float)beta[1], (float2*)dst, ldd, read_dst);
            break;
    }
    CGB_CUDA(cudaGetLastError());
    return COSMA_GPU_SUCCESS;
}

int scale_matrix_device(Scalar sc, int64_t rows, int64_t cols, const double* beta, void* C, int64_t ldc,
                        cudaStream_t s) {
    if (rows == 0 || cols == 0) return COSMA_GPU_SUCCESS;
    const bool one = beta[0] == 1.0 && (!scalar_complex(sc) || beta[1] == 0.0);
    if (one) return COSMA_GPU_SUCCESS;
    const uintptr_t align = sc == Scalar::Z ? 16 : (sc == Scalar::S ? 4 : 8);
    if ((uintptr_t)C % align)
        return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "scale: C must be aligned to the element size");  // scale_matrix returns early for beta == 1 (cosma_pxgemm.cpp:399)
    dim3 g = grid2d(rows, cols, 256);
    switch (sc) {
        case Scalar::D: scale_real_kernel<double><<<g, 256, 0, s>>>(rows, cols, beta[0], (double*)C, ldc); break;
        case Scalar::S: scale_real_kernel<float><<<g, 256, 0, s>>>(rows, cols, (float)beta[0], (float*)C, ldc); break;
        case Scalar::Z:
            scale_cplx_kernel<double, double2><<<g, 256, 0, s>>>(rows, cols, beta[0], beta[1], (double2*)C, ldc);
            break;
        case Scalar::C:
            scale_cplx_kernel<float, float2><<<g, 256, 0, s>>>(rows, cols, (float)beta[0], (float)beta[1],
                                                               (float2*)C, ldc);
            break;
    }
    CGB_CUDA(cudaGetLastError());
    return COSMA_GPU_SUCCESS;
}

}  // namespace cgb

extern "C" {

int costa_gpu_pack(char op, int is_complex, int elem_bytes, int64_t rows, int64_t cols, const void* src,
                   int64_t ld_src, void* dst, int64_t ld_dst, void* stream) {
    cgb::clear_error();
    int o = cgb::parse_op(op);
    if (o < 0) return cgb::set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "costa_gpu_pack: op must be N, T or C");
    if (rows < 0 || cols < 0) return cgb::set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "costa_gpu_pack: negative size");
    // src is (rows x cols) for N, (cols x rows) for T/C
    int64_t src_rows = o == 0 ? rows : cols;
    if (ld_src < (src_rows > 1 ? src_rows : 1) || ld_dst < (rows > 1 ? rows : 1))
        return cgb::set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "costa_gpu_pack: leading dimension too small");
    return cgb::pack_device(o, is_complex != 0, elem_bytes, rows, cols, src, ld_src, dst, ld_dst,
                            (cudaStream_t)stream);
}

static int unpack_common(cgb::Scalar sc, int64_t rows, int64_t cols, const double* a, const void* src, int64_t lds,
                         const double* b, void* dst, int64_t ldd, void* stream) {
    cgb::clear_error();
    if (rows < 0 || cols < 0 || lds < (rows > 1 ? rows : 1) || ldd < (rows > 1 ? rows : 1))
        return cgb::set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "costa_gpu_unpack: bad size or leading dimension");
    return cgb::unpack_device(sc, rows, cols, a, src, lds, b, dst, ldd, (cudaStream_t)stream);
}

int costa_gpu_unpack_d(int64_t rows, int64_t cols, double alpha, const double* src, int64_t ld_src, double beta,
                       double* dst, int64_t ld_dst, void* stream) {
    double a[2] = {alpha, 0}, b[2] = {beta, 0};
    return unpack_common(cgb::Scalar::D, rows, cols, a, src, ld_src, b, dst, ld_dst, stream);
}
int costa_gpu_unpack_s(int64_t rows, int64_t cols, float alpha, const float* src, int64_t ld_src, float beta,
                       float* dst, int64_t ld_dst, void* stream) {
    double a[2] = {alpha, 0}, b[2] = {beta, 0};
    return unpack_common(cgb::Scalar::S, rows, cols, a, src, ld_src, b, dst, ld_dst, stream);
}
int costa_gpu_unpack_z(int64_t rows, int64_t cols, const double* alpha, const double* src, int64_t ld_src,
                       const double* beta, double* dst, int64_t ld_dst, void* stream) {
    double a[2] = {alpha[0], alpha[1]}, b[2] = {beta[0], beta[1]};
    return unpack_common(cgb::Scalar::Z, rows, cols, a, src, ld_src, b, dst, ld_dst, stream);
}
int costa_gpu_unpack_c(int64_t rows, int64_t cols, const float* alpha, const float* src, int64_t ld_src,
                       const float* beta, float* dst, int64_t ld_dst, void* stream) {
    double a[2] = {alpha[0], alpha[1]}, b[2] = {beta[0], beta[1]};
    return unpack_common(cgb::Scalar::C, rows, cols, a, src, ld_src, b, dst, ld_dst, stream);
}

}  // extern "C"
