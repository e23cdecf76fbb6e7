// Shared device code of the Ozaki-split GEMMs (single problems in ozaki.cu,
// grouped batches in ozaki_grouped.cu): tile constants, the accumulator-group
// schedule, row scaling, digit slicing, the 128-bit recombination and the
// epilogue that drains TMEM into it.
#pragma once

#include "common.cuh"
#include "tc_common.cuh"
#include "runtime.hpp"

#include <cuda_fp8.h>

#include <cstdint>

namespace cgb {
namespace oz {

constexpr int BM = 128, BN = 256, BK = 128;  // BK in bytes = FP8 elements
constexpr int STAGES = 4;
constexpr int A_STAGE = BM * BK, B_STAGE = BN * BK, STAGE_BYTES = A_STAGE + B_STAGE;
constexpr int THREADS = 192;
constexpr int MAX_SLICES = 16;
constexpr int MAX_UNITS = 144, MAX_GROUPS = 144;
constexpr int64_t MAX_K_PER_CALL = 65536;  // 256 * k <= 2^24 for one product per accumulator
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 256;
constexpr int KB_CHUNK = 4;  // K blocks per chunk in the group loop (512 FP8 elements)

struct Schedule {
    int n_groups;
    int kb_count;           // K blocks of 128
    int a_rows_pad, b_rows_pad;
    uint8_t us[MAX_UNITS], ut[MAX_UNITS];        // slice indices (0-based) of each product
    uint16_t gfirst[MAX_GROUPS];                 // first product of each accumulator group
    uint8_t gcount[MAX_GROUPS], gshift[MAX_GROUPS];
};

// --------------------------------------------------------------- scaling
struct RowState {
    int emax;     // floor(log2 max |x|) over the elements seen, INT_MIN/2 if none
    float mass;   // sum of 2^(floor(log2|x|) - emax)
    int lsbmin = 1 << 30;  // lowest weight of a set significand bit (log2), where tracked
};

__device__ __forceinline__ float pow2f(int e) {  // 2^e as float, 0 below the normal range
    return e < -126 ? 0.0f : __int_as_float((127 + e) << 23);
}

// floor(log2|x|) of a finite nonzero double from its bits, and the log2
// weight of its lowest set significand bit; sets *bad for Inf/NaN.
__device__ __forceinline__ bool element_log2(double x, int* lb, unsigned* bad, int* lsb = nullptr) {
    unsigned long long b = (unsigned long long)__double_as_longlong(x);
    int ef = (int)((b >> 52) & 0x7FF);
    unsigned long long frac = b & 0xFFFFFFFFFFFFFull;
    if (ef == 0x7FF) { *bad = 1; return false; }
    if (ef == 0) {
        if (frac == 0) return false;
        *lb = (63 - __clzll((long long)frac)) - 1074;
        if (lsb) *lsb = __ffsll((long long)frac) - 1 - 1074;
        return true;
    }
    *lb = ef - 1023;
    if (lsb) *lsb = __ffsll((long long)(frac | (1ull << 52))) - 1 + ef - 1075;
    return true;
}

__device__ __forceinline__ void state_add(RowState& s, int lb, int lsb = 1 << 30) {
    if (lb > s.emax) {
        s.mass = s.mass * pow2f(s.emax - lb) + 1.0f;
        s.emax = lb;
    } else {
        s.mass += pow2f(lb - s.emax);
    }
    s.lsbmin = min(s.lsbmin, lsb);
}
__device__ __forceinline__ RowState state_merge(RowState a, RowState b) {
    RowState r;
    r.emax = max(a.emax, b.emax);
    r.mass = a.mass * pow2f(a.emax - r.emax) + b.mass * pow2f(b.emax - r.emax);
    r.lsbmin = min(a.lsbmin, b.lsbmin);
    return r;
}

struct Stats {
    unsigned nonfinite;
    float spread[2];    // max over rows of log2(2k / mass) for A rows / B columns
    int exact_bits[2];  // max over rows of E - (lowest set bit): fraction bits that keep every element exact
};

// Finishes one row: writes the scale exponent (E = emax + 1, 0 for zero
// rows) and folds the row's spread estimate into the global maximum.
__device__ __forceinline__ void finish_row(RowState s, int64_t k, int* exp_out, Stats* st, int which) {
    if (s.mass <= 0.0f) {
        *exp_out = 0;
        return;
    }
    *exp_out = s.emax + 1;
    if (s.lsbmin < (1 << 30)) atomicMax(&st->exact_bits[which], s.emax + 1 - s.lsbmin);
    float spread = log2f(2.0f * (float)k / s.mass);
    if (spread < 0.0f) spread = 0.0f;
    atomicMax((int*)&st->spread[which], __float_as_int(spread));  // non-negative floats order as ints
}

// --------------------------------------------------------------- slicing
// 16 in every 5-bit field below the top digit: adding it to X turns the
// balanced digits into plain 5-bit fields offset by 16 (see digits_of).
template <int S>
struct DigitOffset {
    static constexpr unsigned long long word(int w) {
        unsigned long long v = 0;
        for (int p = 0; p < S - 1; ++p) {
            const int bit = 5 * p + 4;
            if (bit / 64 == w) v |= 1ull << (bit % 64);
        }
        return v;
    }
    static constexpr unsigned long long lo = word(0), hi = word(1);
};

// 5-bit field at bit `pos` of the 128-bit integer (hi:lo); pos is a constant.
template <int POS>
__device__ __forceinline__ int field5(unsigned long long lo, unsigned long long hi) {
    if constexpr (POS + 5 <= 64) return (int)((lo >> POS) & 31ull);
    else if constexpr (POS >= 64) return (int)((hi >> (POS - 64)) & 31ull);
    else return (int)(((lo >> POS) | (hi << (64 - POS))) & 31ull);
}

template <int S, int P>
struct DigitLoop {
    __device__ __forceinline__ static void run(unsigned long long lo, unsigned long long hi, bool neg,
                                               int (&d)[S]) {
        const int dd = field5<5 * P>(lo, hi) - 16;
        d[S - 1 - P] = neg ? -dd : dd;
        DigitLoop<S, P + 1>::run(lo, hi, neg, d);
    }
};
template <int S>
struct DigitLoop<S, S - 1> {  // the leading digit: everything above the last field
    __device__ __forceinline__ static void run(unsigned long long lo, unsigned long long hi, bool neg,
                                               int (&d)[S]) {
        constexpr int pos = 5 * (S - 1);
        const int top = pos >= 64 ? (int)(hi >> (pos - 64)) : (int)((lo >> pos) | (hi << (64 - pos)));
        d[0] = neg ? -top : top;
    }
};

// Balanced base-32 digits of |x| / 2^E rounded to F = 4 + 5(S-1) fraction
// bits (round half away from zero), most significant first, sign applied.
// With X = round(|x| 2^(F-E)) < 2^(F+1), the digits below the top one are
// d_p = u_p - 32 c_(p+1) with u_p = (5-bit field p of X) + c_p and carry
// c_(p+1) = [u_p >= 16].  Adding B = sum_p 16 * 32^p to X performs exactly that
// carry chain: field p of X + B equals u_p + 16 - 32 c_(p+1), so d_p = field_p(X + B) - 16,
// and the leading digit is what remains above the last field.
template <int S>
__device__ __forceinline__ void digits_of(double x, int E, int (&d)[S]) {
    unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const bool neg = (b >> 63) != 0;
    const int ef = (int)((b >> 52) & 0x7FF);
    unsigned long long M = b & 0xFFFFFFFFFFFFFull;
    int eu;
    if (ef == 0) eu = -1074; else { M |= 1ull << 52; eu = ef - 1075; }
    constexpr int F = 4 + 5 * (S - 1);
    int sh = eu - E + F;  // X = M * 2^sh
    if (M == 0) sh = 0;
    if (sh < 0) {
        const int r = -sh;
        M = r > 63 ? 0ull : (M + (1ull << (r - 1))) >> r;
        sh = 0;
    }
    // X = M << sh as a 128-bit integer (0 <= sh < F, X < 2^(F+1) <= 2^80)
    unsigned long long xlo, xhi;
    if (sh == 0) { xlo = M; xhi = 0; }
    else if (sh < 64) { xlo = M << sh; xhi = M >> (64 - sh); }
    else { xlo = 0; xhi = M << (sh - 64); }
    const unsigned long long ylo = xlo + DigitOffset<S>::lo;
    const unsigned long long yhi = xhi + DigitOffset<S>::hi + (ylo < xlo ? 1ull : 0ull);
    DigitLoop<S, 0>::run(ylo, yhi, neg, d);
}

__device__ __forceinline__ uint32_t pack4_e4m3(int a, int b, int c, int e) {
    __nv_fp8x2_storage_t lo = __nv_cvt_float2_to_fp8x2(make_float2((float)a, (float)b), __NV_SATFINITE, __NV_E4M3);
    __nv_fp8x2_storage_t hi = __nv_cvt_float2_to_fp8x2(make_float2((float)c, (float)e), __NV_SATFINITE, __NV_E4M3);
    return (uint32_t)lo | ((uint32_t)hi << 16);
}

// Writes the S E4M3 digit slices of a (rows x k) operand, row-major with
// row pitch k_pad, zero-padded to rows_pad x k_pad.  Each thread handles 16
// consecutive K elements of one row.  kcontig: element (r, l) at X[l + r*ld],
// else at X[r + l*ld].  A warp covers 8 rows x 64 K elements, so its slice
// stores are 64-byte runs along K in either layout, and its loads are
// 64-byte runs along rows (X[r + l*ld]) or along K (X[l + r*ld]).
template <int S, bool KCONTIG>
__device__ __forceinline__ void split_block(const double* __restrict__ X, int64_t ld, int64_t rows, int64_t k,
                                            const int* __restrict__ exps, int64_t k_pad, int64_t rows_pad,
                                            uint8_t* __restrict__ out, int64_t bx, int64_t by) {
    const int t = threadIdx.x;
    const int64_t r = bx * 64 + t / 4;
    const int kc = t % 4;
    const int64_t l0 = by * 64 + kc * 16;
    if (r >= rows_pad || l0 >= k_pad) return;
    const int E = r < rows ? exps[r] : 0;
    uint32_t packed[S][4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        int dg[4][S];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int64_t l = l0 + q * 4 + e;
            double x = 0.0;
            if (r < rows && l < k) x = KCONTIG ? X[l + r * ld] : X[r + l * ld];
            digits_of<S>(x, E, dg[e]);
        }
#pragma unroll
        for (int s = 0; s < S; ++s) packed[s][q] = pack4_e4m3(dg[0][s], dg[1][s], dg[2][s], dg[3][s]);
    }
#pragma unroll
    for (int s = 0; s < S; ++s) {
        uint4 v = make_uint4(packed[s][0], packed[s][1], packed[s][2], packed[s][3]);
        *reinterpret_cast<uint4*>(out + (int64_t)s * rows_pad * k_pad + r * k_pad + l0) = v;
    }
}

// --------------------------------------------------- 128-bit recombination
__device__ __forceinline__ void add_shifted(unsigned long long& lo, unsigned long long& hi, int x, int sh) {
    const long long xs = x;
    unsigned long long alo, ahi;
    if (sh == 0) { alo = (unsigned long long)xs; ahi = (unsigned long long)(xs >> 63); }
    else if (sh < 64) { alo = (unsigned long long)xs << sh; ahi = (unsigned long long)(xs >> (64 - sh)); }
    else { alo = 0; ahi = (unsigned long long)(xs << (sh - 64)); }
    const unsigned long long nlo = lo + alo;
    hi = hi + ahi + (nlo < lo ? 1ull : 0ull);
    lo = nlo;
}

// Round-to-nearest-even conversion of the signed 128-bit integer (hi:lo)
// times 2^e2 to double (subnormal and overflow results included).
__device__ __forceinline__ double i128_to_double(unsigned long long lo, unsigned long long hi, int e2) {
    const bool neg = (long long)hi < 0;
    if (neg) {
        lo = ~lo + 1ull;
        hi = ~hi + (lo == 0 ? 1ull : 0ull);
    }
    if (hi == 0 && lo == 0) return 0.0;
    const int msb = hi ? 127 - __clzll((long long)hi) : 63 - __clzll((long long)lo);
    int e_lsb = msb - 52 + e2;  // weight of the last kept bit for a normal result
    int r = msb - 52;           // bits dropped
    if (e_lsb < -1074) {        // subnormal result: fixed last-bit weight 2^-1074
        r += -1074 - e_lsb;
        e_lsb = -1074;
    }
    unsigned long long mant;
    if (r <= 0) {
        mant = lo << (-r);  // msb <= 52: the value fits in lo
    } else if (r > 127) {
        mant = 0;  // far below the smallest subnormal
    } else {
        // mant = V >> r, guard = bit r-1, sticky = bits below r-1
        unsigned long long q, g, st;
        if (r < 64) {
            q = (lo >> r) | (hi << (64 - r));
            g = (lo >> (r - 1)) & 1ull;
            st = (r - 1) > 0 ? (lo & ((1ull << (r - 1)) - 1ull)) : 0ull;
        } else if (r == 64) {
            q = hi;
            g = lo >> 63;
            st = lo & 0x7FFFFFFFFFFFFFFFull;
        } else {
            q = hi >> (r - 64);
            g = (hi >> (r - 65)) & 1ull;
            st = lo | ((r - 65) > 0 ? (hi & ((1ull << (r - 65)) - 1ull)) : 0ull);
        }
        mant = q;
        if (g && (st || (mant & 1ull))) ++mant;
    }
    unsigned long long bits;
    const bool normal = e_lsb > -1074 || mant >= (1ull << 52);
    if (mant >= (1ull << 53)) {  // rounding carried into a new bit
        mant >>= 1;
        ++e_lsb;
    }
    if (normal && mant >= (1ull << 52)) {
        const int be = e_lsb + 52 + 1023;
        if (be >= 2047) bits = 0x7FF0000000000000ull;
        else bits = ((unsigned long long)be << 52) | (mant & 0xFFFFFFFFFFFFFull);
    } else {
        bits = mant;  // subnormal (or the smallest normal reached by rounding)
    }
    if (neg) bits |= 0x8000000000000000ull;
    return __longlong_as_double((long long)bits);
}

// Tile order: strips of kStripM M-tiles, N-tiles within a strip, M-tiles
// fastest.  The 152 CTAs of one wave then cover a ~16 x 10 block of tiles,
// so every A- and B-slice panel a wave needs is fetched from HBM once and
// served to the other CTAs of its row / column from L2.
constexpr int kStripM = 16;
__device__ __forceinline__ void tile_coords(int tile, int num_m, int num_n, int& mb, int& nb,
                                            int strip_m = kStripM) {
    const int strip = tile / (strip_m * num_n);
    const int r = tile - strip * strip_m * num_n;
    const int h = min(strip_m, num_m - strip * strip_m);  // the last strip may be shorter
    nb = r / h;
    mb = strip * strip_m + r % h;
}

// Epilogue of one output tile (rows mb*128.., columns nb*256..): drains the
// tile's accumulator groups from TMEM, adds each at its weight into the
// 128-bit partial sums W and, after the last group, rounds the sums to FP64
// and writes alpha*r + beta*C.  `release(buf)` hands accumulator `buf` back
// to the MMA issuer.  Returns false if a wait failed.
// P supplies the output description: m, n, ldc, n_split, cs, C, expA, expB,
// alpha, beta, alpha_one, beta_zero, L, err.
template <class P, class Release>
__device__ __forceinline__ bool epilogue_tile(const P& p, const Schedule& sc, int mb, int nb, uint32_t tmem, int quad,
                                              int lane, ulonglong2* W, uint64_t* accf, uint32_t& acc_it,
                                              uint64_t pol_keep, uint64_t pol_stream, Release release) {
    const int row = quad * 32 + lane;
    const int64_t gi = (int64_t)mb * BM + row;
    const int Ei = p.expA[gi];
    const int last = sc.n_groups - 1;
    for (int g = 0; g <= last; ++g, ++acc_it) {
        const uint32_t buf = acc_it & 1;
        // all lanes must agree before the warp-collective TMEM loads
        if (!__all_sync(0xffffffffu, tc::mbar_wait(&accf[buf], (acc_it >> 1) & 1, p.err, kDevTimeoutAcc)))
            return false;
        tc::tc_fence_after();
        const int sh = sc.gshift[g];
#pragma unroll 1
        for (int c = 0; c < BN / 32; ++c) {
            uint32_t v[32];
            tc::tmem_ld_32x32b_x32(tmem + ((uint32_t)(quad * 32) << 16) + buf * BN + c * 32, v);
            // the partial sums of this chunk are requested all at once, and kept
            // at the back of the L2 eviction order: between two drains of a tile
            // they must survive the operand tiles streaming through L2
            ulonglong2 w[32];
            ulonglong2* wp = W + (c * 32) * BM + row;
            if (g > 0) {
#pragma unroll
                for (int j = 0; j < 32; ++j) w[j] = tc::ld_u128_hint(wp + j * BM, pol_keep);
            }
            tc::tmem_ld_wait();
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const int col = c * 32 + j;
                const int x = __float2int_rn(__uint_as_float(v[j]));
                unsigned long long lo = 0, hi = 0;
                if (g > 0) {
                    lo = w[j].x;
                    hi = w[j].y;
                }
                add_shifted(lo, hi, x, sh);
                if (g < last) {
                    tc::st_u128_hint(wp + j * BM, make_ulonglong2(lo, hi), pol_keep);
                } else {
                    int64_t gj = (int64_t)nb * BN + col;
                    int part = 0;
                    if (gj >= p.n_split) {
                        gj -= p.n_split;
                        part = 1;
                    }
                    if (gi < p.m && gj < p.n) {
                        double r = i128_to_double(lo, hi, Ei + p.expB[gj] - p.L);
                        double* cp = p.C + (gi + gj * p.ldc) * p.cs + part;
                        // C = fl(fl(alpha*r) + fl(beta*C)), no contraction
                        if (!p.alpha_one) r = __dmul_rn(p.alpha, r);
                        if (!p.beta_zero) r = __dadd_rn(r, __dmul_rn(p.beta, *cp));
                        tc::st_f64_hint(cp, r, pol_stream);
                    }
                }
            }
        }
        tc::tc_fence_before();
        release(buf);
    }
    return true;
}

// Host helpers defined in ozaki.cu.
// Row exponents (1 + floor(log2 max |x|)) and spread statistics of a
// (rows x k) operand; kcontig: element (r, l) at X[l + r*ld], else at
// X[r + l*ld]; es = 2 for complex operands (ld in complex elements).  `part`
// holds the partial states of the row-contiguous form.
int scale_operand(bool kcontig, const double* X, int64_t ld, int64_t rows, int64_t k, int* exps, DeviceBuffer& part,
                  Stats* st_dev, int which, cudaStream_t st, int es);
int num_sms();
// Fraction bits of the operands' fixed-point form that reach ~1e-15 relative
// accuracy for this exponent spread and depth (calibrated on u*2^e inputs).
double required_fraction_bits(double spread_bits, int64_t k);
int choose_slices(double spread_bits, int64_t k);
int build_schedule(int S, int64_t k, int64_t k_pad, int a_rows_pad, int b_rows_pad, Schedule* sc, int* L);

}  // namespace oz
}  // namespace cgb
