// Shared code of the Chinese-remainder (Ozaki scheme II) FP64 GEMMs: single
// problems in ozaki2.cu, grouped batches in ozaki2_grouped.cu.  The moduli,
// the residue split of scaled integers, the CRT constants and the exact
// reconstruction with one rounding to FP64.
#pragma once

#include "common.cuh"
#include "ozaki_common.cuh"
#include "runtime.hpp"

#include <cstdint>

namespace cgb {
namespace oz2 {

constexpr int MAX_MODULI = 28;
// Pairwise coprime, largest first: 255 = 3*5*17, 254 = 2*127, 253 = 11*23,
// 247 = 13*19, the rest primes.
constexpr uint32_t kModuli[MAX_MODULI] = {255, 254, 253, 251, 247, 241, 239, 233, 229, 227, 223, 211, 199, 197,
                                          193, 191, 181, 179, 173, 167, 163, 157, 151, 149, 139, 137, 131, 113};
constexpr int LIMBS = 8;  // 32-bit limbs of the reconstruction (M < 2^214, sums < 2^227)

// ------------------------------------------------------------ modular helpers
// u mod p for u < 2^32, magic = floor(2^32 / p): the quotient estimate
// umulhi(u, magic) is floor(u/p) or one less, so one correction suffices.
__device__ __forceinline__ uint32_t mod32(uint32_t u, uint32_t p, uint32_t magic) {
    const uint32_t q = __umulhi(u, magic);
    const uint32_t r = u - q * p;
    return r >= p ? r - p : r;
}

constexpr int LIMB13 = 9;  // 13-bit limbs of a scaled integer (P <= 116: at most 117 bits)

struct SplitParams {
    int nmod;
    int P;      // fraction bits
    int limbs;  // 13-bit limbs the scaled integers need: ceil((P + 1) / 13)
    uint32_t p[MAX_MODULI], magic[MAX_MODULI], h[MAX_MODULI];  // magic = ceil(2^32 / p), h = floor(p / 2)
    float bias[MAX_MODULI];                                      // -(2^23 + h)
    uint32_t c13[MAX_MODULI][LIMB13];                            // 2^(13 i) mod p
};

// The scaled integer X = round_half_away(|x| 2^(P - E)) of one operand
// element as 13-bit limbs (X < 2^(P+1)), with its sign as an FP32 sign bit
// (0x80000000 for negative x).  |x| = M 2^eu with the 53-bit significand M;
// X = M 2^sh exactly when sh >= 0.  NARROW: P <= 63, so that X < 2^P fits
// one 64-bit word (|x| < 2^E) and the limbs are fixed shifts of it; else X
// is formed as a 128-bit integer.
struct Scaled {
    uint32_t d[LIMB13];
    uint32_t sgn;
};

template <bool NARROW = false>
__device__ __forceinline__ Scaled scaled_integer(double x, int E, int P) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    Scaled v;
    v.sgn = (uint32_t)(b >> 32) & 0x80000000u;
    const int ef = (int)((b >> 52) & 0x7FF);
    unsigned long long M = b & 0xFFFFFFFFFFFFFull;
    int eu;
    if (ef == 0) eu = -1074; else { M |= 1ull << 52; eu = ef - 1075; }
    int sh = eu - E + P;  // < P: |x| < 2^E
    if (M == 0) sh = 0;
    if (sh < 0) {  // round half away from zero
        const int r = -sh;
        M = r > 63 ? 0ull : (M + (1ull << (r - 1))) >> r;
        sh = 0;
    }
    if constexpr (NARROW) {  // M << sh < 2^P <= 2^63 (sh <= 62 when M != 0)
        const unsigned long long X = M << sh;
#pragma unroll
        for (int i = 0; i < LIMB13; ++i) v.d[i] = 13 * i < 64 ? (uint32_t)(X >> (13 * i)) & 0x1FFFu : 0u;
        return v;
    }
    // X = M << sh as a 128-bit integer (hi:lo), then cut into 13-bit limbs
    unsigned long long lo, hi;
    if (sh == 0) { lo = M; hi = 0; }
    else if (sh < 64) { lo = M << sh; hi = M >> (64 - sh); }
    else { lo = 0; hi = M << (sh - 64); }
#pragma unroll
    for (int i = 0; i < LIMB13; ++i) {
        const int pos = 13 * i;
        unsigned long long w;
        if (pos + 13 <= 64) w = lo >> pos;
        else if (pos >= 64) w = hi >> (pos - 64);
        else w = (lo >> pos) | (hi << (64 - pos));
        v.d[i] = (uint32_t)w & 0x1FFFu;
    }
    return v;
}

// FP32 bits of the balanced residue of the magnitude X modulo p,
// b = ((X + h) mod p) - h in [-h, p - 1 - h] (|b| <= 127); the residue of the
// signed integer is -b for negative x (the caller flips the sign bit).
// u = X_0 + h + sum_i X_i (2^(13 i) mod p) stays below 2^24 (NL <= 9), where
// umulhi(u, ceil(2^32 / p)) is exactly floor(u / p) for every modulus here
// (checked exhaustively), so r = u - q p needs no correction.  The value is
// then formed on the FP32 pipe: 2^23 + r has the bits 0x4B000000 | r, and
// 2^23 + r - 2^23 - h is exact.  Its upper 16 bits are its BF16 encoding
// (exact: at most 8 significant bits).
template <int NL>
__device__ __forceinline__ uint32_t residue_bits(const Scaled& v, uint32_t p, uint32_t magic, uint32_t h, float bias,
                                                 const uint32_t* c13) {
    uint32_t u = v.d[0] + h;
#pragma unroll
    for (int i = 1; i < NL; ++i) u += v.d[i] * c13[i];
    const uint32_t r = u - __umulhi(u, magic) * p;
    return __float_as_uint(__uint_as_float(0x4B000000u | r) + bias);
}

// Two FP32 residues packed as two BF16 values (upper halves), low one first.
__device__ __forceinline__ uint32_t pack_bf16(uint32_t lo, uint32_t hi) { return __byte_perm(lo, hi, 0x7632); }

// The sign bits of a packed BF16 pair of residues of (lo, hi): XOR-ed into
// the pair, they give the residues of the signed integers.
__device__ __forceinline__ uint32_t pair_signs(const Scaled& lo, const Scaled& hi) { return (lo.sgn >> 16) | hi.sgn; }

// Residues of one block of 32 rows x 64 K elements of a real (rows x k)
// operand into N BF16 matrices [t][rows_pad][k_pad], zero padded; 256
// threads, each 8 consecutive K elements of one row (one 16-byte store per
// modulus).  A warp covers 4 rows x 64 K elements: its stores are four
// 128-byte row segments per modulus, its loads (either layout) whole 32-byte
// sectors; a K-contiguous row segment that is 16-byte aligned is read as four
// 16-byte loads.  kcontig: element (r, l) at X[l + r*ld], else at
// X[r + l*ld].  NL: 13-bit limbs of the scaled integers (P < 13 NL).
// NARROW: P <= 63 (scaled_integer).  keep_k_pad: the K padding [k, k_pad)
// already holds zero residues (an arena zeroed once and never written there),
// so threads wholly inside it return at once.  Measured at 16384^2 with 16 moduli
// (P = 55): 3.11 ms for the M-contiguous layout and 2.47 ms for the
// K-contiguous one, against 3.28 and 2.73 ms with the 128-bit form, scalar
// loads and the modulus loop not unrolled.
template <bool KCONTIG, int NL, bool NARROW = false>
__device__ __forceinline__ void split_block(const double* __restrict__ X, int64_t ld, int64_t rows, int64_t k,
                                            const int* __restrict__ exps, int64_t k_pad, int64_t rows_pad,
                                            uint16_t* __restrict__ out, const SplitParams& sp, int P, int64_t bx,
                                            int64_t by, bool keep_k_pad = false) {
    const int t = threadIdx.x;
    const int64_t r = bx * 32 + t / 8;
    const int64_t l0 = by * 64 + (t % 8) * 8;
    if (r >= rows_pad || l0 >= (keep_k_pad ? k : k_pad)) return;
    const int E = r < rows ? exps[r] : 0;
    Scaled v[8];
    const double* seg = X + (KCONTIG ? l0 + r * ld : r + l0 * ld);
    if (KCONTIG && r < rows && l0 + 8 <= k && (reinterpret_cast<uintptr_t>(seg) & 15) == 0) {
        const double2* s2 = reinterpret_cast<const double2*>(seg);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const double2 q = s2[e];
            v[2 * e] = scaled_integer<NARROW>(q.x, E, P);
            v[2 * e + 1] = scaled_integer<NARROW>(q.y, E, P);
        }
    } else {
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int64_t l = l0 + e;
            double x = 0.0;
            if (r < rows && l < k) x = KCONTIG ? X[l + r * ld] : X[r + l * ld];
            v[e] = scaled_integer<NARROW>(x, E, P);
        }
    }
    uint16_t* o = out + r * k_pad + l0;
    const int64_t slab = rows_pad * k_pad;
    uint32_t sg[4];
#pragma unroll
    for (int e = 0; e < 8; e += 2) sg[e / 2] = pair_signs(v[e], v[e + 1]);
    auto modulus = [&](int m) {
        const uint32_t p = sp.p[m], mg = sp.magic[m], h = sp.h[m];
        const float bias = sp.bias[m];
        uint32_t w[4];
#pragma unroll
        for (int e = 0; e < 8; e += 2)
            w[e / 2] = pack_bf16(residue_bits<NL>(v[e], p, mg, h, bias, sp.c13[m]),
                                 residue_bits<NL>(v[e + 1], p, mg, h, bias, sp.c13[m])) ^ sg[e / 2];
        *reinterpret_cast<uint4*>(o + m * slab) = make_uint4(w[0], w[1], w[2], w[3]);
    };
    if constexpr (KCONTIG) {
#pragma unroll 1
        for (int m = 0; m < sp.nmod; ++m) modulus(m);
    } else {  // two moduli per trip: 5 % faster here, 6 % slower for the K-contiguous layout
#pragma unroll 2
        for (int m = 0; m < sp.nmod; ++m) modulus(m);
    }
}

// ------------------------------------------------------------- reconstruction
// CRT constants of the first nmod moduli.
struct CrtConst {
    int nmod;
    uint32_t w[MAX_MODULI][LIMBS];  // CRT weights w_t = (M/p_t) * ((M/p_t)^-1 mod p_t)
    uint32_t w16[MAX_MODULI][2 * LIMBS];  // the same in 16-bit pieces, lowest first
    uint32_t M[LIMBS];
    float inv_m2;                   // 2^(32 (L-2)) / M for the quotient estimate (L = limbs_for(nmod))
};

// Round-to-nearest-even conversion of the unsigned 128-bit integer (hi:lo)
// times 2^e2 to the bits of a double (subnormal and overflow results
// included), formed with integer operations only.
__device__ __forceinline__ unsigned long long u128_to_bits(unsigned long long lo, unsigned long long hi, int e2) {
    if (hi == 0 && lo == 0) return 0ull;
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
        unsigned long long q, g, st;  // kept bits, guard bit, sticky bits
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
    const bool normal = e_lsb > -1074 || mant >= (1ull << 52);
    if (mant >= (1ull << 53)) {  // rounding carried into a new bit
        mant >>= 1;
        ++e_lsb;
    }
    unsigned long long bits;
    if (normal && mant >= (1ull << 52)) {
        const int be = e_lsb + 52 + 1023;
        bits = be >= 2047 ? 0x7FF0000000000000ull : (((unsigned long long)be << 52) | (mant & 0xFFFFFFFFFFFFFull));
    } else {
        bits = mant;  // subnormal (or the smallest normal reached by rounding)
    }
    return bits;
}

// |x| (L limbs) * 2^e2 rounded once to FP64, negated if neg: the top four
// limbs from the highest nonzero one, the limbs below folded into a sticky
// last bit (below the rounding position: the window keeps 97+ bits).
template <int L>
__device__ __forceinline__ double limbs_to_double(const uint32_t (&x)[L], bool neg, int e2) {
    int tl = -1;
#pragma unroll
    for (int l = 0; l < L; ++l)
        if (x[l]) tl = l;
    if (tl < 0) return 0.0;
    uint32_t w3 = 0, w2 = 0, w1 = 0, w0 = 0, sticky = 0;
#pragma unroll
    for (int l = 0; l < L; ++l) {
        const uint32_t v = x[l];
        if (l == tl) w3 = v;
        else if (l == tl - 1) w2 = v;
        else if (l == tl - 2) w1 = v;
        else if (l == tl - 3) w0 = v;
        else if (l < tl - 3) sticky |= v;
    }
    const unsigned long long hi = ((unsigned long long)w3 << 32) | w2;
    const unsigned long long lo = ((unsigned long long)w1 << 32) | w0 | (sticky ? 1ull : 0ull);
    const unsigned long long bits = u128_to_bits(lo, hi, e2 + 32 * (tl - 3));
    return __longlong_as_double((long long)(bits | ((unsigned long long)neg << 63)));  // sign by bit, no FP64 op
}

// x = m << s as limbs (m < 2^53, s + 53 <= 32 L).
template <int L>
__device__ __forceinline__ void set_shifted(uint32_t (&x)[L], unsigned long long m, int s) {
#pragma unroll
    for (int l = 0; l < L; ++l) {
        const int pos = s - 32 * l;  // where bit 0 of m lands relative to limb l
        uint32_t v = 0;
        if (pos >= 0 && pos < 32) v = (uint32_t)(m << pos);
        else if (pos < 0 && pos > -64) v = (uint32_t)(m >> -pos);
        x[l] = v;
    }
}

template <int L>
__device__ __forceinline__ void negate_limbs(uint32_t (&x)[L]) {
    unsigned long long c = 1;
#pragma unroll
    for (int l = 0; l < L; ++l) {
        c += (uint32_t)~x[l];
        x[l] = (uint32_t)c;
        c >>= 32;
    }
}

// x -= y (two's complement over L limbs).
template <int L>
__device__ __forceinline__ void sub_limbs(uint32_t (&x)[L], const uint32_t (&y)[L]) {
    unsigned long long br = 0;
#pragma unroll
    for (int l = 0; l < L; ++l) {
        const unsigned long long d = (unsigned long long)x[l] - y[l] - br;
        x[l] = (uint32_t)d;
        br = (d >> 63) & 1ull;
    }
}

// V from X = sum_t r_t w_t (L 64-bit partial limbs): carries, then one
// subtraction of q M with q = rint(X / M) estimated in FP32 from the top three
// limbs (error < 0.003).  |V| <= M/4 (the modulus count is chosen so), so
// X - q M lies in (-0.51 M, 0.51 M) and is V itself, as an L-limb two's
// complement number.  Returns |V| in x and its sign.
template <int L>
__device__ __forceinline__ bool reduce_crt(const unsigned long long (&acc)[L], uint32_t (&x)[L], const CrtConst& p) {
    unsigned long long c = 0;
#pragma unroll
    for (int l = 0; l < L; ++l) {
        c += acc[l];
        x[l] = (uint32_t)c;
        c >>= 32;
    }
    const float xs = __uint2float_rn(x[L - 1]) * 4294967296.0f + __uint2float_rn(x[L - 2]) +
                     __uint2float_rn(x[L - 3]) * 2.3283064365386963e-10f;
    const uint32_t q = __float2uint_rn(xs * p.inv_m2);
    unsigned long long br = 0, cm = 0;
#pragma unroll
    for (int l = 0; l < L; ++l) {  // x -= q * M
        cm += (unsigned long long)q * p.M[l];
        const unsigned long long d = (unsigned long long)x[l] - (uint32_t)cm - br;
        x[l] = (uint32_t)d;
        br = (d >> 63) & 1ull;
        cm >>= 32;
    }
    const bool neg = (x[L - 1] >> 31) != 0;
    if (neg) negate_limbs<L>(x);
    return neg;
}

// X_c = sum_t r_{t,c} w_t (L 64-bit partial limbs) for the four residue bytes
// c of the words rp[t * stride], t < nmod.  The sums run over the weights'
// 16-bit pieces in 32-bit registers (at most 28 * 255 * 65535 < 2^29 each),
// one integer multiply-add per piece, instead of 64-bit products and sums;
// the pieces are folded into 64-bit partial limbs at the end.  The words of
// eight moduli are loaded before their products are summed, so that eight
// loads are in flight per thread.
template <int L>
__device__ __forceinline__ void crt_accumulate(const uint32_t* __restrict__ rp, int64_t stride, int nmod,
                                               const CrtConst& crt, unsigned long long (&acc)[4][L]) {
    uint32_t a[4][2 * L];
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
        for (int q = 0; q < 2 * L; ++q) a[c][q] = 0;
#pragma unroll 1
    for (int t0 = 0; t0 < nmod; t0 += 8) {
        uint32_t rr[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) rr[u] = t0 + u < nmod ? __ldg(rp + (int64_t)(t0 + u) * stride) : 0u;
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            if (t0 + u >= nmod) break;
            const int t = t0 + u;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const uint32_t r = (rr[u] >> (8 * c)) & 0xFFu;
#pragma unroll
                for (int q = 0; q < 2 * L; ++q) a[c][q] += r * crt.w16[t][q];
            }
        }
    }
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
        for (int l = 0; l < L; ++l)
            acc[c][l] = (unsigned long long)a[c][2 * l] + ((unsigned long long)a[c][2 * l + 1] << 16);
}

// ---------------------------------------------------------------- host side
// (ozaki2.cu)
void fill_split(SplitParams& sp, int nmod, int P);
void fill_crt(CrtConst& c, int nmod);
// Limbs the reconstruction needs: sum_t r_t w_t < nmod * 255 * M < 2^(bitlen(M) + 13).
int limbs_for(int nmod);
// Largest P with M >= 2^(2P + ceil(log2 k) + 2), i.e. M > 4 k 2^(2P) > 2 max|V|.
int max_fraction_bits(int nmod, int64_t k);
// The fewest moduli whose product admits `want` fraction bits at depth k
// (MAX_MODULI + 1 when none does).
int fewest_moduli(int want, int64_t k);
// Fraction bits added to the accuracy rule (COSMA_GPU_OZAKI2_EXTRA_BITS, default 16).
int extra_fraction_bits();

}  // namespace oz2
}  // namespace cgb
