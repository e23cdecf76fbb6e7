// FP64-accurate GEMM by the Chinese-remainder form of the Ozaki scheme
// ("Ozaki scheme II", Ozaki, Uchino & Imamura 2025) on the BF16 tensor cores.
//
// The reference runs a native DGEMM (cuBLAS through Tiled-MM); this is a
// precision form of the same operation, C = alpha*op(A)*op(B) + beta*C, next
// to the digit-slice form of ozaki.cu.  It needs one GEMM per modulus where
// the slice form needs S(S+1)/2 slice products, which is what makes it the
// faster of the two at FP64 accuracy.
//
// Method:
//  1. Row scaling (shared with the slice form): row i of op(A) gets the
//     exponent E_i = 1 + floor(log2 max_l |a_il|), column j of op(B) F_j.
//  2. Integers.  a'_il = sign(a) round_half_away(|a_il| 2^(P - E_i)), an
//     integer of at most P bits; b'_lj likewise.  P is the fraction width,
//     chosen from the requested accuracy and the exponent spread.
//  3. Residues.  For N pairwise coprime moduli p_t <= 255 (product M >
//     4 k 2^(2P)), the balanced residues of a' and b' modulo p_t lie in
//     [-127, 127] and are exact in BF16; they are written as N BF16 matrices
//     per operand, K-major.
//  4. Modular GEMMs.  For each t, A_t * B_t runs on the BF16 tensor cores
//     (tcgen05 kind::f16, CTA pairs, TMA).  One TMEM accumulation spans a
//     1024-wide K chunk: 1024 products of magnitude <= 127^2 sum below 2^24,
//     so the FP32 accumulator is exact.  The epilogue adds each chunk, as an
//     integer, into 32-bit running sums in registers and finally reduces them
//     modulo p_t: one residue byte per output and modulus.
//  5. Reconstruction.  V_ij = sum_t r_t w_t mod M (w_t the CRT weights), taken
//     in (-M/2, M/2), is exactly sum_l a'_il b'_lj; it is rounded once to FP64
//     with the scale 2^(E_i + F_j - 2P) (round to nearest even), then alpha
//     and beta are applied.  The integer arithmetic is 32-bit limbs; no FP64
//     arithmetic is used before the final conversion.
//
// The integer tensor op (tcgen05 kind::i8) does not exist on sm_103a and FP8
// E4M3 holds integers only up to 16, too few pairwise coprime moduli for
// FP64 accuracy; BF16 holds all integers up to 256.
//
// GEMM kernel: persistent CTA pairs, 256 x 256 output tiles (M = 256 over the
// pair), 64-element (128-byte) BF16 K blocks through a 4-stage TMA ring with
// 128-byte swizzle, two 256-column FP32 accumulators in TMEM so that the
// drain of one K chunk overlaps the MMAs of the next.  Work units are
// (modulus, tile) pairs, modulus-major: at any time the wave of CTAs runs
// one ordinary BF16 GEMM, whose operand panels it shares through L2.
//   warp 0      TMA producer         warp 1   TMEM owner + MMA issuer
//   warps 2..9  epilogue (TMEM -> registers -> 32-bit running sums)
#include "common.cuh"
#include "runtime.hpp"
#include "ozaki_common.cuh"
#include "ozaki2_common.cuh"
#include "tc_common.cuh"
#include "tma_host.hpp"
#include "pipeline.hpp"

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <condition_variable>
#include <deque>
#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <chrono>
#include <vector>

namespace cgb {
namespace oz2 {

using oz::Stats;


constexpr int BM = 128, BN = 256, BKE = 64;  // BKE: BF16 elements per K block (128 bytes)
constexpr int KB_PER_CHUNK = 16;             // 1024-element K chunk per exact TMEM accumulation
constexpr int CHUNKS_PER_REDUCE = 64;        // running sums reduced mod p after this many chunks
constexpr int STAGES = 4;
constexpr int A_STAGE = BM * 128, B_STAGE = (BN / 2) * 128, STAGE = A_STAGE + B_STAGE;  // per CTA
constexpr int EPI_WARPS = 8;
constexpr int THREADS = 64 + 32 * EPI_WARPS;
constexpr int SMEM_BYTES = STAGES * STAGE + 1024 + 256;
static_assert(SMEM_BYTES <= 232448, "shared memory");
constexpr int kStripPairs = 8;  // tile order: strips of 8 pair rows (2048 rows), see oz::tile_coords
constexpr int64_t KMAX = 64 * 65535;  // K of one exact pass: the split grids' K extent


// Residue matrices of a real (rows x k) operand: N BF16 matrices [t][rows_pad][k_pad]
// (split_block), one block per 32 rows x 64 K elements.
template <bool KCONTIG, int NL, bool NARROW>
__global__ void __launch_bounds__(256) split_kernel(const double* __restrict__ X, int64_t ld, int64_t rows,
                                                    int64_t k, const int* __restrict__ exps, int64_t k_pad,
                                                    int64_t rows_pad, uint16_t* __restrict__ out,
                                                    const __grid_constant__ SplitParams sp) {
    split_block<KCONTIG, NL, NARROW>(X, ld, rows, k, exps, k_pad, rows_pad, out, sp, sp.P, blockIdx.x, blockIdx.y);
}

// Complex operands, laid out like the slice form's complex split: one real
// GEMM of depth 2*kh gives both parts of C,
//   A_cat row r                 [ Re a | sa*Im a ]
//   B_cat row r                 [ Re b | -sb*Im b ]   -> Re C column r
//   B_cat row rows_pad + r      [ sb*Im b | Re b ]    -> Im C column r
// (sa, sb = -1 for a conjugated operand).  A negated residue is the residue
// of the negated integer, so the signs are applied to the residues.  kh is k
// padded to 64; the row pitch is 2*kh; modulus t starts at t * slice_rows *
// 2*kh.  X holds interleaved complex doubles, ld in complex elements.
template <bool KCONTIG, bool BSIDE, int NL>
__global__ void __launch_bounds__(256) split_cplx_kernel(const double2* __restrict__ X, int64_t ld, int64_t rows,
                                                         int64_t k, const int* __restrict__ exps, int64_t kh,
                                                         int64_t rows_pad, int64_t slice_rows, int conj,
                                                         uint16_t* __restrict__ out,
                                                         const __grid_constant__ SplitParams sp) {
    const int t = threadIdx.x;  // a warp covers 4 rows x 64 K elements (see split_kernel)
    const int64_t r = (int64_t)blockIdx.x * 32 + t / 8;
    const int64_t l0 = (int64_t)blockIdx.y * 64 + (t % 8) * 8;
    if (r >= rows_pad || l0 >= kh) return;
    const int E = r < rows ? exps[r] : 0;
    const int64_t pitch = 2 * kh, slab = slice_rows * pitch;
    const double* Xd = reinterpret_cast<const double*>(X);
#pragma unroll 1
    for (int part = 0; part < 2; ++part) {
        Scaled v[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int64_t l = l0 + e;
            double x = 0.0;
            if (r < rows && l < k) x = Xd[2 * (KCONTIG ? l + r * ld : r + l * ld) + part];
            v[e] = scaled_integer<false>(x, E, sp.P);
            if (part && conj) v[e].sgn ^= 0x80000000u;  // the conjugated imaginary part
        }
#pragma unroll 1
        for (int m = 0; m < sp.nmod; ++m) {
            const uint32_t p = sp.p[m], mg = sp.magic[m], h = sp.h[m];
            const float bias = sp.bias[m];
            uint32_t w[4], nw[4];
#pragma unroll
            for (int e = 0; e < 8; e += 2) {
                w[e / 2] = pack_bf16(residue_bits<NL>(v[e], p, mg, h, bias, sp.c13[m]),
                                     residue_bits<NL>(v[e + 1], p, mg, h, bias, sp.c13[m])) ^
                           pair_signs(v[e], v[e + 1]);
                nw[e / 2] = w[e / 2] ^ 0x80008000u;  // the negated pair: both sign bits flipped
            }
            uint16_t* base = out + m * slab;
            const uint4 val = make_uint4(w[0], w[1], w[2], w[3]);
            if (!BSIDE) {
                *reinterpret_cast<uint4*>(base + r * pitch + part * kh + l0) = val;
            } else if (part == 0) {  // Re b: first half of row r, second half of row rows_pad + r
                *reinterpret_cast<uint4*>(base + r * pitch + l0) = val;
                *reinterpret_cast<uint4*>(base + (rows_pad + r) * pitch + kh + l0) = val;
            } else {  // Im b: negated in row r, as is in row rows_pad + r
                *reinterpret_cast<uint4*>(base + r * pitch + kh + l0) = make_uint4(nw[0], nw[1], nw[2], nw[3]);
                *reinterpret_cast<uint4*>(base + (rows_pad + r) * pitch + l0) = val;
            }
        }
    }
}

// ------------------------------------------------------------------ GEMM
struct GemmParams {
    int num_m_tiles, num_n_tiles, num_tiles;  // 128-row / 256-column tiles; num_tiles counts 256 x 256
    int nmod, kb_count;
    int a_rows_pad, b_rows_pad;  // rows of one modulus' residue matrix
    int64_t m_pad, nb16;         // residue output: [t][n_pad / 16][m_pad][16] bytes
    uint8_t* R;
    uint32_t p[MAX_MODULI], magic[MAX_MODULI], bias[MAX_MODULI];  // bias: a multiple of p >= 2^30
    unsigned* err;
};

// Reduces the 32 running sums of one column group to residues in [0, p).
__device__ __forceinline__ void reduce_sums(int (&s)[32], uint32_t p, uint32_t magic, uint32_t bias) {
#pragma unroll
    for (int j = 0; j < 32; ++j) s[j] = (int)mod32((uint32_t)s[j] + bias, p, magic);  // s + bias in [0, 2^32)
}

__global__ void __launch_bounds__(THREADS, 1)
    gemm_pair_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                     const __grid_constant__ GemmParams p) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* full = (uint64_t*)(smem + STAGES * STAGE);
    uint64_t* empty = full + STAGES;
    uint64_t* accf = empty + STAGES;
    uint64_t* acce = accf + 2;
    uint64_t* drain = acce + 2;
    uint32_t* tmem_slot = (uint32_t*)(drain + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rank = (int)tc::cluster_ctarank();
    const bool leader = rank == 0;
    const int pair = blockIdx.x / 2, npairs = gridDim.x / 2;
    const int num_pm = p.num_m_tiles / 2;  // 256-row tiles
    const int units = p.nmod * p.num_tiles;
    const int nchunks = (p.kb_count + KB_PER_CHUNK - 1) / KB_PER_CHUNK;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            tc::mbar_init(&full[s], 1);   // the even CTA's expect_tx (bytes of both CTAs)
            tc::mbar_init(&empty[s], 1);  // one MMA commit per use
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&accf[b], 1);
            tc::mbar_init(&acce[b], 2 * EPI_WARPS);  // every epilogue warp of both CTAs
        }
        tc::mbar_init(drain, 1);
        tc::fence_mbar_init();
        tc::prefetch_tmap(&tmA);
        tc::prefetch_tmap(&tmB);
    }
    if (warp == 1) tc::tmem_alloc_pair(tmem_slot, 512);
    __syncthreads();
    tc::cluster_sync();  // the peer's loads and commits reach this CTA's barriers
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {  // ---------------------------------- TMA producer (both CTAs)
            const uint32_t full0 = tc::mapa_shared(full, 0);
            uint32_t it = 0;
            bool ok = true;
            for (int u = pair; u < units && ok; u += npairs) {
                const int t = u / p.num_tiles, tile = u - t * p.num_tiles;
                int mbp, nb;
                oz::tile_coords(tile, num_pm, p.num_n_tiles, mbp, nb, kStripPairs);
                const int arow = t * p.a_rows_pad + (2 * mbp + rank) * BM;
                const int brow = t * p.b_rows_pad + nb * BN + rank * (BN / 2);
                for (int kb = 0; kb < p.kb_count; ++kb, ++it) {
                    const int st = it % STAGES;
                    if (!tc::mbar_wait(&empty[st], ((it / STAGES) & 1) ^ 1, p.err, kDevTimeoutEmpty)) {
                        ok = false;
                        break;
                    }
                    if (leader) tc::mbar_arrive_expect_tx(&full[st], 2 * STAGE);
                    uint8_t* sa = smem + st * STAGE;
                    tc::tma_load_2d_pair(sa, &tmA, kb * BKE, arow, full0 + st * 8);
                    tc::tma_load_2d_pair(sa + A_STAGE, &tmB, kb * BKE, brow, full0 + st * 8);
                }
            }
            if (leader) {  // nothing may still be in flight into either CTA when it exits
                const uint32_t first = it > STAGES ? it - STAGES : 0;
                for (uint32_t j = first; j < it; ++j) tc::mbar_wait_drain(&full[j % STAGES], (j / STAGES) & 1);
            }
        }
    } else if (warp == 1) {
        if (lane == 0 && leader) {  // ------------------------ MMA issuer (even CTA)
            constexpr uint32_t ID = tc::idesc(tc::kFmtBF16, tc::kFmtBF16, 2 * BM, BN);
            uint32_t it = 0, acc_it = 0;
            bool ok = true;
            for (int u = pair; u < units && ok; u += npairs) {
                for (int c = 0; c < nchunks && ok; ++c, ++acc_it) {
                    const uint32_t buf = acc_it & 1;
                    if (!tc::mbar_wait_cluster(&acce[buf], ((acc_it >> 1) & 1) ^ 1, p.err, kDevTimeoutAccEmpty)) {
                        ok = false;
                        break;
                    }
                    tc::tc_fence_after();
                    const uint32_t d_tmem = tmem + buf * BN;
                    uint32_t accumulate = 0;
                    const int kb1 = min(p.kb_count, (c + 1) * KB_PER_CHUNK);
                    for (int kb = c * KB_PER_CHUNK; kb < kb1; ++kb, ++it) {
                        const int st = it % STAGES;
                        if (!tc::mbar_wait(&full[st], (it / STAGES) & 1, p.err, kDevTimeoutFull)) {
                            ok = false;
                            break;
                        }
                        tc::tc_fence_after();
                        const uint32_t sa = tc::smem_u32(smem + st * STAGE);
                        const uint64_t ad = tc::sdesc_k_sw128(sa), bd = tc::sdesc_k_sw128(sa + A_STAGE);
#pragma unroll
                        for (int kk = 0; kk < BKE / 16; ++kk) {  // K = 16 per MMA: 32 bytes
                            tc::mma_pair_f16(d_tmem, ad + 2 * kk, bd + 2 * kk, ID, accumulate);
                            accumulate = 1;
                        }
                        tc::mma_pair_commit_multicast(&empty[st], 3);
                    }
                    if (ok) tc::mma_pair_commit_multicast(&accf[buf], 3);
                }
            }
            tc::mma_pair_commit_multicast(drain, 1);  // every MMA complete before TMEM is released
            tc::mbar_wait_drain(drain, 0);
        }
    } else {  // ------------------------------------------------ epilogue (both CTAs)
        const int quad = warp & 3;             // TMEM lanes this warp may access
        const int half = (warp - 2) >> 2;      // columns [half*128, half*128 + 128) of the tile
        const int row = quad * 32 + lane;
        const uint32_t acce0 = tc::mapa_shared(acce, 0);
        uint32_t acc_it = 0;
        bool ok = true;
        for (int u = pair; u < units && ok; u += npairs) {
            const int t = u / p.num_tiles, tile = u - t * p.num_tiles;
            int mbp, nb;
            oz::tile_coords(tile, num_pm, p.num_n_tiles, mbp, nb, kStripPairs);
            const int mb = 2 * mbp + rank;
            const uint32_t pm = p.p[t], mg = p.magic[t], bias = p.bias[t];
            int s[4][32];
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int j = 0; j < 32; ++j) s[q][j] = 0;
            for (int c = 0; c < nchunks; ++c, ++acc_it) {
                const uint32_t buf = acc_it & 1;
                // all lanes must agree before the warp-collective TMEM loads
                if (!__all_sync(0xffffffffu, tc::mbar_wait(&accf[buf], (acc_it >> 1) & 1, p.err, kDevTimeoutAcc))) {
                    ok = false;
                    break;
                }
                tc::tc_fence_after();
                const uint32_t base = tmem + ((uint32_t)(quad * 32) << 16) + buf * BN + half * 128;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    uint32_t v[32];
                    tc::tmem_ld_32x32b_x32(base + q * 32, v);
                    tc::tmem_ld_wait();
#pragma unroll
                    for (int j = 0; j < 32; ++j) s[q][j] += __float2int_rn(__uint_as_float(v[j]));
                }
                tc::tc_fence_before();
                __syncwarp();
                if (lane == 0) tc::mbar_arrive_cluster(acce0 + buf * 8);
                if ((c + 1) % CHUNKS_PER_REDUCE == 0) {  // keep |s| below 2^30 for any K
#pragma unroll
                    for (int q = 0; q < 4; ++q) reduce_sums(s[q], pm, mg, bias);
                }
            }
            if (!ok) break;
            // residues of the 128 columns of this thread's row: 8 groups of 16
            const int64_t i = (int64_t)mb * BM + row;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                reduce_sums(s[q], pm, mg, bias);
#pragma unroll
                for (int g = 0; g < 2; ++g) {
                    uint32_t w[4];
#pragma unroll
                    for (int b = 0; b < 4; ++b) {
                        const int j0 = g * 16 + b * 4;
                        w[b] = (uint32_t)s[q][j0] | ((uint32_t)s[q][j0 + 1] << 8) | ((uint32_t)s[q][j0 + 2] << 16) |
                               ((uint32_t)s[q][j0 + 3] << 24);
                    }
                    const int64_t jb = (int64_t)nb * (BN / 16) + half * 8 + q * 2 + g;
                    *reinterpret_cast<uint4*>(p.R + (((int64_t)t * p.nb16 + jb) * p.m_pad + i) * 16) =
                        make_uint4(w[0], w[1], w[2], w[3]);
                }
            }
        }
    }
    __syncthreads();
    tc::cluster_sync();  // the even CTA's MMAs read this CTA's shared memory and write its TMEM
    if (warp == 1) {
        __syncwarp();
        tc::tc_fence_after();
        tc::tmem_dealloc_pair(tmem, 512);
    }
}

// ------------------------------------------------------------- reconstruction
struct CombineParams {
    int nmod, twoP;
    CrtConst crt;
    int64_t m, n, ldc, m_pad, nb16, row_blocks;
    int64_t n_split;  // complex: GEMM columns [0, n_split) are real parts, the rest imaginary parts
    int cs;           // doubles per element of C (1 real, 2 complex)
    const uint8_t* R;
    const int* expA;
    const int* expB;
    double* C;
    double alpha, beta;
    int alpha_one, beta_zero;
    // residual mode (real only): E = V 2^e - Ct exactly rounded, Rx = V 2^e rounded
    const double* Ct;
    int64_t ldt, ldo;
    double* E;
    double* Rx;
};


// Four output elements per thread: a block of 4 warps covers 32 rows x 16
// GEMM columns (block b: row block b % row_blocks, column block b /
// row_blocks); warp g takes columns 16 cb + 4 g .. + 3, lane the row 32 rb +
// lane, and one 32-bit load gives the thread its four residues of a modulus.
// MODE: kStoreC writes the rounded product, kScaleC alpha * it + beta * C,
// kResidual the residual pair.  The store-only form is its own instantiation:
// the compiler predicates rather than branches around the alpha / beta
// arithmetic, and three predicated FP64 instructions per entry occupy
// GB300's narrow FP64 pipe.
constexpr int kStoreC = 0, kScaleC = 1, kResidual = 2;

template <int L, int MODE>
__global__ void __launch_bounds__(128) combine_kernel(const __grid_constant__ CombineParams p) {
    constexpr bool RESIDUAL = MODE == kResidual;
    const int lane = threadIdx.x & 31, g = threadIdx.x >> 5;
    const int64_t rb = (int64_t)blockIdx.x % p.row_blocks, cb = (int64_t)blockIdx.x / p.row_blocks;
    const int64_t i = rb * 32 + lane;
    if (i >= p.m) return;
    const int64_t gj0 = cb * 16 + 4 * g;  // first GEMM column of this thread
    int64_t j0 = gj0;
    int part = 0;
    if (j0 >= p.n_split) {
        j0 -= p.n_split;
        part = 1;
    }
    if (j0 >= p.n) return;
    const uint32_t* rp = reinterpret_cast<const uint32_t*>(p.R + (cb * p.m_pad + i) * 16) + g;
    const int64_t stride = p.nb16 * p.m_pad * 4;  // 32-bit words per modulus
    unsigned long long acc[4][L];
    crt_accumulate<L>(rp, stride, p.nmod, p.crt, acc);
    const int Ei = p.expA[i];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const int64_t j = j0 + c;
        if (j >= p.n) break;
        uint32_t x[L];
        const bool neg = reduce_crt<L>(acc[c], x, p.crt);
        const int e2 = Ei + p.expB[j] - p.twoP;
        double r = limbs_to_double<L>(x, neg, e2);
        if constexpr (RESIDUAL) {
            // T = Ct * 2^-e2 is an integer whenever Ct's last bit weighs at
            // least 2^e2 (always, but for a Ct below ~2^(e2 + 52)); then
            // E = (V - T) 2^e2 is exact before its one rounding.  Otherwise,
            // or when T does not fit the limbs, E is NaN.
            const double ct = p.Ct[i + j * p.ldt];
            const unsigned long long b = (unsigned long long)__double_as_longlong(ct);
            const bool cneg = (b >> 63) != 0;
            const int ef = (int)((b >> 52) & 0x7FF);
            unsigned long long mc = b & 0xFFFFFFFFFFFFFull;
            int ec;
            if (ef == 0) ec = -1074; else { mc |= 1ull << 52; ec = ef - 1075; }
            const int s = ec - e2;
            double err;
            if (ef == 0x7FF || (mc && (s < 0 || s + 53 > 32 * L - 2))) {
                err = __longlong_as_double(0x7FF8000000000000ll);
            } else {
                uint32_t t[L];
                set_shifted<L>(t, mc, mc ? s : 0);
                if (neg) negate_limbs<L>(x);   // signed V
                if (cneg) negate_limbs<L>(t);  // signed T
                sub_limbs<L>(x, t);            // D = V - T, |D| < 2^(32 L - 1)
                const bool dneg = (x[L - 1] >> 31) != 0;
                if (dneg) negate_limbs<L>(x);
                err = limbs_to_double<L>(x, dneg, e2);
            }
            p.E[i + j * p.ldo] = err;
            p.Rx[i + j * p.ldo] = r;
            continue;
        }
        double* cp = p.C + (i + j * p.ldc) * p.cs + part;
        if constexpr (MODE == kScaleC) {
            if (!p.alpha_one) r = __dmul_rn(p.alpha, r);
            if (!p.beta_zero) r = __dadd_rn(r, __dmul_rn(p.beta, *cp));
        }
        *cp = r;
    }
}

// ---------------------------------------------------------------- host side
struct Big {  // little-endian 32-bit limbs
    uint32_t w[LIMBS] = {};
    void mul_small(uint32_t x) {
        unsigned long long c = 0;
        for (int i = 0; i < LIMBS; ++i) {
            c += (unsigned long long)w[i] * x;
            w[i] = (uint32_t)c;
            c >>= 32;
        }
    }
    uint32_t mod_small(uint32_t p) const {
        unsigned long long r = 0;
        for (int i = LIMBS - 1; i >= 0; --i) r = ((r << 32) | w[i]) % p;
        return (uint32_t)r;
    }
    int bitlen() const {
        for (int i = LIMBS - 1; i >= 0; --i)
            if (w[i]) return 32 * i + 32 - __builtin_clz(w[i]);
        return 0;
    }
};

uint32_t inverse_mod(uint32_t a, uint32_t p) {  // a^-1 mod p, gcd(a, p) = 1
    long long t = 0, nt = 1, r = p, nr = a % p;
    while (nr) {
        const long long q = r / nr;
        std::swap(t, nt);
        nt -= q * t;
        std::swap(r, nr);
        nr -= q * r;
    }
    return (uint32_t)(t < 0 ? t + p : t);
}

Big modulus_product(int nmod) {
    Big M;
    M.w[0] = 1;
    for (int t = 0; t < nmod; ++t) M.mul_small(kModuli[t]);
    return M;
}

int ceil_log2(int64_t k) {
    int b = 0;
    while (((int64_t)1 << b) < k) ++b;
    return b;
}

int max_fraction_bits(int nmod, int64_t k) { return (modulus_product(nmod).bitlen() - 1 - ceil_log2(k) - 2) / 2; }

// Fraction bits the requested accuracy needs for inputs with this exponent
// spread: the width calibrated for the slice form on sampled entries
// (oz::required_fraction_bits) plus 16 bits (COSMA_GPU_OZAKI2_EXTRA_BITS).
// Checking every entry of 16384^3 products showed the sampled calibration
// short for the worst-cancelling entries: u*2^e inputs with phi = 8 had 5,499
// entries above 1e-15 relative error at P = 65 (max 4e-11), phi = 32 had
// 1,266 at P = 69 (max 8e-13); the input-rounding error falls by 2^-16 for
// 16 more bits, below the target for both.
int extra_fraction_bits() {
    static const long long extra = env_ll("COSMA_GPU_OZAKI2_EXTRA_BITS", 16);
    return (int)extra;
}

int requested_fraction_bits(double spread, int64_t k) {
    return (int)std::ceil(oz::required_fraction_bits(spread, k)) + extra_fraction_bits();
}

// Modulus count and fraction bits: the caller's count, or the fewest moduli
// that either keep every input bit (exact_bits: then the product is exact
// and C is correctly rounded) or admit the fraction bits the accuracy rule
// asks for, whichever is fewer; P is then the largest the count allows.
int fewest_moduli(int want, int64_t k) {
    for (int t = 2; t <= MAX_MODULI; ++t)
        if (max_fraction_bits(t, k) >= want) return t;
    return MAX_MODULI + 1;
}

int choose(int nmod_req, double spread, int64_t k, int* nmod, int* P, int exact_bits = 1 << 30) {
    if (nmod_req > 0) {
        *nmod = std::min(nmod_req, MAX_MODULI);
    } else {
        *nmod = std::min({fewest_moduli(requested_fraction_bits(spread, k), k),
                          fewest_moduli(std::max(exact_bits, 1), k), MAX_MODULI});
    }
    *P = std::min(max_fraction_bits(*nmod, k), 116);  // at most nine 13-bit limbs per scaled integer
    if (*P < 1) return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "ozaki2: too few moduli for this k");
    return COSMA_GPU_SUCCESS;
}

void fill_split(SplitParams& sp, int nmod, int P) {
    std::memset(&sp, 0, sizeof(sp));
    sp.nmod = nmod;
    sp.P = P;
    sp.limbs = (P + 1 + 12) / 13;
    for (int t = 0; t < nmod; ++t) {
        const uint32_t p = kModuli[t];
        sp.p[t] = p;
        sp.magic[t] = (uint32_t)(((1ull << 32) + p - 1) / p);
        sp.h[t] = p / 2;
        sp.bias[t] = -(8388608.0f + (float)(p / 2));
        unsigned long long c = 1;
        for (int i = 0; i < LIMB13; ++i) {
            sp.c13[t][i] = (uint32_t)c;
            c = (c << 13) % p;
        }
    }
}

int limbs_for(int nmod) { return std::max(4, (modulus_product(nmod).bitlen() + 13 + 31) / 32); }

void fill_crt(CrtConst& cp, int nmod) {
    std::memset(&cp, 0, sizeof(cp));
    cp.nmod = nmod;
    const Big M = modulus_product(nmod);
    for (int t = 0; t < nmod; ++t) {
        Big Mt;
        Mt.w[0] = 1;
        for (int s = 0; s < nmod; ++s)
            if (s != t) Mt.mul_small(kModuli[s]);
        const uint32_t y = inverse_mod(Mt.mod_small(kModuli[t]), kModuli[t]);
        Mt.mul_small(y);
        std::memcpy(cp.w[t], Mt.w, sizeof(Mt.w));
        for (int q = 0; q < 2 * LIMBS; ++q) cp.w16[t][q] = (Mt.w[q / 2] >> (16 * (q % 2))) & 0xFFFFu;
    }
    std::memcpy(cp.M, M.w, sizeof(M.w));
    // M / 2^(32 (L-2)) from its top three limbs, as the kernel forms X's
    const int L = limbs_for(nmod);
    const double m2 = (double)M.w[L - 1] * 4294967296.0 + (double)M.w[L - 2] + (double)M.w[L - 3] / 4294967296.0;
    cp.inv_m2 = (float)(1.0 / m2);
}

void fill_combine(CombineParams& cp, int nmod, int P) {
    std::memset(&cp, 0, sizeof(cp));
    cp.nmod = nmod;
    cp.twoP = 2 * P;
    fill_crt(cp.crt, nmod);
}

template <int NL>
void launch_split_nl(bool kcontig, const double* X, int64_t ld, int64_t rows, int64_t k, const int* exps,
                     int64_t k_pad, int64_t rows_pad, uint16_t* out, const SplitParams& sp, dim3 grid,
                     cudaStream_t st) {
    if constexpr (NL <= 5) {
        if (sp.P <= 63) {  // the scaled integers fit one 64-bit word
            if (kcontig) split_kernel<true, NL, true><<<grid, 256, 0, st>>>(X, ld, rows, k, exps, k_pad, rows_pad, out, sp);
            else split_kernel<false, NL, true><<<grid, 256, 0, st>>>(X, ld, rows, k, exps, k_pad, rows_pad, out, sp);
            return;
        }
    }
    if (kcontig) split_kernel<true, NL, false><<<grid, 256, 0, st>>>(X, ld, rows, k, exps, k_pad, rows_pad, out, sp);
    else split_kernel<false, NL, false><<<grid, 256, 0, st>>>(X, ld, rows, k, exps, k_pad, rows_pad, out, sp);
}

void launch_split(bool kcontig, const double* X, int64_t ld, int64_t rows, int64_t k, const int* exps,
                  int64_t k_pad, int64_t rows_pad, uint16_t* out, const SplitParams& sp, dim3 grid, cudaStream_t st) {
#define CGB_SPLIT_NL(NL) launch_split_nl<NL>(kcontig, X, ld, rows, k, exps, k_pad, rows_pad, out, sp, grid, st)
    switch (sp.limbs) {  // P <= 64: 5 limbs; <= 77: 6; <= 90: 7; <= 103: 8; else 9
        case 1: case 2: case 3: case 4: case 5: CGB_SPLIT_NL(5); break;
        case 6: CGB_SPLIT_NL(6); break;
        case 7: CGB_SPLIT_NL(7); break;
        case 8: CGB_SPLIT_NL(8); break;
        default: CGB_SPLIT_NL(9); break;
    }
#undef CGB_SPLIT_NL
}

template <int NL>
void launch_split_cplx_nl(bool kcontig, bool bside, const double2* X, int64_t ld, int64_t rows, int64_t k,
                          const int* exps, int64_t kh, int64_t rows_pad, int64_t slice_rows, int conj, uint16_t* out,
                          const SplitParams& sp, dim3 grid, cudaStream_t st) {
#define CGB_SPLITC(KC, BS) \
    split_cplx_kernel<KC, BS, NL><<<grid, 256, 0, st>>>(X, ld, rows, k, exps, kh, rows_pad, slice_rows, conj, out, sp)
    if (kcontig) {
        if (bside) CGB_SPLITC(true, true); else CGB_SPLITC(true, false);
    } else {
        if (bside) CGB_SPLITC(false, true); else CGB_SPLITC(false, false);
    }
#undef CGB_SPLITC
}

void launch_split_cplx(bool kcontig, bool bside, const double2* X, int64_t ld, int64_t rows, int64_t k,
                       const int* exps, int64_t kh, int64_t rows_pad, int64_t slice_rows, int conj, uint16_t* out,
                       const SplitParams& sp, dim3 grid, cudaStream_t st) {
#define CGB_SPLITC_NL(NL) \
    launch_split_cplx_nl<NL>(kcontig, bside, X, ld, rows, k, exps, kh, rows_pad, slice_rows, conj, out, sp, grid, st)
    switch (sp.limbs) {
        case 1: case 2: case 3: case 4: case 5: CGB_SPLITC_NL(5); break;
        case 6: CGB_SPLITC_NL(6); break;
        case 7: CGB_SPLITC_NL(7); break;
        case 8: CGB_SPLITC_NL(8); break;
        default: CGB_SPLITC_NL(9); break;
    }
#undef CGB_SPLITC_NL
}

struct Workspace {
    DeviceBuffer resA, resB, expA, expB, part, R, stats, err;
    DeviceBuffer T;  // complex alpha/beta: the product before alpha*T + beta*C
    Stats* host_stats = nullptr;
    unsigned* host_err = nullptr;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
};

std::mutex g_ws_mu;
std::map<std::pair<int, cudaStream_t>, Workspace*> g_ws;

Workspace* workspace(cudaStream_t s) {
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lock(g_ws_mu);
    auto& w = g_ws[{dev, s}];
    if (!w) w = new Workspace();
    // pinned staging and events, (re)tried until they exist: a failed
    // allocation fails this call only
    if (!w->host_stats && pinned_alloc((void**)&w->host_stats, sizeof(Stats)) != cudaSuccess) w->host_stats = nullptr;
    if (!w->host_err && pinned_alloc((void**)&w->host_err, sizeof(unsigned)) != cudaSuccess) w->host_err = nullptr;
    for (auto& e : w->ev)
        if (!e && cudaEventCreate(&e) != cudaSuccess) e = nullptr;
    cudaGetLastError();
    return w;
}

// Frees the workspace of a stream that is about to be destroyed: a later
// stream may get the same handle and must not inherit it (nor may the memory
// outlive the stream).  Work on the stream must be complete.
void release_workspace(cudaStream_t s) {
    int dev = 0;
    cudaGetDevice(&dev);
    Workspace* w = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_ws_mu);
        auto it = g_ws.find({dev, s});
        if (it == g_ws.end()) return;
        w = it->second;
        g_ws.erase(it);
    }
    if (w->host_stats) cudaFreeHost(w->host_stats);
    if (w->host_err) cudaFreeHost(w->host_err);
    for (auto e : w->ev)
        if (e) cudaEventDestroy(e);
    delete w;  // the device buffers free themselves
    cudaGetLastError();
}

int pair_grid(int units, int* grid) {
    static PerDevice<int> pairs;
    int n = 0;
    CGB_CHECK(pairs.get(
        [](int& v) {
            CGB_CUDA(cudaFuncSetAttribute(gemm_pair_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(2 * device_sm_count(), 1, 1);
            cfg.blockDim = dim3(THREADS, 1, 1);
            cfg.dynamicSmemBytes = SMEM_BYTES;
            cudaLaunchAttribute attr;
            attr.id = cudaLaunchAttributeClusterDimension;
            attr.val.clusterDim.x = 2;
            attr.val.clusterDim.y = 1;
            attr.val.clusterDim.z = 1;
            cfg.attrs = &attr;
            cfg.numAttrs = 1;
            CGB_CUDA(cudaOccupancyMaxActiveClusters(&v, gemm_pair_kernel, &cfg));
            v = std::min(v, device_sm_count() / 2);
            if (v < 1) return set_error(COSMA_GPU_ERROR_CUDA, "ozaki2: no CTA pair of the GEMM fits on the GPU");
            return COSMA_GPU_SUCCESS;
        },
        &n));
    *grid = 2 * std::min(units, n);
    return COSMA_GPU_SUCCESS;
}

int launch_gemm(const void* resA, const void* resB, int64_t k_pad, const GemmParams& p, cudaStream_t st) {
    CUtensorMap tmA, tmB;
    CGB_CHECK(make_tmap_2d(&tmA, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, resA, (uint64_t)k_pad,
                           (uint64_t)p.nmod * p.a_rows_pad, (uint64_t)k_pad * 2, BKE, BM));
    CGB_CHECK(make_tmap_2d(&tmB, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, resB, (uint64_t)k_pad,
                           (uint64_t)p.nmod * p.b_rows_pad, (uint64_t)k_pad * 2, BKE, BN / 2));
    int grid = 0;
    CGB_CHECK(pair_grid(p.nmod * p.num_tiles, &grid));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid, 1, 1);
    cfg.blockDim = dim3(THREADS, 1, 1);
    cfg.dynamicSmemBytes = SMEM_BYTES;
    cfg.stream = st;
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = 2;
    attr.val.clusterDim.y = 1;
    attr.val.clusterDim.z = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    CGB_CUDA(cudaLaunchKernelEx(&cfg, gemm_pair_kernel, tmA, tmB, p));
    return COSMA_GPU_SUCCESS;
}

template <int MODE>
void launch_combine_t(const CombineParams& cp, int limbs, unsigned grid, cudaStream_t st) {
    switch (limbs) {
        case 4: combine_kernel<4, MODE><<<grid, 128, 0, st>>>(cp); break;
        case 5: combine_kernel<5, MODE><<<grid, 128, 0, st>>>(cp); break;
        case 6: combine_kernel<6, MODE><<<grid, 128, 0, st>>>(cp); break;
        case 7: combine_kernel<7, MODE><<<grid, 128, 0, st>>>(cp); break;
        default: combine_kernel<8, MODE><<<grid, 128, 0, st>>>(cp); break;
    }
}

int launch_combine(CombineParams& cp, int nmod, int64_t gemm_cols, cudaStream_t st) {
    cp.row_blocks = ceil_div(cp.m, 32);
    const int64_t blocks = cp.row_blocks * ceil_div(gemm_cols, 16);
    if (blocks > 0x7FFFFFFF) return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "ozaki2: C too large for the combine grid");
    const int L = limbs_for(nmod);
    if (cp.E) launch_combine_t<kResidual>(cp, L, (unsigned)blocks, st);
    else if (cp.alpha_one && cp.beta_zero) launch_combine_t<kStoreC>(cp, L, (unsigned)blocks, st);
    else launch_combine_t<kScaleC>(cp, L, (unsigned)blocks, st);
    CGB_CUDA(cudaGetLastError());
    return COSMA_GPU_SUCCESS;
}

void fill_gemm(GemmParams& p, int nmod, int64_t m_pad, int64_t n_pad, int64_t k_pad, void* R, unsigned* err) {
    std::memset(&p, 0, sizeof(p));
    p.num_m_tiles = (int)(m_pad / BM);
    p.num_n_tiles = (int)(n_pad / BN);
    p.num_tiles = (p.num_m_tiles / 2) * p.num_n_tiles;
    p.nmod = nmod;
    p.kb_count = (int)(k_pad / BKE);
    p.a_rows_pad = (int)m_pad;
    p.b_rows_pad = (int)n_pad;
    p.m_pad = m_pad;
    p.nb16 = n_pad / 16;
    p.R = (uint8_t*)R;
    for (int t = 0; t < nmod; ++t) {
        const uint32_t q = kModuli[t];
        p.p[t] = q;
        p.magic[t] = (uint32_t)((1ull << 32) / q);
        p.bias[t] = (uint32_t)((((1ull << 30) + q - 1) / q) * q);
    }
    p.err = err;
}

// Shared front end: row scaling, statistics read-back, choice of N and P.
// Returns with *fallback set when the inputs hold Inf/NaN.
struct Plan {
    int nmod = 0, P = 0;
    double spread = 0.0;
    bool exact = false;  // every input bit kept: the product is exact
};

int finish_info(cosma_gpu_ozaki_info* info, Workspace* w, const Plan& pl, int64_t kb_count) {
    if (!info) return COSMA_GPU_SUCCESS;
    float prep = 0.f, gemm = 0.f;
    cudaEventElapsedTime(&prep, w->ev[0], w->ev[1]);
    cudaEventElapsedTime(&gemm, w->ev[2], w->ev[3]);
    info->slices = pl.nmod;
    info->products = pl.nmod;
    info->fraction_bits = pl.P;
    info->exact_product = pl.exact ? 1 : 0;
    info->groups = pl.nmod * (int)((kb_count + KB_PER_CHUNK - 1) / KB_PER_CHUNK);
    info->spread_bits = pl.spread;
    info->prep_ms += prep;
    info->gemm_ms += gemm;
    return COSMA_GPU_SUCCESS;
}

int check_device_error(Workspace* w, cudaStream_t st) {
    CGB_CUDA(cudaMemcpyAsync(w->host_err, w->err.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaStreamSynchronize(st));
    if (*w->host_err)
        return set_error(COSMA_GPU_ERROR_DEVICE_TIMEOUT,
                         "ozaki2 gemm: a pipeline wait timed out (device code " + std::to_string(*w->host_err) + ")");
    return COSMA_GPU_SUCCESS;
}

// Residual mode: instead of writing C, E = op(A) op(B) - Ct (exact before its
// one rounding) and Rx = op(A) op(B) rounded once, both m x n with ld ldo.
struct Residual {
    const double* Ct = nullptr;
    int64_t ldt = 0;
    double* E = nullptr;
    double* Rx = nullptr;
    int64_t ldo = 0;
};

int dgemm(const GemmDesc& g, int nmod_req, cudaStream_t st, cosma_gpu_ozaki_info* info, const Residual* res = nullptr) {
    const int64_t m = g.m, n = g.n, k = g.k;
    const bool a_kc = g.opa != 0, b_kc = g.opb == 0;  // op(A) rows / op(B) columns contiguous along K
    const double* A = (const double*)g.A;
    const double* B = (const double*)g.B;
    Workspace* w = workspace(st);
    if (!w->host_stats || !w->host_err) return set_error(COSMA_GPU_ERROR_OUT_OF_MEMORY, "ozaki2: pinned staging");
    if (!w->ev[0] || !w->ev[3]) return set_error(COSMA_GPU_ERROR_CUDA, "ozaki2: timing events");
    const int64_t m_pad = ceil_div(m, 2 * BM) * 2 * BM, n_pad = ceil_div(n, BN) * BN, k_pad = ceil_div(k, BKE) * BKE;

    // 1. scaling + spread statistics
    CGB_CHECK(w->stats.reserve(sizeof(Stats), st));
    CGB_CHECK(w->err.reserve(sizeof(unsigned), st));
    CGB_CHECK(w->expA.reserve((size_t)m_pad * 4, st));
    CGB_CHECK(w->expB.reserve((size_t)n_pad * 4, st));
    Stats* st_dev = (Stats*)w->stats.ptr;
    CGB_CUDA(cudaEventRecord(w->ev[0], st));
    CGB_CUDA(cudaMemsetAsync(st_dev, 0, sizeof(Stats), st));
    CGB_CUDA(cudaMemsetAsync(w->err.ptr, 0, sizeof(unsigned), st));
    CGB_CUDA(cudaMemsetAsync(w->expA.ptr, 0, (size_t)m_pad * 4, st));
    CGB_CUDA(cudaMemsetAsync(w->expB.ptr, 0, (size_t)n_pad * 4, st));
    CGB_CHECK(oz::scale_operand(a_kc, A, g.lda, m, k, (int*)w->expA.ptr, w->part, st_dev, 0, st, 1));
    CGB_CHECK(oz::scale_operand(b_kc, B, g.ldb, n, k, (int*)w->expB.ptr, w->part, st_dev, 1, st, 1));
    CGB_CUDA(cudaMemcpyAsync(w->host_stats, st_dev, sizeof(Stats), cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaStreamSynchronize(st));
    const Stats hs = *w->host_stats;
    Plan pl;
    pl.spread = (double)hs.spread[0] + (double)hs.spread[1];
    if (hs.nonfinite) {  // Inf/NaN have no residues: the native FP64 kernel propagates them
        if (res) return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "ozaki2 residual: A and B must be finite");
        if (info) info->fallback_native = 1;
        return native_gemm(g, st);
    }
    CGB_CHECK(choose(nmod_req, pl.spread, k, &pl.nmod, &pl.P, std::max(hs.exact_bits[0], hs.exact_bits[1])));
    pl.exact = pl.P >= std::max(hs.exact_bits[0], hs.exact_bits[1]);

    // 2. residue matrices
    const size_t resA_bytes = (size_t)pl.nmod * m_pad * k_pad * 2, resB_bytes = (size_t)pl.nmod * n_pad * k_pad * 2;
    CGB_CHECK(w->resA.reserve(resA_bytes, st));
    CGB_CHECK(w->resB.reserve(resB_bytes, st));
    SplitParams sp;
    fill_split(sp, pl.nmod, pl.P);
    {
        dim3 gA((unsigned)(m_pad / 32), (unsigned)(k_pad / 64)), gB((unsigned)(n_pad / 32), (unsigned)(k_pad / 64));
        if (gA.y > 65535 || gB.y > 65535) return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "ozaki2: k too large");
        launch_split(a_kc, A, g.lda, m, k, (const int*)w->expA.ptr, k_pad, m_pad, (uint16_t*)w->resA.ptr, sp, gA, st);
        launch_split(b_kc, B, g.ldb, n, k, (const int*)w->expB.ptr, k_pad, n_pad, (uint16_t*)w->resB.ptr, sp, gB, st);
        CGB_CUDA(cudaGetLastError());
    }
    CGB_CUDA(cudaEventRecord(w->ev[1], st));

    // 3. modular GEMMs -> residue bytes
    CGB_CHECK(w->R.reserve((size_t)pl.nmod * m_pad * n_pad, st));
    GemmParams gp;
    fill_gemm(gp, pl.nmod, m_pad, n_pad, k_pad, w->R.ptr, (unsigned*)w->err.ptr);
    CGB_CUDA(cudaEventRecord(w->ev[2], st));
    CGB_CHECK(launch_gemm(w->resA.ptr, w->resB.ptr, k_pad, gp, st));
    CGB_CUDA(cudaEventRecord(w->ev[3], st));

    // 4. reconstruction, scaling, alpha and beta
    CombineParams cp;
    fill_combine(cp, pl.nmod, pl.P);
    cp.m = m;
    cp.n = n;
    cp.ldc = g.ldc;
    cp.m_pad = m_pad;
    cp.nb16 = n_pad / 16;
    cp.n_split = INT64_MAX;
    cp.cs = 1;
    cp.R = (const uint8_t*)w->R.ptr;
    cp.expA = (const int*)w->expA.ptr;
    cp.expB = (const int*)w->expB.ptr;
    cp.C = (double*)g.C;
    cp.alpha = g.alpha[0];
    cp.beta = g.beta[0];
    cp.alpha_one = g.alpha[0] == 1.0;
    cp.beta_zero = g.beta[0] == 0.0;
    if (res) {
        cp.Ct = res->Ct;
        cp.ldt = res->ldt;
        cp.E = res->E;
        cp.Rx = res->Rx;
        cp.ldo = res->ldo;
    }
    CGB_CHECK(launch_combine(cp, pl.nmod, n, st));
    CGB_CHECK(check_device_error(w, st));
    return finish_info(info, w, pl, gp.kb_count);
}

int zgemm(const GemmDesc& g, int nmod_req, cudaStream_t st, cosma_gpu_ozaki_info* info) {
    const int64_t m = g.m, n = g.n, k = g.k;
    const bool a_kc = g.opa != 0, b_kc = g.opb == 0;
    const double2* A = (const double2*)g.A;
    const double2* B = (const double2*)g.B;
    Workspace* w = workspace(st);
    if (!w->host_stats || !w->host_err) return set_error(COSMA_GPU_ERROR_OUT_OF_MEMORY, "ozaki2: pinned staging");
    if (!w->ev[0] || !w->ev[3]) return set_error(COSMA_GPU_ERROR_CUDA, "ozaki2: timing events");
    const int64_t m_pad = ceil_div(m, 2 * BM) * 2 * BM, nh = ceil_div(n, BN) * BN, kh = ceil_div(k, BKE) * BKE;
    const int64_t k_pad = 2 * kh, n_pad = 2 * nh;

    CGB_CHECK(w->stats.reserve(sizeof(Stats), st));
    CGB_CHECK(w->err.reserve(sizeof(unsigned), st));
    CGB_CHECK(w->expA.reserve((size_t)m_pad * 4, st));
    CGB_CHECK(w->expB.reserve((size_t)nh * 4, st));
    Stats* st_dev = (Stats*)w->stats.ptr;
    CGB_CUDA(cudaEventRecord(w->ev[0], st));
    CGB_CUDA(cudaMemsetAsync(st_dev, 0, sizeof(Stats), st));
    CGB_CUDA(cudaMemsetAsync(w->err.ptr, 0, sizeof(unsigned), st));
    CGB_CUDA(cudaMemsetAsync(w->expA.ptr, 0, (size_t)m_pad * 4, st));
    CGB_CUDA(cudaMemsetAsync(w->expB.ptr, 0, (size_t)nh * 4, st));
    CGB_CHECK(oz::scale_operand(a_kc, (const double*)A, g.lda, m, k, (int*)w->expA.ptr, w->part, st_dev, 0, st, 2));
    CGB_CHECK(oz::scale_operand(b_kc, (const double*)B, g.ldb, n, k, (int*)w->expB.ptr, w->part, st_dev, 1, st, 2));
    CGB_CUDA(cudaMemcpyAsync(w->host_stats, st_dev, sizeof(Stats), cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaStreamSynchronize(st));
    const Stats hs = *w->host_stats;
    Plan pl;
    pl.spread = (double)hs.spread[0] + (double)hs.spread[1];
    if (hs.nonfinite) {
        if (info) info->fallback_native = 1;
        return native_gemm(g, st);
    }
    CGB_CHECK(choose(nmod_req, pl.spread, 2 * k, &pl.nmod, &pl.P, std::max(hs.exact_bits[0], hs.exact_bits[1])));
    pl.exact = pl.P >= std::max(hs.exact_bits[0], hs.exact_bits[1]);

    CGB_CHECK(w->resA.reserve((size_t)pl.nmod * m_pad * k_pad * 2, st));
    CGB_CHECK(w->resB.reserve((size_t)pl.nmod * n_pad * k_pad * 2, st));
    SplitParams sp;
    fill_split(sp, pl.nmod, pl.P);
    {
        dim3 gA((unsigned)(m_pad / 32), (unsigned)(kh / 64)), gB((unsigned)(nh / 32), (unsigned)(kh / 64));
        if (gA.y > 65535) return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "ozaki2: k too large");
        uint16_t* rA = (uint16_t*)w->resA.ptr;
        uint16_t* rB = (uint16_t*)w->resB.ptr;
        const int* eA = (const int*)w->expA.ptr;
        const int* eB = (const int*)w->expB.ptr;
        launch_split_cplx(a_kc, false, A, g.lda, m, k, eA, kh, m_pad, m_pad, g.opa == 2, rA, sp, gA, st);
        launch_split_cplx(b_kc, true, B, g.ldb, n, k, eB, kh, nh, n_pad, g.opb == 2, rB, sp, gB, st);
        CGB_CUDA(cudaGetLastError());
    }
    CGB_CUDA(cudaEventRecord(w->ev[1], st));

    CGB_CHECK(w->R.reserve((size_t)pl.nmod * m_pad * n_pad, st));
    GemmParams gp;
    fill_gemm(gp, pl.nmod, m_pad, n_pad, k_pad, w->R.ptr, (unsigned*)w->err.ptr);
    CGB_CUDA(cudaEventRecord(w->ev[2], st));
    CGB_CHECK(launch_gemm(w->resA.ptr, w->resB.ptr, k_pad, gp, st));
    CGB_CUDA(cudaEventRecord(w->ev[3], st));

    // real alpha and beta are applied by the combine kernel, complex ones by
    // alpha*T + beta*C afterwards
    const bool fused = g.alpha[1] == 0.0 && g.beta[1] == 0.0;
    CombineParams cp;
    fill_combine(cp, pl.nmod, pl.P);
    cp.m = m;
    cp.n = n;
    cp.m_pad = m_pad;
    cp.nb16 = n_pad / 16;
    cp.n_split = nh;
    cp.cs = 2;
    cp.R = (const uint8_t*)w->R.ptr;
    cp.expA = (const int*)w->expA.ptr;
    cp.expB = (const int*)w->expB.ptr;
    if (fused) {
        cp.C = (double*)g.C;
        cp.ldc = g.ldc;
        cp.alpha = g.alpha[0];
        cp.beta = g.beta[0];
    } else {
        CGB_CHECK(w->T.reserve((size_t)m * n * 16, st));
        cp.C = (double*)w->T.ptr;
        cp.ldc = m;
        cp.alpha = 1.0;
        cp.beta = 0.0;
    }
    cp.alpha_one = cp.alpha == 1.0;
    cp.beta_zero = cp.beta == 0.0;
    CGB_CHECK(launch_combine(cp, pl.nmod, n_pad, st));
    CGB_CHECK(check_device_error(w, st));
    if (!fused) CGB_CHECK(unpack_device(Scalar::Z, m, n, g.alpha, w->T.ptr, m, g.beta, g.C, g.ldc, st));
    return finish_info(info, w, pl, gp.kb_count);
}

// ------------------------------------------------------ host operands, overlapped
// One-step DGEMM, or ZGEMM with real alpha and beta, on host A, B and C
// (C = alpha op(A) op(B) + beta C), with the host link's copies overlapped
// with the work: op(A) arrives in MA row panels and op(B) in NB column
// panels on the copy stream, each panel's exponents
// and statistics are taken as it lands, block (i, j)'s residue split and
// modular GEMM start as soon as its two panels are in, and each block's C
// leaves on its own stream while the next block computes.  The modulus count
// is chosen from the first two panels and must be the one the whole data
// gives (so the result is bit-identical to the device path's); it is checked
// before any C is written, and when it differs, or the data holds Inf/NaN,
// the call returns with *taken = false, C untouched and nothing in flight.
struct PipeWorkspace {
    DeviceBuffer a, b, resA, resB, expA, expB, part, R[8], C[8], stats, err;
    Stats* host_stats = nullptr;  // one record per panel
    unsigned* host_err = nullptr;
    std::vector<cudaEvent_t> ev;
    cudaStream_t ss = nullptr;  // exponents and statistics of landed panels, beside the GEMMs
    std::unique_ptr<CopyWorker> worker;
};

std::mutex g_pipe_mu;
std::map<std::pair<int, cudaStream_t>, PipeWorkspace*> g_pipe;
constexpr int kPipeMaxPanels = 16;
constexpr int kPipeEvents = 64;
constexpr int kPipeRing = 8;                        // blocks in flight: residue bytes and C slots
constexpr size_t kPipeRingBytes = (size_t)8 << 30;  // at most this much HBM for the ring, 2 blocks at least

PipeWorkspace* pipe_workspace(cudaStream_t s) {
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lock(g_pipe_mu);
    auto& w = g_pipe[{dev, s}];
    if (!w) w = new PipeWorkspace();
    if (!w->host_stats && pinned_alloc((void**)&w->host_stats, kPipeMaxPanels * sizeof(Stats)) != cudaSuccess)
        w->host_stats = nullptr;
    if (!w->host_err && pinned_alloc((void**)&w->host_err, sizeof(unsigned)) != cudaSuccess) w->host_err = nullptr;
    if (w->ev.empty()) {
        w->ev.assign(kPipeEvents, nullptr);
        for (auto& e : w->ev)
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) e = nullptr;
    }
    if (!w->ss && cudaStreamCreateWithFlags(&w->ss, cudaStreamNonBlocking) != cudaSuccess) w->ss = nullptr;
    if (!w->worker) {
        try {
            w->worker.reset(new CopyWorker(dev));
        } catch (...) {  // no thread to be had: the overlapped form is not taken
            w->worker.reset();
        }
    }
    cudaGetLastError();
    return w;
}

void release_pipe_workspace(cudaStream_t s) {
    int dev = 0;
    cudaGetDevice(&dev);
    PipeWorkspace* w = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_pipe_mu);
        auto it = g_pipe.find({dev, s});
        if (it == g_pipe.end()) return;
        w = it->second;
        g_pipe.erase(it);
    }
    w->worker.reset();  // runs what is queued (copies recording the events below), then joins
    if (w->host_stats) cudaFreeHost(w->host_stats);
    if (w->host_err) cudaFreeHost(w->host_err);
    for (auto e : w->ev)
        if (e) cudaEventDestroy(e);
    if (w->ss) {
        cudaStreamSynchronize(w->ss);
        cudaStreamDestroy(w->ss);
    }
    delete w;
    cudaGetLastError();
}

// Combined statistics of a set of panel records (A panels in field 0, B in 1).
Stats merge_stats(const Stats* s, const std::vector<int>& idx) {
    Stats r{};
    for (int i : idx) {
        r.nonfinite |= s[i].nonfinite;
        for (int w = 0; w < 2; ++w) {
            r.spread[w] = std::max(r.spread[w], s[i].spread[w]);
            r.exact_bits[w] = std::max(r.exact_bits[w], s[i].exact_bits[w]);
        }
    }
    return r;
}

int gemm_host_pipelined_body(const GemmDesc& g, int nmod_req, cudaStream_t cs, cudaStream_t hs, cudaStream_t ds,
                              cosma_gpu_ozaki_info* info, int64_t* h2d_bytes, int64_t* d2h_bytes, bool* taken) {
    *taken = false;
    const int64_t m = g.m, n = g.n, k = g.k;
    const bool cplx = g.scalar == Scalar::Z;
    if ((g.scalar != Scalar::D && !cplx) || k > KMAX || k < 1 || m < 1 || n < 1) return COSMA_GPU_SUCCESS;
    // complex alpha / beta need a product buffer and an unpack per block: the
    // regular path
    if (cplx && (g.alpha[1] != 0.0 || g.beta[1] != 0.0)) return COSMA_GPU_SUCCESS;
    // Complex operands follow the device ZGEMM's layout: op(A) rows
    // [Re | sa Im] of 2 kh, op(B) columns as two stacked rows (Re C, Im C) of
    // each block's GEMM; es doubles per element.
    const int es = cplx ? 2 : 1;
    const int64_t eb8 = 8 * es;  // bytes per element
    const bool a_kc = g.opa != 0, b_kc = g.opb == 0;  // op(A) rows / op(B) columns contiguous along K
    // op(A) in row panels: a lead panel of at most 2048 rows, then panels of
    // half the rows (the last one shorter: 2048, 8192, 6144 at m = 16384);
    // op(B) in up to 4 column panels.  At 16384^3 the first block waits for
    // 0.75 GB instead of 1.5 GB.
    const Panels PA = make_panels(m, m >= 2048 ? 2 : 1, 2048);
    const Panels PB = make_panels(n, n >= 4096 ? 4 : (n >= 2048 ? 2 : 1), n);
    const int MA = PA.count, NB = PB.count, NP = MA + NB;
    if (MA * NB < 2 || NP > kPipeMaxPanels) return COSMA_GPU_SUCCESS;
    PipeWorkspace* w = pipe_workspace(cs);
    if (!w->host_stats || !w->host_err) return set_error(COSMA_GPU_ERROR_OUT_OF_MEMORY, "ozaki2: pinned staging");
    for (auto e : w->ev)
        if (!e) return set_error(COSMA_GPU_ERROR_CUDA, "ozaki2: pipeline events");
    if (!w->ss) return set_error(COSMA_GPU_ERROR_CUDA, "ozaki2: pipeline stream");
    if (!w->worker) return COSMA_GPU_SUCCESS;  // no copy thread: the regular path
    cudaStream_t ss = w->ss;
    const int64_t kh = ceil_div(k, BKE) * BKE, k_pad = es * kh;
    const double* A = (const double*)g.A;
    const double* B = (const double*)g.B;
    double* C = (double*)g.C;
    const bool beta_zero = g.beta[0] == 0.0;

    // panel geometry: compact device copies, padded exponent / residue blocks
    std::vector<int64_t> offA(MA), offB(NB), eoffA(MA), eoffB(NB);
    int64_t a_elems = 0, b_elems = 0, ea = 0, eb = 0;
    for (int i = 0; i < MA; ++i) {
        offA[i] = a_elems; a_elems += PA.rows(i, m) * k;
        eoffA[i] = ea; ea += ceil_div(PA.rows(i, m), 2 * BM) * 2 * BM;
    }
    for (int j = 0; j < NB; ++j) {
        offB[j] = b_elems; b_elems += PB.rows(j, n) * k;
        eoffB[j] = eb; eb += ceil_div(PB.rows(j, n), BN) * BN;
    }
    const int64_t ma_pad = ceil_div(PA.largest(), 2 * BM) * 2 * BM, nb_pad = ceil_div(PB.largest(), BN) * BN;
    // everything that could allocate is reserved before the first copy: a
    // growing buffer frees its old memory, which waits for the whole device
    CGB_CHECK(w->a.reserve((size_t)a_elems * eb8, cs));
    CGB_CHECK(w->b.reserve((size_t)b_elems * eb8, cs));
    CGB_CHECK(w->expA.reserve((size_t)ea * 4, cs));
    CGB_CHECK(w->expB.reserve((size_t)eb * 4, cs));
    CGB_CHECK(w->part.reserve((size_t)64 * std::max(PA.largest(), PB.largest()) * 12, cs));
    CGB_CHECK(w->stats.reserve((size_t)NP * sizeof(Stats), cs));
    CGB_CHECK(w->err.reserve(sizeof(unsigned), cs));
    Stats* sdev = (Stats*)w->stats.ptr;
    double* dA = (double*)w->a.ptr;
    double* dB = (double*)w->b.ptr;
    int* expA = (int*)w->expA.ptr;
    int* expB = (int*)w->expB.ptr;
    CGB_CUDA(cudaMemsetAsync(sdev, 0, (size_t)NP * sizeof(Stats), cs));
    CGB_CUDA(cudaMemsetAsync(w->err.ptr, 0, sizeof(unsigned), cs));
    CGB_CUDA(cudaMemsetAsync(expA, 0, (size_t)ea * 4, cs));
    CGB_CUDA(cudaMemsetAsync(expB, 0, (size_t)eb * 4, cs));
    CGB_CUDA(cudaStreamSynchronize(cs));
    int evi = 0;
    auto next_event = [&]() { return w->ev[evi++]; };
    cudaEvent_t ev_copy[kPipeMaxPanels];    // panel p landed in HBM (A panels 0..MA-1, B panels MA..)
    cudaEvent_t ev_scaled[kPipeMaxPanels];  // its exponents and statistics are in
    *h2d_bytes = 0;
    *d2h_bytes = 0;

    // The first panel of each operand crosses before any kernel of the call
    // runs, so a pageable one may take the device copy kernel (at the link's
    // rate); every later copy runs beside the persistent GEMMs, whose CTAs a
    // copy kernel would hold up, and goes through the copy engines, issued by
    // the copy thread (pageable memory through the pinned staging buffers).
    CopyWorker& cw = *w->worker;
    auto copy_task = [](void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t cols,
                        cudaMemcpyKind kind, cudaStream_t st, cudaEvent_t wait_ev, cudaEvent_t done_ev) {
        return [=]() -> int {
            if (wait_ev) CGB_CUDA(cudaStreamWaitEvent(st, wait_ev, 0));
            CGB_CHECK(copy_2d_from_thread(dst, dpitch, src, spitch, width, cols, kind, st));
            CGB_CUDA(cudaEventRecord(done_ev, st));
            return COSMA_GPU_SUCCESS;
        };
    };
    uint64_t tk_copy[kPipeMaxPanels] = {};
    auto copy_in = [&](int p, void* dst, size_t dpitch, const void* src, size_t spitch, size_t width,
                       size_t cols) -> int {
        if (p == 0 || p == MA) {
            CGB_CHECK(copy_2d_overlapped(dst, dpitch, src, spitch, width, cols, cudaMemcpyHostToDevice, hs));
            CGB_CUDA(cudaEventRecord(ev_copy[p], hs));
            tk_copy[p] = 0;  // nothing to wait for on the copy thread
        } else {
            tk_copy[p] = cw.post(copy_task(dst, dpitch, src, spitch, width, cols, cudaMemcpyHostToDevice, hs,
                                           nullptr, ev_copy[p]));
        }
        return COSMA_GPU_SUCCESS;
    };
    // device copy of op(A) rows / op(B) columns of one panel, compact
    auto copy_panel = [&](int p) -> int {
        ev_copy[p] = next_event();
        if (p < MA) {
            const int64_t i0 = PA.first(p), mi = PA.rows(p, m);
            if (!a_kc) CGB_CHECK(copy_in(p, dA + offA[p] * es, mi * eb8, A + i0 * es, g.lda * eb8, mi * eb8, k));
            else CGB_CHECK(copy_in(p, dA + offA[p] * es, k * eb8, A + i0 * g.lda * es, g.lda * eb8, k * eb8, mi));
            *h2d_bytes += mi * k * eb8;
        } else {
            const int j = p - MA;
            const int64_t j0 = PB.first(j), nj = PB.rows(j, n);
            if (b_kc) CGB_CHECK(copy_in(p, dB + offB[j] * es, k * eb8, B + j0 * g.ldb * es, g.ldb * eb8, k * eb8, nj));
            else CGB_CHECK(copy_in(p, dB + offB[j] * es, nj * eb8, B + j0 * es, g.ldb * eb8, nj * eb8, k));
            *h2d_bytes += nj * k * eb8;
        }
        return COSMA_GPU_SUCCESS;
    };
    // exponents and statistics of one panel as soon as it lands, on the
    // statistics stream (small kernels that run beside the GEMMs)
    auto scale_panel = [&](int p) -> int {
        CGB_CHECK(cw.wait(tk_copy[p]));  // its event is recorded
        CGB_CUDA(cudaStreamWaitEvent(ss, ev_copy[p], 0));
        if (p < MA) {
            const int64_t mi = PA.rows(p, m);
            CGB_CHECK(oz::scale_operand(a_kc, dA + offA[p] * es, a_kc ? k : mi, mi, k, expA + eoffA[p], w->part,
                                        sdev + p, 0, ss, es));
        } else {
            const int j = p - MA;
            const int64_t nj = PB.rows(j, n);
            CGB_CHECK(oz::scale_operand(b_kc, dB + offB[j] * es, b_kc ? k : nj, nj, k, expB + eoffB[j], w->part,
                                        sdev + p, 1, ss, es));
        }
        ev_scaled[p] = next_event();
        CGB_CUDA(cudaEventRecord(ev_scaled[p], ss));
        return COSMA_GPU_SUCCESS;
    };
    // drains the copy worker and every stream (the caller then runs the regular path)
    auto abandon = [&]() -> int {
        CGB_CHECK(cw.drain());
        for (cudaStream_t s : {cs, hs, ds, ss}) CGB_CUDA(cudaStreamSynchronize(s));
        *h2d_bytes = 0;
        return COSMA_GPU_SUCCESS;
    };

    // 1. the first panels of each operand; the modulus count from them
    CGB_CUDA(cudaStreamSynchronize(ss));  // memsets on cs above: ss starts after them
    CGB_CHECK(copy_panel(0));
    CGB_CHECK(copy_panel(MA));
    CGB_CHECK(scale_panel(0));
    CGB_CHECK(scale_panel(MA));
    CGB_CUDA(cudaMemcpyAsync(w->host_stats, sdev, (size_t)NP * sizeof(Stats), cudaMemcpyDeviceToHost, ss));
    CGB_CUDA(cudaStreamSynchronize(ss));
    const Stats s0 = merge_stats(w->host_stats, {0, MA});
    if (s0.nonfinite) return abandon();
    Plan pl;
    pl.spread = (double)s0.spread[0] + (double)s0.spread[1];
    if (choose(nmod_req, pl.spread, es * k, &pl.nmod, &pl.P, std::max(s0.exact_bits[0], s0.exact_bits[1])) !=
        COSMA_GPU_SUCCESS) {
        clear_error();
        return abandon();
    }
    const int N = pl.nmod;
    std::vector<int64_t> roffA(MA), roffB(NB);
    int64_t ra = 0, rb = 0;
    for (int i = 0; i < MA; ++i) { roffA[i] = ra; ra += (int64_t)N * ceil_div(PA.rows(i, m), 2 * BM) * 2 * BM * k_pad; }
    for (int j = 0; j < NB; ++j) { roffB[j] = rb; rb += (int64_t)N * es * ceil_div(PB.rows(j, n), BN) * BN * k_pad; }
    CGB_CHECK(w->resA.reserve((size_t)ra * 2, cs));  // nothing in flight: the first panels are in
    CGB_CHECK(w->resB.reserve((size_t)rb * 2, cs));
    // A ring of NR blocks in flight, each with the residue bytes of its
    // modular GEMM and a C slot: NR blocks are queued before the host has
    // checked every panel's statistics (the wait is for the last panel to
    // cross), and after the check each block's reconstruction follows its
    // GEMM directly, so that one reconstruction and one copy-out remain
    // after the last GEMM.
    const int NBLK = MA * NB;
    const size_t r_bytes = (size_t)N * ma_pad * es * nb_pad, c_bytes = (size_t)PA.largest() * PB.largest() * eb8;
    int NR = std::min(NBLK, kPipeRing);
    while (NR > 2 && (size_t)NR * (r_bytes + c_bytes) > kPipeRingBytes) --NR;
    for (int r = 0; r < NR; ++r) {
        CGB_CHECK(w->R[r].reserve(r_bytes, cs));
        CGB_CHECK(w->C[r].reserve(c_bytes, cs));
    }

    // 2. the other panels: B's first (block row 0 uses them), then A's
    std::vector<int> order;
    for (int p = MA + 1; p < NP; ++p) order.push_back(p);
    for (int p = 1; p < MA; ++p) order.push_back(p);
    for (int p : order) CGB_CHECK(copy_panel(p));
    std::vector<char> scaled(NP, 0);
    scaled[0] = scaled[MA] = 1;
    auto ensure_scaled = [&](int p) -> int {
        if (scaled[p]) return COSMA_GPU_SUCCESS;
        scaled[p] = 1;
        return scale_panel(p);
    };

    SplitParams sp;
    fill_split(sp, N, pl.P);
    std::vector<char> split_done(NP, 0);
    auto split_panel = [&](int p) -> int {
        if (split_done[p]) return COSMA_GPU_SUCCESS;
        split_done[p] = 1;
        CGB_CUDA(cudaStreamWaitEvent(cs, ev_scaled[p], 0));
        if (p < MA) {
            const int64_t mi = PA.rows(p, m), mi_pad = ceil_div(mi, 2 * BM) * 2 * BM;
            const dim3 grid((unsigned)(mi_pad / 32), (unsigned)(kh / 64));
            uint16_t* out = (uint16_t*)w->resA.ptr + roffA[p];
            if (cplx)
                launch_split_cplx(a_kc, false, (const double2*)(dA + offA[p] * 2), a_kc ? k : mi, mi, k, expA + eoffA[p],
                                  kh, mi_pad, mi_pad, g.opa == 2, out, sp, grid, cs);
            else
                launch_split(a_kc, dA + offA[p], a_kc ? k : mi, mi, k, expA + eoffA[p], k_pad, mi_pad, out, sp, grid, cs);
        } else {
            const int j = p - MA;
            const int64_t nj = PB.rows(j, n), nj_pad = ceil_div(nj, BN) * BN;
            const dim3 grid((unsigned)(nj_pad / 32), (unsigned)(kh / 64));
            uint16_t* out = (uint16_t*)w->resB.ptr + roffB[j];
            if (cplx)
                launch_split_cplx(b_kc, true, (const double2*)(dB + offB[j] * 2), b_kc ? k : nj, nj, k, expB + eoffB[j],
                                  kh, nj_pad, 2 * nj_pad, g.opb == 2, out, sp, grid, cs);
            else
                launch_split(b_kc, dB + offB[j], b_kc ? k : nj, nj, k, expB + eoffB[j], k_pad, nj_pad, out, sp, grid, cs);
        }
        CGB_CUDA(cudaGetLastError());
        return COSMA_GPU_SUCCESS;
    };
    // block b = i NB + j (row-major): its residue bytes go to R[b % NR], which
    // the reconstruction of block b - NR has read by then (same stream)
    auto gemm_block = [&](int b) -> int {
        const int i = b / NB, j = b % NB;
        CGB_CHECK(split_panel(i));
        CGB_CHECK(split_panel(MA + j));
        const int64_t mi_pad = ceil_div(PA.rows(i, m), 2 * BM) * 2 * BM;
        const int64_t nj_pad = ceil_div(PB.rows(j, n), BN) * BN;
        GemmParams gp;
        fill_gemm(gp, N, mi_pad, es * nj_pad, k_pad, w->R[b % NR].ptr, (unsigned*)w->err.ptr);
        return launch_gemm((uint16_t*)w->resA.ptr + roffA[i], (uint16_t*)w->resB.ptr + roffB[j], k_pad, gp, cs);
    };

    // 3. the first NR blocks start while the other panels are on the way,
    // so that the GPU has work until every panel is in and checked; every
    // other panel is scaled as it lands.  A panel's scale kernels are issued
    // once its copy task has run (for pageable memory, once the copy itself
    // is done), so block 0 is launched first and each later block once its
    // panels are in.
    CGB_CHECK(gemm_block(0));
    for (int b = 1; b < NR; ++b) {
        CGB_CHECK(ensure_scaled(b / NB));
        CGB_CHECK(ensure_scaled(MA + b % NB));
        CGB_CHECK(gemm_block(b));
    }
    for (int p : order) CGB_CHECK(ensure_scaled(p));
    cudaEvent_t ev_stats = next_event();
    CGB_CUDA(cudaMemcpyAsync(w->host_stats, sdev, (size_t)NP * sizeof(Stats), cudaMemcpyDeviceToHost, ss));
    CGB_CUDA(cudaEventRecord(ev_stats, ss));
    // every panel's statistics, then the check that the first panels chose
    // the modulus count the whole data gives.  The wait sleeps between polls:
    // a spinning thread would take a core from the host threads that copy
    // pageable panels meanwhile.
    for (;;) {
        const cudaError_t q = cudaEventQuery(ev_stats);
        if (q == cudaSuccess) break;
        if (q != cudaErrorNotReady) CGB_CUDA(q);
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    std::vector<int> all(NP);
    for (int p = 0; p < NP; ++p) all[p] = p;
    const Stats sa = merge_stats(w->host_stats, all);
    if (sa.nonfinite) return abandon();
    Plan full;
    full.spread = (double)sa.spread[0] + (double)sa.spread[1];
    const int exact_bits = std::max(sa.exact_bits[0], sa.exact_bits[1]);
    if (choose(nmod_req, full.spread, es * k, &full.nmod, &full.P, exact_bits) != COSMA_GPU_SUCCESS) {
        clear_error();
        return abandon();
    }
    if (full.nmod != N || full.P != pl.P) return abandon();
    full.exact = full.P >= exact_bits;

    // 4. blocks in order; block b's C leaves on ds while block b+1 computes.
    // From here the call owns C: an error is the caller's, not a fall-back.
    // A pageable C on a host whose page tables the device uses is read and
    // written in place by the reconstruction kernel instead (its stores cross
    // the link; no C slot, C-in or copy-out): the copies of pageable memory
    // from the copy thread go through host threads and the staging buffers,
    // whose rate does not keep up with both operands and C.
    *taken = true;
    const bool c_direct =
        !host_page_locked(C) && prepare_direct_host(C, (size_t)(g.ldc * eb8), (size_t)(m * eb8), (size_t)n, true);
    CombineParams cp0;
    fill_combine(cp0, N, pl.P);
    cudaEvent_t ev_comb[kPipeRing], ev_out[kPipeRing], ev_cin[kPipeRing];
    for (int r = 0; r < NR; ++r) {
        ev_comb[r] = next_event();
        ev_out[r] = next_event();
        ev_cin[r] = next_event();
    }
    bool out_used[kPipeRing] = {};
    uint64_t tk_out[kPipeRing] = {};  // the copy-out of each C slot
    for (int b = 0; b < NBLK; ++b) {
        // blocks 0 .. NR-1 are queued; block b >= NR takes the ring entry of
        // block b - NR, whose reconstruction is ahead of it on the stream
        if (b >= NR) CGB_CHECK(gemm_block(b));
        {
            const int i = b / NB, j = b % NB;
            const int64_t i0 = PA.first(i), mi = PA.rows(i, m), j0 = PB.first(j), nj = PB.rows(j, n);
            const int slot = b % NR;
            double* const chost = C + (i0 + j0 * g.ldc) * es;
            double* cdev = c_direct ? chost : (double*)w->C[slot].ptr;
            if (c_direct) {
                if (!beta_zero) *h2d_bytes += mi * nj * eb8;
            } else if (!beta_zero) {  // the old C block comes in once its slot has been drained
                const uint64_t t = cw.post(copy_task(cdev, mi * eb8, chost, g.ldc * eb8, mi * eb8, nj,
                                                     cudaMemcpyHostToDevice, hs, out_used[slot] ? ev_out[slot] : nullptr,
                                                     ev_cin[slot]));
                *h2d_bytes += mi * nj * eb8;
                CGB_CHECK(cw.wait(t));
                CGB_CUDA(cudaStreamWaitEvent(cs, ev_cin[slot], 0));
            } else if (out_used[slot]) {
                CGB_CHECK(cw.wait(tk_out[slot]));
                CGB_CUDA(cudaStreamWaitEvent(cs, ev_out[slot], 0));
            }
            CombineParams cp = cp0;
            cp.m = mi;
            cp.n = nj;
            cp.ldc = c_direct ? g.ldc : mi;
            const int64_t nj_pad = ceil_div(nj, BN) * BN;
            cp.m_pad = ceil_div(mi, 2 * BM) * 2 * BM;
            cp.nb16 = es * nj_pad / 16;
            cp.n_split = cplx ? nj_pad : INT64_MAX;  // complex: GEMM columns nj_pad.. are Im C
            cp.cs = es;
            cp.R = (const uint8_t*)w->R[slot].ptr;
            cp.expA = expA + eoffA[i];
            cp.expB = expB + eoffB[j];
            cp.C = cdev;
            cp.alpha = g.alpha[0];
            cp.beta = g.beta[0];
            cp.alpha_one = g.alpha[0] == 1.0;
            cp.beta_zero = beta_zero;
            CGB_CHECK(launch_combine(cp, N, cplx ? 2 * nj_pad : nj, cs));
            *d2h_bytes += mi * nj * eb8;
            if (!c_direct) {
                CGB_CUDA(cudaEventRecord(ev_comb[slot], cs));
                tk_out[slot] = cw.post(copy_task(chost, g.ldc * eb8, cdev, mi * eb8, mi * eb8, nj,
                                                 cudaMemcpyDeviceToHost, ds, ev_comb[slot], ev_out[slot]));
                out_used[slot] = true;
            }
        }
    }
    CGB_CHECK(cw.drain());
    for (cudaStream_t s : {cs, hs, ds, ss}) CGB_CUDA(cudaStreamSynchronize(s));
    CGB_CUDA(cudaMemcpy(w->host_err, w->err.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost));
    if (*w->host_err)
        return set_error(COSMA_GPU_ERROR_DEVICE_TIMEOUT,
                         "ozaki2 gemm: a pipeline wait timed out (device code " + std::to_string(*w->host_err) + ")");
    if (info) {
        info->slices = N;
        info->products = N;
        info->fraction_bits = pl.P;
        info->exact_product = full.exact ? 1 : 0;
        info->groups = N * (int)ceil_div(k_pad / BKE, KB_PER_CHUNK);
        info->spread_bits = full.spread;
    }
    return COSMA_GPU_SUCCESS;
}

// The overlapped form with its error exit: whatever fails, nothing is left in
// flight on its streams when it returns.
int gemm_host_pipelined(const GemmDesc& g, int nmod_req, cudaStream_t cs, cudaStream_t hs, cudaStream_t ds,
                         cosma_gpu_ozaki_info* info, int64_t* h2d_bytes, int64_t* d2h_bytes, bool* taken) {
    const int st = gemm_host_pipelined_body(g, nmod_req, cs, hs, ds, info, h2d_bytes, d2h_bytes, taken);
    if (st != COSMA_GPU_SUCCESS) {
        PipeWorkspace* w = pipe_workspace(cs);
        if (w->worker) w->worker->drain();
        for (cudaStream_t s : {cs, hs, ds, w->ss})
            if (s) cudaStreamSynchronize(s);
        cudaGetLastError();
        if (st == COSMA_GPU_ERROR_OUT_OF_MEMORY && !*taken) {
            // the caller runs the regular path next, with its own workspace:
            // this form's buffers go back first
            for (DeviceBuffer* b : {&w->a, &w->b, &w->resA, &w->resB, &w->expA, &w->expB, &w->part}) b->release();
            for (auto& r : w->R) r.release();
            for (auto& c : w->C) c.release();
        }
    }
    return st;
}

}  // namespace oz2

}  // namespace cgb

extern "C" int cosma_gpu_dgemm_ozaki2_residual(char transa, char transb, int64_t m, int64_t n, int64_t k,
                                               const double* A, int64_t lda, const double* B, int64_t ldb,
                                               const double* Ct, int64_t ldt, int moduli, double* E, double* Rx,
                                               int64_t ldo, void* stream, cosma_gpu_ozaki_info* info) {
    using namespace cgb;
    clear_error();
    if (info) *info = cosma_gpu_ozaki_info{0, 0, 0, 0, 0.0, 0.0, 0.0, 0, 0};
    const int opa = parse_op(transa), opb = parse_op(transb);
    if (opa < 0 || opb < 0 || opa == 2 || opb == 2)
        return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "ozaki2 residual: op must be N or T");
    if (m < 1 || n < 1 || k < 1 || k > oz2::KMAX)
        return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "ozaki2 residual: 1 <= m, n and 1 <= k <= 4194240");
    const int64_t a_rows = opa == 0 ? m : k, b_rows = opb == 0 ? k : n;
    if (lda < a_rows || ldb < b_rows || ldt < m || ldo < m || !A || !B || !Ct || !E || !Rx)
        return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "ozaki2 residual: bad pointer or leading dimension");
    if (((uintptr_t)A | (uintptr_t)B | (uintptr_t)Ct | (uintptr_t)E | (uintptr_t)Rx) % 8)
        return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "ozaki2 residual: buffers must be 8-byte aligned");
    double one[2] = {1.0, 0.0}, zero[2] = {0.0, 0.0};
    GemmDesc g = make_gemm_desc(Scalar::D, transa, transb, m, n, k, one, A, lda, B, ldb, zero, E, ldo);
    oz2::Residual r;
    r.Ct = Ct;
    r.ldt = ldt;
    r.E = E;
    r.Rx = Rx;
    r.ldo = ldo;
    return oz2::dgemm(g, moduli, (cudaStream_t)stream, info, &r);
}

extern "C" int cosma_gpu_ozaki2_choose(int64_t k, double spread_bits, int exact_bits, int moduli, int* nmod,
                                       int* fraction_bits) {
    cgb::clear_error();
    if (k < 1 || !nmod || !fraction_bits)
        return cgb::set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "ozaki2_choose: k >= 1 and output pointers needed");
    return cgb::oz2::choose(moduli, spread_bits, k, nmod, fraction_bits, exact_bits > 0 ? exact_bits : (1 << 30));
}

namespace cgb {

void ozaki2_release_stream(cudaStream_t s) {
    oz2::release_workspace(s);
    oz2::release_pipe_workspace(s);
}

int ozaki2_gemm_host(const GemmDesc& g, int moduli, cudaStream_t cs, cudaStream_t hs, cudaStream_t ds,
                      cosma_gpu_ozaki_info* info, int64_t* h2d_bytes, int64_t* d2h_bytes, bool* taken) {
    *taken = false;
    if (((uintptr_t)g.A | (uintptr_t)g.B | (uintptr_t)g.C) % 8) return COSMA_GPU_SUCCESS;
    if (g.m > (int64_t)1 << 24 || g.n > (int64_t)1 << 24) return COSMA_GPU_SUCCESS;
    return oz2::gemm_host_pipelined(g, moduli, cs, hs, ds, info, h2d_bytes, d2h_bytes, taken);
}

int ozaki2_dgemm(const GemmDesc& g, int moduli, cudaStream_t stream, cosma_gpu_ozaki_info* info) {
    if (g.scalar != Scalar::D) return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "ozaki2: double only");
    if (((uintptr_t)g.A | (uintptr_t)g.B | (uintptr_t)g.C) % 8)
        return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "ozaki2: buffers must be 8-byte aligned");
    if (g.m > (int64_t)1 << 24 || g.n > (int64_t)1 << 24)
        return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "ozaki2: m and n are limited to 2^24");
    if (info) *info = cosma_gpu_ozaki_info{0, 0, 0, 0, 0.0, 0.0, 0.0, 0, 0};
    // one pass is exact for k up to KMAX (the split grid's K extent); longer
    // K runs in passes accumulated through C (beta = 1 after the first)
    GemmDesc c = g;
    for (int64_t k0 = 0; k0 < g.k; k0 += oz2::KMAX) {
        c.k = std::min<int64_t>(oz2::KMAX, g.k - k0);
        c.A = (const double*)g.A + (g.opa == 0 ? k0 * g.lda : k0);
        c.B = (const double*)g.B + (g.opb == 0 ? k0 : k0 * g.ldb);
        if (k0 > 0) { c.beta[0] = 1.0; c.beta[1] = 0.0; }
        CGB_CHECK(oz2::dgemm(c, moduli, stream, info));
    }
    return COSMA_GPU_SUCCESS;
}

int ozaki2_zgemm(const GemmDesc& g, int moduli, cudaStream_t stream, cosma_gpu_ozaki_info* info) {
    if (g.scalar != Scalar::Z) return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "ozaki2: complex double only");
    if (((uintptr_t)g.A | (uintptr_t)g.B | (uintptr_t)g.C) % 16)
        return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "ozaki2: complex buffers must be 16-byte aligned");
    if (g.m > (int64_t)1 << 24 || g.n > (int64_t)1 << 23)
        return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "ozaki2: m is limited to 2^24 and n to 2^23 (complex)");
    if (info) *info = cosma_gpu_ozaki_info{0, 0, 0, 0, 0.0, 0.0, 0.0, 0, 0};
    const int64_t kmax = oz2::KMAX / 2;  // each complex term is two real terms
    GemmDesc c = g;
    for (int64_t k0 = 0; k0 < g.k; k0 += kmax) {
        c.k = std::min<int64_t>(kmax, g.k - k0);
        c.A = (const double2*)g.A + (g.opa == 0 ? k0 * g.lda : k0);
        c.B = (const double2*)g.B + (g.opb == 0 ? k0 : k0 * g.ldb);
        if (k0 > 0) { c.beta[0] = 1.0; c.beta[1] = 0.0; }
        CGB_CHECK(oz2::zgemm(c, moduli, stream, info));
    }
    return COSMA_GPU_SUCCESS;
}

}  // namespace cgb
