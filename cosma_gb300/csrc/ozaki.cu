// FP64-accurate GEMM by Ozaki-style splitting on the FP8 tensor cores.
//
// The reference runs a native DGEMM (cuBLAS through Tiled-MM); this is the
// precision form of the same operation, C = alpha*op(A)*op(B) + beta*C.
//
// Method (error-free splitting after Ozaki, Ogita, Oishi & Rump 2012, in the
// integer-slice form of Ootomo, Ozaki & Yokota 2024):
//  1. Row scaling.  Row i of op(A) gets sigma_i = 2^E_i with E_i = 1 +
//     floor(log2 max_l |a_il|), so a'_il = a_il / sigma_i lies in (-1, 1);
//     column j of op(B) likewise (exponent F_j).  The same pass sums
//     2^(floor(log2|a|) - max) per row, a measure of how spread the row's
//     exponents are, used to size the slice count.
//  2. Slicing.  a' is rounded to F = 4 + 5(S-1) fraction bits and written
//     as S balanced digits: a' ~= sum_s d_s 2^(-4-5(s-1)), |d_s| <= 16, the
//     digits of |a'| in balanced base 32 (each in [-16, 15], the leading one
//     in [0, 16]) with the sign applied to all.  Integers up to 16 are exact
//     in FP8 E4M3, so each slice is an E4M3 matrix, stored K-major.
//  3. Slice products.  A_s * B_t is computed exactly on the FP8 tensor cores
//     (tcgen05 kind::f8f6f4): every product of digits is an integer of
//     magnitude <= 256 and the FP32 accumulator holds integers up to 2^24
//     exactly, so up to 65536/k same-weight products share one accumulator.
//     Products with s + t > S + 1 are below the working precision and are
//     skipped (S(S+1)/2 products).
//  4. Recombination.  Each accumulator drain is converted to an integer and
//     added, shifted to its weight, into a 128-bit integer per output; the
//     sum is exact.  One final conversion rounds it to FP64 (round to
//     nearest even) and applies 2^(E_i + F_j).  No FP64 arithmetic is used
//     until then: GB300's FP64 pipe delivers ~1 TFLOP/s, far below the
//     integer and tensor paths.
//
// The integer tensor op (tcgen05 kind::i8) does not exist on sm_103a, and the
// legacy warp-level IMMA path measured 151 TOP/s on GB300 against ~3.5
// PFLOP/s for FP8, so the integer digits ride the FP8 pipe.
//
// GEMM kernels: persistent, warp-specialised; 128-byte-wide K blocks through
// a 4-stage TMA ring (128-byte swizzle), two 256-column FP32 accumulators in
// TMEM so that the epilogue of one accumulator group overlaps the MMAs of the
// next.  Two forms: CTA pairs on 256 x 256 tiles (tcgen05 cta_group::2, 32 KB
// per stage and CTA) whenever m spans two or more 128-row tiles, else single
// CTAs on 128 x 256 tiles (48 KB per stage).  Every CTA loads its own operand
// tiles; no TMA load is multicast.
//   warp 0      TMA producer         warp 1   TMEM owner + MMA issuer
//   warps 2..5  epilogue (TMEM -> registers -> 128-bit integer sums)
#include "common.cuh"
#include "runtime.hpp"
#include "ozaki_common.cuh"
#include "tc_common.cuh"
#include "tma_host.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <map>
#include <mutex>

namespace cgb {
namespace oz {

struct GemmParams {
    int num_m_tiles, num_n_tiles, num_tiles;
    int64_t m, n, ldc;
    // complex results: GEMM columns [0, n_split) are the real parts of C's
    // columns, [n_split, 2*n_split) the imaginary parts; cs = 2 doubles per
    // element.  Real results: n_split beyond every column, cs = 1.
    int64_t n_split;
    int cs;
    double* C;
    const int* expA;
    const int* expB;
    double alpha, beta;
    int beta_zero, alpha_one;
    int L;                 // value = V * 2^(E_i + F_j - L)
    ulonglong2* W;         // per-CTA 128 x 256 128-bit partial sums
    unsigned* err;
    Schedule sched;
};

// Rows whose elements are contiguous along K (op(A) stored transposed, op(B)
// stored as is): one warp per row.
__global__ void scale_kcontig_kernel(const double* __restrict__ X, int64_t ld, int64_t rows, int64_t k,
                                     int* __restrict__ exp_out, Stats* st, int which) {
    const int64_t row = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x & 31;
    if (row >= rows) return;
    // four independent states per lane keep four loads in flight
    RowState q[4] = {{-(1 << 30), 0.0f}, {-(1 << 30), 0.0f}, {-(1 << 30), 0.0f}, {-(1 << 30), 0.0f}};
    unsigned bad = 0;
    const double* p = X + row * ld;
    int64_t l = lane;
    for (; l + 96 < k; l += 128) {
        double x[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) x[u] = p[l + 32 * u];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            int lb, lsb;
            if (element_log2(x[u], &lb, &bad, &lsb)) state_add(q[u], lb, lsb);
        }
    }
    for (; l < k; l += 32) {
        int lb, lsb;
        if (element_log2(p[l], &lb, &bad, &lsb)) state_add(q[0], lb, lsb);
    }
    RowState s = state_merge(state_merge(q[0], q[1]), state_merge(q[2], q[3]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        RowState t;
        t.emax = __shfl_xor_sync(0xffffffffu, s.emax, o);
        t.mass = __shfl_xor_sync(0xffffffffu, s.mass, o);
        t.lsbmin = __shfl_xor_sync(0xffffffffu, s.lsbmin, o);
        s = state_merge(s, t);
    }
    bad = __any_sync(0xffffffffu, bad);
    if (lane == 0) {
        if (bad) atomicOr(&st->nonfinite, 1u);
        finish_row(s, k, exp_out + row, st, which);
    }
}

// Rows contiguous in memory (op(A) stored as is, op(B) stored transposed):
// one thread per row over a chunk of K; partial states combined afterwards.
// es = 2 for complex data viewed as doubles: element (row, l) is the pair
// X[2*row + l*ld], X[2*row + 1 + l*ld] and both parts count.
// pl (nullable) receives each chunk's lowest set-bit weight, for callers
// that need the fraction bits keeping every element exact.
__global__ void scale_mcontig_partial_kernel(const double* __restrict__ X, int64_t ld, int es, int64_t rows,
                                             int64_t k, int64_t kchunk, int* __restrict__ pe,
                                             float* __restrict__ pm, int* __restrict__ pl, Stats* st) {
    const int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= rows) return;
    const int64_t l0 = (int64_t)blockIdx.y * kchunk, l1 = min(k, l0 + kchunk);
    // four independent states keep four loads of the row in flight
    RowState q[4] = {{-(1 << 30), 0.0f}, {-(1 << 30), 0.0f}, {-(1 << 30), 0.0f}, {-(1 << 30), 0.0f}};
    unsigned bad = 0;
    int64_t l = l0;
    for (; l + 3 < l1; l += 4) {
        for (int c = 0; c < es; ++c) {
            double x[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) x[u] = X[row * es + c + (l + u) * ld];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                int lb, lsb;
                if (element_log2(x[u], &lb, &bad, &lsb)) state_add(q[u], lb, lsb);
            }
        }
    }
    for (; l < l1; ++l) {
        for (int c = 0; c < es; ++c) {
            int lb, lsb;
            if (element_log2(X[row * es + c + l * ld], &lb, &bad, &lsb)) state_add(q[0], lb, lsb);
        }
    }
    const RowState s = state_merge(state_merge(q[0], q[1]), state_merge(q[2], q[3]));
    if (bad) atomicOr(&st->nonfinite, 1u);
    pe[blockIdx.y * rows + row] = s.emax;
    pm[blockIdx.y * rows + row] = s.mass;
    if (pl) pl[blockIdx.y * rows + row] = s.lsbmin;
}

__global__ void scale_mcontig_combine_kernel(const int* __restrict__ pe, const float* __restrict__ pm,
                                             const int* __restrict__ pl, int nchunks, int64_t rows, int64_t k,
                                             int* __restrict__ exp_out, Stats* st, int which) {
    const int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= rows) return;
    RowState s{-(1 << 30), 0.0f};
    for (int c = 0; c < nchunks; ++c)
        s = state_merge(s, RowState{pe[c * rows + row], pm[c * rows + row], pl ? pl[c * rows + row] : (1 << 30)});
    finish_row(s, k, exp_out + row, st, which);
}

// One 64-row x 64-column block of the slices per CTA of 256 threads.
template <int S, bool KCONTIG>
__global__ void __launch_bounds__(256) split_kernel(const double* __restrict__ X, int64_t ld, int64_t rows,
                                                    int64_t k, const int* __restrict__ exps, int64_t k_pad,
                                                    int64_t rows_pad, uint8_t* __restrict__ out) {
    split_block<S, KCONTIG>(X, ld, rows, k, exps, k_pad, rows_pad, out, blockIdx.x, blockIdx.y);
}

// Complex operands.  One real GEMM of depth 2*kh gives both parts of C:
//   A_cat row r                 [ Re a | sa*Im a ]
//   B_cat row r                 [ Re b | -sb*Im b ]   -> Re C column r
//   B_cat row half_rows + r     [ sb*Im b | Re b ]    -> Im C column r
// (sa, sb = -1 for a conjugated operand), so that
//   Re c = sum Re a Re b - Im a Im b,  Im c = sum Re a Im b + Im a Re b
// accumulate exactly in the same 128-bit integers as the real case.  Both
// parts of a row share its exponent.  Digits of -x are the negated digits of
// x, so a negation flips the sign bit of every E4M3 byte (zero becomes -0,
// which the MMA adds as 0).  kh is k padded to 64; the row pitch is 2*kh;
// slice s starts at s * slice_rows * 2*kh.  X holds interleaved complex
// doubles, ld in complex elements.
template <int S, bool KCONTIG, bool BSIDE>
__global__ void __launch_bounds__(256) split_cplx_kernel(const double2* __restrict__ X, int64_t ld, int64_t rows,
                                                         int64_t k, const int* __restrict__ exps, int64_t kh,
                                                         int64_t rows_pad, int64_t slice_rows, uint32_t conj_mask,
                                                         uint8_t* __restrict__ out) {
    const int t = threadIdx.x;
    int64_t r;
    int kc;
    if (KCONTIG) { r = (int64_t)blockIdx.x * 64 + t / 4; kc = t % 4; }
    else { r = (int64_t)blockIdx.x * 64 + t % 64; kc = t / 64; }
    const int64_t l0 = (int64_t)blockIdx.y * 64 + kc * 16;
    if (r >= rows_pad || l0 >= kh) return;
    const int E = r < rows ? exps[r] : 0;
    constexpr uint32_t NEG = 0x80808080u;
    const int64_t pitch = 2 * kh;
    const double* Xd = reinterpret_cast<const double*>(X);
    // the real parts, then the imaginary parts (each pass as the real split)
#pragma unroll 1
    for (int part = 0; part < 2; ++part) {
        uint32_t pk[S][4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            int dg[4][S];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int64_t l = l0 + q * 4 + e;
                double x = 0.0;
                if (r < rows && l < k) x = Xd[2 * (KCONTIG ? l + r * ld : r + l * ld) + part];
                digits_of<S>(x, E, dg[e]);
            }
#pragma unroll
            for (int s = 0; s < S; ++s) pk[s][q] = pack4_e4m3(dg[0][s], dg[1][s], dg[2][s], dg[3][s]);
        }
        const uint32_t flip = part ? conj_mask : 0u;  // the sign of a conjugated imaginary part
#pragma unroll
        for (int s = 0; s < S; ++s) {
            uint8_t* base = out + (int64_t)s * slice_rows * pitch;
            const uint4 v = make_uint4(pk[s][0] ^ flip, pk[s][1] ^ flip, pk[s][2] ^ flip, pk[s][3] ^ flip);
            if (!BSIDE) {
                *reinterpret_cast<uint4*>(base + r * pitch + part * kh + l0) = v;
            } else if (part == 0) {  // Re b: first half of row r, second half of row half_rows + r
                *reinterpret_cast<uint4*>(base + r * pitch + l0) = v;
                *reinterpret_cast<uint4*>(base + (rows_pad + r) * pitch + kh + l0) = v;
            } else {  // Im b: negated in row r, as is in row half_rows + r
                const uint4 nv = make_uint4(v.x ^ NEG, v.y ^ NEG, v.z ^ NEG, v.w ^ NEG);
                *reinterpret_cast<uint4*>(base + r * pitch + kh + l0) = nv;
                *reinterpret_cast<uint4*>(base + (rows_pad + r) * pitch + l0) = v;
            }
        }
    }
}

// ------------------------------------------------------------------ GEMM
// Single-CTA form on 128 x 256 tiles, used when m spans fewer than two
// 128-row tiles (or an odd number below ten): each CTA loads its own A and B
// tiles of every K block.
__global__ void __launch_bounds__(THREADS, 1)
    ozaki_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                      const __grid_constant__ GemmParams p) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* full = (uint64_t*)(smem + STAGES * STAGE_BYTES);
    uint64_t* empty = full + STAGES;
    uint64_t* accf = empty + STAGES;
    uint64_t* acce = accf + 2;
    uint64_t* drain = acce + 2;
    uint32_t* tmem_slot = (uint32_t*)(drain + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const Schedule& sc = p.sched;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&accf[b], 1);
            tc::mbar_init(&acce[b], 128);
        }
        tc::mbar_init(drain, 1);
        tc::fence_mbar_init();
        tc::prefetch_tmap(&tmA);
        tc::prefetch_tmap(&tmB);
    }
    if (warp == 1) tc::tmem_alloc(tmem_slot, 512);
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {  // ---------------------------------- TMA producer
            uint32_t it = 0;
            bool ok = true;
            for (int ct = blockIdx.x; ct < p.num_tiles && ok; ct += gridDim.x) {
                int mb, nb;
                tile_coords(ct, p.num_m_tiles, p.num_n_tiles, mb, nb);
                for (int g = 0; g < sc.n_groups && ok; ++g) {
                    for (int kc = 0; kc < sc.kb_count && ok; kc += KB_CHUNK) {  // same order as the MMA issuer
                        const int kc1 = min(sc.kb_count, kc + KB_CHUNK);
                        for (int u = sc.gfirst[g]; u < sc.gfirst[g] + sc.gcount[g] && ok; ++u) {
                            const int arow = sc.us[u] * sc.a_rows_pad + mb * BM;
                            const int brow = sc.ut[u] * sc.b_rows_pad + nb * BN;
                            for (int kb = kc; kb < kc1; ++kb, ++it) {
                                const int st = it % STAGES;
                                if (!tc::mbar_wait(&empty[st], ((it / STAGES) & 1) ^ 1, p.err, kDevTimeoutEmpty)) {
                                    ok = false;
                                    break;
                                }
                                tc::mbar_arrive_expect_tx(&full[st], STAGE_BYTES);
                                uint8_t* sa = smem + st * STAGE_BYTES;
                                tc::tma_load_2d(sa, &tmA, kb * BK, arow, &full[st]);
                                tc::tma_load_2d(sa + A_STAGE, &tmB, kb * BK, brow, &full[st]);
                            }
                        }
                    }
                }
            }
            // let the copies in flight land before the CTA can exit
            const uint32_t first = it > STAGES ? it - STAGES : 0;
            for (uint32_t j = first; j < it; ++j) tc::mbar_wait_drain(&full[j % STAGES], (j / STAGES) & 1);
        }
    } else if (warp == 1) {
        if (lane == 0) {  // ---------------------------------- MMA issuer
            constexpr uint32_t ID = tc::idesc(tc::kFmtE4M3, tc::kFmtE4M3, BM, BN);
            uint32_t it = 0, acc_it = 0;
            bool ok = true;
            for (int ct = blockIdx.x; ct < p.num_tiles && ok; ct += gridDim.x) {
                for (int g = 0; g < sc.n_groups && ok; ++g, ++acc_it) {
                    const uint32_t buf = acc_it & 1;
                    if (!tc::mbar_wait(&acce[buf], ((acc_it >> 1) & 1) ^ 1, p.err, kDevTimeoutAccEmpty)) {
                        ok = false;
                        break;
                    }
                    tc::tc_fence_after();
                    const uint32_t d_tmem = tmem + buf * BN;
                    uint32_t accumulate = 0;
                    // K-chunk-major within the group: every slice product of the group
                    // advances through one 512-wide K chunk before the next chunk, so a
                    // wave of CTAs shares a small, L2-resident set of operand panels
                    // (the integer sum in the accumulator does not depend on the order)
                    for (int kc = 0; kc < sc.kb_count && ok; kc += KB_CHUNK) {
                        const int kc1 = min(sc.kb_count, kc + KB_CHUNK);
                        for (int u = sc.gfirst[g]; u < sc.gfirst[g] + sc.gcount[g] && ok; ++u) {
                            for (int kb = kc; kb < kc1; ++kb, ++it) {
                                const int st = it % STAGES;
                                if (!tc::mbar_wait(&full[st], (it / STAGES) & 1, p.err, kDevTimeoutFull)) {
                                    ok = false;
                                    break;
                                }
                                tc::tc_fence_after();
                                const uint32_t sa = tc::smem_u32(smem + st * STAGE_BYTES);
                                const uint64_t ad = tc::sdesc_k_sw128(sa), bd = tc::sdesc_k_sw128(sa + A_STAGE);
#pragma unroll
                                for (int kk = 0; kk < BK / 32; ++kk) {
                                    tc::mma_f8f6f4(d_tmem, ad + 2 * kk, bd + 2 * kk, ID, accumulate);
                                    accumulate = 1;
                                }
                                tc::mma_commit(&empty[st]);
                            }
                        }
                    }
                    if (ok) tc::mma_commit(&accf[buf]);
                }
            }
            // every MMA must be complete before TMEM is released
            tc::mma_commit(drain);
            tc::mbar_wait_drain(drain, 0);
        }
    } else {  // ------------------------------------------------ epilogue
        const int quad = warp & 3;  // TMEM lanes this warp may access
        ulonglong2* W = p.W + (size_t)blockIdx.x * (BM * BN);
        const uint64_t pol_keep = tc::policy_evict_last(), pol_stream = tc::policy_evict_first();
        uint32_t acc_it = 0;
        for (int ct = blockIdx.x; ct < p.num_tiles; ct += gridDim.x) {
            int mb, nb;
            tile_coords(ct, p.num_m_tiles, p.num_n_tiles, mb, nb);
            if (!epilogue_tile(p, p.sched, mb, nb, tmem, quad, lane, W, accf, acc_it, pol_keep, pol_stream,
                               [&](uint32_t buf) { tc::mbar_arrive(&acce[buf]); }))
                break;
        }
    }
    __syncthreads();
    if (warp == 1) {
        __syncwarp();
        tc::tc_fence_after();
        tc::tmem_dealloc(tmem, 512);
    }
}

// CTA-pair form of the slice-product GEMM, used when m spans two or more
// 128-row tiles.  A cluster of 2 CTAs computes one 256 x 256 output tile with
// tcgen05.mma.cta_group::2 (M = 256 over the pair).  Per K block each CTA
// loads its own 128 rows of the A slab and one half (128 rows) of the B slab:
// 32 KB per stage and SM instead of 48 KB, so operand traffic from L2 falls by
// a third for the same MMA work.  The even CTA issues the MMAs and owns the
// `full` barriers, on which the TMA loads of both CTAs count; its MMA commits
// free the stages and the accumulators of both CTAs.  Each CTA drains the
// accumulator of its own 128 rows, and both epilogues hand an accumulator
// back on the even CTA's `acce` barrier.
//
// Four stages, not the seven that would fit: the operands of a wave of tiles
// are shared through L2 only while the CTAs of the wave stay close together
// in their K stream.  A deeper ring lets each CTA run further ahead, spreads
// the wave's working set past the L2 and multiplies HBM traffic; measured at
// m = n = k = 16384, 4 stages took 275 ms, 5 took 323 ms and 7 took 427 ms
// (DRAM reads 2.9 TB at 7 stages).
constexpr int P_STAGES = 4;
constexpr int P_A = BM * BK, P_B = (BN / 2) * BK, P_STAGE = P_A + P_B;
constexpr int P_SMEM_BYTES = P_STAGES * P_STAGE + 1024 + 256;
static_assert(P_SMEM_BYTES <= 232448, "pair GEMM shared memory");

__global__ void __launch_bounds__(THREADS, 1)
    ozaki_gemm_pair_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                           const __grid_constant__ GemmParams p) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* full = (uint64_t*)(smem + P_STAGES * P_STAGE);
    uint64_t* empty = full + P_STAGES;
    uint64_t* accf = empty + P_STAGES;
    uint64_t* acce = accf + 2;
    uint64_t* drain = acce + 2;
    uint32_t* tmem_slot = (uint32_t*)(drain + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const Schedule& sc = p.sched;
    const int rank = (int)tc::cluster_ctarank();
    const bool leader = rank == 0;
    const int pair = blockIdx.x / 2, npairs = gridDim.x / 2;
    const int num_pm = p.num_m_tiles / 2;  // 256-row tiles

    if (threadIdx.x == 0) {
        for (int s = 0; s < P_STAGES; ++s) {
            tc::mbar_init(&full[s], 1);   // the even CTA's expect_tx (bytes of both CTAs)
            tc::mbar_init(&empty[s], 1);  // one MMA commit per use
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&accf[b], 1);
            tc::mbar_init(&acce[b], 8);  // the 4 epilogue warps of each CTA
        }
        tc::mbar_init(drain, 1);
        tc::fence_mbar_init();
        tc::prefetch_tmap(&tmA);
        tc::prefetch_tmap(&tmB);
    }
    if (warp == 1) tc::tmem_alloc_pair(tmem_slot, 512);
    __syncthreads();
    // the peer's loads and commits reach this CTA's barriers: both CTAs must
    // have initialised them first
    tc::cluster_sync();
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {  // ---------------------------------- TMA producer (both CTAs)
            const uint32_t full0 = tc::mapa_shared(full, 0);  // full[0] of the even CTA
            uint32_t it = 0;
            bool ok = true;
            for (int ct = pair; ct < p.num_tiles && ok; ct += npairs) {
                int mbp, nb;
                tile_coords(ct, num_pm, p.num_n_tiles, mbp, nb, kStripM / 2);
                const int mb = 2 * mbp + rank;
                for (int g = 0; g < sc.n_groups && ok; ++g) {
                    for (int kc = 0; kc < sc.kb_count && ok; kc += KB_CHUNK) {  // same order as the MMA issuer
                        const int kc1 = min(sc.kb_count, kc + KB_CHUNK);
                        for (int u = sc.gfirst[g]; u < sc.gfirst[g] + sc.gcount[g] && ok; ++u) {
                            const int arow = sc.us[u] * sc.a_rows_pad + mb * BM;
                            const int brow = sc.ut[u] * sc.b_rows_pad + nb * BN + rank * (BN / 2);
                            for (int kb = kc; kb < kc1; ++kb, ++it) {
                                const int st = it % P_STAGES;
                                if (!tc::mbar_wait(&empty[st], ((it / P_STAGES) & 1) ^ 1, p.err, kDevTimeoutEmpty)) {
                                    ok = false;
                                    break;
                                }
                                if (leader) tc::mbar_arrive_expect_tx(&full[st], 2 * P_STAGE);
                                uint8_t* sa = smem + st * P_STAGE;
                                tc::tma_load_2d_pair(sa, &tmA, kb * BK, arow, full0 + st * 8);
                                tc::tma_load_2d_pair(sa + P_A, &tmB, kb * BK, brow, full0 + st * 8);
                            }
                        }
                    }
                }
            }
            // the even CTA's last stages count the copies of both CTAs: once they
            // are complete nothing is in flight into either CTA
            if (leader) {
                const uint32_t first = it > P_STAGES ? it - P_STAGES : 0;
                for (uint32_t j = first; j < it; ++j) tc::mbar_wait_drain(&full[j % P_STAGES], (j / P_STAGES) & 1);
            }
        }
    } else if (warp == 1) {
        if (lane == 0 && leader) {  // ------------------------ MMA issuer (even CTA)
            constexpr uint32_t ID = tc::idesc(tc::kFmtE4M3, tc::kFmtE4M3, 2 * BM, BN);
            uint32_t it = 0, acc_it = 0;
            bool ok = true;
            for (int ct = pair; ct < p.num_tiles && ok; ct += npairs) {
                for (int g = 0; g < sc.n_groups && ok; ++g, ++acc_it) {
                    const uint32_t buf = acc_it & 1;
                    if (!tc::mbar_wait_cluster(&acce[buf], ((acc_it >> 1) & 1) ^ 1, p.err, kDevTimeoutAccEmpty)) {
                        ok = false;
                        break;
                    }
                    tc::tc_fence_after();
                    const uint32_t d_tmem = tmem + buf * BN;
                    uint32_t accumulate = 0;
                    for (int kc = 0; kc < sc.kb_count && ok; kc += KB_CHUNK) {
                        const int kc1 = min(sc.kb_count, kc + KB_CHUNK);
                        for (int u = sc.gfirst[g]; u < sc.gfirst[g] + sc.gcount[g] && ok; ++u) {
                            for (int kb = kc; kb < kc1; ++kb, ++it) {
                                const int st = it % P_STAGES;
                                if (!tc::mbar_wait(&full[st], (it / P_STAGES) & 1, p.err, kDevTimeoutFull)) {
                                    ok = false;
                                    break;
                                }
                                tc::tc_fence_after();
                                const uint32_t sa = tc::smem_u32(smem + st * P_STAGE);
                                const uint64_t ad = tc::sdesc_k_sw128(sa), bd = tc::sdesc_k_sw128(sa + P_A);
#pragma unroll
                                for (int kk = 0; kk < BK / 32; ++kk) {
                                    tc::mma_pair_f8f6f4(d_tmem, ad + 2 * kk, bd + 2 * kk, ID, accumulate);
                                    accumulate = 1;
                                }
                                tc::mma_pair_commit_multicast(&empty[st], 3);
                            }
                        }
                    }
                    if (ok) tc::mma_pair_commit_multicast(&accf[buf], 3);
                }
            }
            // every MMA must be complete before either CTA releases its TMEM
            tc::mma_pair_commit_multicast(drain, 1);
            tc::mbar_wait_drain(drain, 0);
        }
    } else {  // ------------------------------------------------ epilogue (both CTAs)
        const int quad = warp & 3;
        ulonglong2* W = p.W + (size_t)blockIdx.x * (BM * BN);
        const uint64_t pol_keep = tc::policy_evict_last(), pol_stream = tc::policy_evict_first();
        const uint32_t acce0 = tc::mapa_shared(acce, 0);
        uint32_t acc_it = 0;
        for (int ct = pair; ct < p.num_tiles; ct += npairs) {
            int mbp, nb;
            tile_coords(ct, num_pm, p.num_n_tiles, mbp, nb, kStripM / 2);
            if (!epilogue_tile(p, p.sched, 2 * mbp + rank, nb, tmem, quad, lane, W, accf, acc_it, pol_keep, pol_stream,
                               [&](uint32_t buf) {
                                   __syncwarp();
                                   if (lane == 0) tc::mbar_arrive_cluster(acce0 + buf * 8);
                               }))
                break;
        }
    }
    __syncthreads();
    // the even CTA's MMAs read this CTA's shared memory and write its TMEM
    tc::cluster_sync();
    if (warp == 1) {
        __syncwarp();
        tc::tc_fence_after();
        tc::tmem_dealloc_pair(tmem, 512);
    }
}

// ------------------------------------------------------------------ host
struct Workspace {
    DeviceBuffer slicesA, slicesB, expA, expB, part, W, stats, err;
    DeviceBuffer T;  // complex alpha/beta: the product before alpha*T + beta*C
    Stats* host_stats = nullptr;
    unsigned* host_err = nullptr;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};  // prep start/end, gemm start/end
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

int num_sms() { return device_sm_count(); }

// Slice count from the requested accuracy and the measured exponent spread.
// The fixed-point width F = 4 + 5(S-1) must reach ~1e-15 elementwise
// relative error against an exactly rounded product.  Calibrated against the
// double-double oracle on u*2^e inputs (u ~ U[-1,1], e ~ U{-phi..phi}): wider
// exponent spreads need more bits (|A||B| falls short of k*sigma_i*sigma_j),
// longer K needs fewer (the truncation errors average out against a C that
// grows with k), and 60 bits are the floor for well-scaled data; 3 bits of
// margin cover the worst-conditioned entries of larger samples.
double required_fraction_bits(double spread_bits, int64_t k) {
    const double lk = std::log2((double)std::max<int64_t>(k, 1));
    return std::max(60.0, 65.0 + 0.85 * (spread_bits - 3.3) - (lk - 8.0));
}

int choose_slices(double spread_bits, int64_t k) {
    const double F = required_fraction_bits(spread_bits, k);
    int S = (int)std::ceil((F - 4.0) / 5.0) + 1;
    return std::min(std::max(S, 2), MAX_SLICES);
}

int build_schedule(int S, int64_t k, int64_t k_pad, int a_rows_pad, int b_rows_pad, Schedule* sc, int* L) {
    std::memset(sc, 0, sizeof(*sc));
    sc->kb_count = (int)(k_pad / BK);
    sc->a_rows_pad = a_rows_pad;
    sc->b_rows_pad = b_rows_pad;
    const int per_group = (int)std::max<int64_t>(1, MAX_K_PER_CALL / std::max<int64_t>(k, 1));
    const int dmax = S + 1;  // 1-based diagonal index s + t of the last kept products
    int nu = 0, ng = 0;
    for (int d = 2; d <= dmax; ++d) {
        const int s_lo = std::max(1, d - S), s_hi = std::min(S, d - 1);
        for (int s0 = s_lo; s0 <= s_hi; s0 += per_group) {
            if (ng >= MAX_GROUPS) return set_error(COSMA_GPU_ERROR_INTERNAL, "ozaki: schedule too long");
            sc->gfirst[ng] = (uint16_t)nu;
            int cnt = 0;
            for (int s = s0; s <= std::min(s_hi, s0 + per_group - 1); ++s) {
                if (nu >= MAX_UNITS) return set_error(COSMA_GPU_ERROR_INTERNAL, "ozaki: schedule too long");
                sc->us[nu] = (uint8_t)(s - 1);
                sc->ut[nu] = (uint8_t)(d - s - 1);
                ++nu;
                ++cnt;
            }
            sc->gcount[ng] = (uint8_t)cnt;
            sc->gshift[ng] = (uint8_t)(5 * (dmax - d));
            ++ng;
        }
    }
    sc->n_groups = ng;
    *L = 8 + 5 * (S - 1);
    return COSMA_GPU_SUCCESS;
}

template <int S>
void launch_split(bool kcontig, const double* X, int64_t ld, int64_t rows, int64_t k, const int* exps, int64_t k_pad,
                  int64_t rows_pad, uint8_t* out, cudaStream_t st) {
    dim3 grid((unsigned)(rows_pad / 64), (unsigned)(k_pad / 64));
    if (kcontig) split_kernel<S, true><<<grid, 256, 0, st>>>(X, ld, rows, k, exps, k_pad, rows_pad, out);
    else split_kernel<S, false><<<grid, 256, 0, st>>>(X, ld, rows, k, exps, k_pad, rows_pad, out);
}

void split(int S, bool kcontig, const double* X, int64_t ld, int64_t rows, int64_t k, const int* exps, int64_t k_pad,
           int64_t rows_pad, uint8_t* out, cudaStream_t st) {
    switch (S) {
#define CGB_SPLIT_CASE(n) case n: launch_split<n>(kcontig, X, ld, rows, k, exps, k_pad, rows_pad, out, st); break;
        CGB_SPLIT_CASE(2) CGB_SPLIT_CASE(3) CGB_SPLIT_CASE(4) CGB_SPLIT_CASE(5) CGB_SPLIT_CASE(6) CGB_SPLIT_CASE(7)
        CGB_SPLIT_CASE(8) CGB_SPLIT_CASE(9) CGB_SPLIT_CASE(10) CGB_SPLIT_CASE(11) CGB_SPLIT_CASE(12)
        CGB_SPLIT_CASE(13) CGB_SPLIT_CASE(14) CGB_SPLIT_CASE(15) CGB_SPLIT_CASE(16)
#undef CGB_SPLIT_CASE
        default: break;
    }
}

// Row scaling of a (rows x k) operand; kcontig as in split_kernel.  es = 2
// for complex operands (ld in complex elements): a row's exponent covers the
// real and imaginary parts, and the spread is measured over 2k terms.
int scale_operand(bool kcontig, const double* X, int64_t ld, int64_t rows, int64_t k, int* exps, DeviceBuffer& part,
                  Stats* st_dev, int which, cudaStream_t st, int es) {
    if (rows == 0) return COSMA_GPU_SUCCESS;
    if (kcontig) {
        // a complex row is 2k consecutive doubles
        scale_kcontig_kernel<<<(unsigned)ceil_div(rows, 8), 256, 0, st>>>(X, ld * es, rows, k * es, exps, st_dev,
                                                                          which);
    } else {
        // enough K chunks for ~16 blocks per SM: each thread walks one row's chunk
        const int64_t row_blocks = ceil_div(rows, 256);
        int nchunks = (int)std::min<int64_t>(std::max<int64_t>(1, (16 * num_sms()) / row_blocks), 64);
        nchunks = (int)std::min<int64_t>(nchunks, std::max<int64_t>(1, k / 64));
        const int64_t kchunk = ceil_div(k, nchunks);
        CGB_CHECK(part.reserve((size_t)nchunks * rows * 12, st));
        int* pe = (int*)part.ptr;
        float* pm = (float*)((char*)part.ptr + (size_t)nchunks * rows * 4);
        int* pl = (int*)((char*)part.ptr + (size_t)nchunks * rows * 8);
        scale_mcontig_partial_kernel<<<dim3((unsigned)row_blocks, (unsigned)nchunks), 256, 0, st>>>(
            X, ld * es, es, rows, k, kchunk, pe, pm, pl, st_dev);
        scale_mcontig_combine_kernel<<<(unsigned)row_blocks, 256, 0, st>>>(pe, pm, pl, nchunks, rows, k * es, exps,
                                                                            st_dev, which);
    }
    CGB_CUDA(cudaGetLastError());
    return COSMA_GPU_SUCCESS;
}

int scale_rows(bool kcontig, const double* X, int64_t ld, int64_t rows, int64_t k, int* exps, Workspace* w,
               Stats* st_dev, int which, cudaStream_t st, int es = 1) {
    return scale_operand(kcontig, X, ld, rows, k, exps, w->part, st_dev, which, st, es);
}

// Which form of the slice-product GEMM runs, and the padded operand extents
// it needs.  The CTA-pair form (256 x 256 tiles) runs whenever m spans two or
// more 128-row tiles and padding m to 256 costs at most ~10% more work; the
// single-CTA form (128 x 256 tiles) takes the rest.
struct GemmShape {
    bool pair;
    int64_t m_pad, n_pad;
};

GemmShape gemm_shape(int64_t m, int64_t n) {
    GemmShape g;
    const int64_t mt = ceil_div(m, BM), nt = ceil_div(n, BN);
    // COSMA_GPU_OZAKI_PAIR=OFF keeps every GEMM on the single-CTA form
    static const bool pairs = env_bool("COSMA_GPU_OZAKI_PAIR", true);
    g.pair = pairs && mt >= 2 && (mt % 2 == 0 || mt >= 10);
    g.m_pad = g.pair ? ceil_div(m, 2 * BM) * 2 * BM : mt * BM;
    g.n_pad = nt * BN;
    return g;
}

template <class Kernel>
int max_active_clusters(Kernel kern, int cl, int smem, int* out) {
    CGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cl * num_sms(), 1, 1);
    cfg.blockDim = dim3(THREADS, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = cl;
    attr.val.clusterDim.y = 1;
    attr.val.clusterDim.z = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    CGB_CUDA(cudaOccupancyMaxActiveClusters(out, kern, &cfg));
    return COSMA_GPU_SUCCESS;
}

// Persistent grid: one CTA per SM (CTA pairs for the pair form), but no more
// than there are tiles.  num_tiles counts 128 x 256 tiles for the single-CTA
// form and 256 x 256 tiles for the pair form.
int gemm_grid(const GemmShape& sh, int num_tiles, int* grid) {
    if (!sh.pair) {
        *grid = std::min(num_tiles, num_sms());
        return COSMA_GPU_SUCCESS;
    }
    static PerDevice<int> pair_clusters;
    int n = 0;
    CGB_CHECK(pair_clusters.get(
        [](int& v) {
            CGB_CHECK(max_active_clusters(ozaki_gemm_pair_kernel, 2, P_SMEM_BYTES, &v));
            v = std::min(v, num_sms() / 2);  // one CTA per SM: never more CTAs than SMs
            if (v < 1) return set_error(COSMA_GPU_ERROR_CUDA, "ozaki: no CTA pair of the slice GEMM fits on the GPU");
            return COSMA_GPU_SUCCESS;
        },
        &n));
    *grid = std::min(num_tiles, n) * 2;
    return COSMA_GPU_SUCCESS;
}

// Fills the tile counts of p for the chosen form.
void set_tiles(const GemmShape& sh, GemmParams& p) {
    p.num_m_tiles = (int)(sh.m_pad / BM);
    p.num_n_tiles = (int)(sh.n_pad / BN);
    p.num_tiles = sh.pair ? (p.num_m_tiles / 2) * p.num_n_tiles : p.num_m_tiles * p.num_n_tiles;
}

// Launches the slice-product GEMM over digit slices laid out [S][rows_pad][k_pad].
int launch_slice_gemm(const GemmShape& sh, int grid, const void* slicesA, const void* slicesB, int S, int64_t k_pad,
                      const GemmParams& p, cudaStream_t st) {
    CUtensorMap tmA, tmB;
    // pairs: each CTA loads its 128 rows of A and half of the B tile
    const int a_box = BM, b_box = sh.pair ? BN / 2 : BN;
    CGB_CHECK(make_tmap_2d(&tmA, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, slicesA, (uint64_t)k_pad,
                           (uint64_t)(S * sh.m_pad), (uint64_t)k_pad, BK, a_box));
    CGB_CHECK(make_tmap_2d(&tmB, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, slicesB, (uint64_t)k_pad,
                           (uint64_t)(S * sh.n_pad), (uint64_t)k_pad, BK, b_box));
    if (sh.pair) {
        CGB_CUDA(cudaFuncSetAttribute(ozaki_gemm_pair_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      P_SMEM_BYTES));
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(grid, 1, 1);
        cfg.blockDim = dim3(THREADS, 1, 1);
        cfg.dynamicSmemBytes = P_SMEM_BYTES;
        cfg.stream = st;
        cudaLaunchAttribute attr;
        attr.id = cudaLaunchAttributeClusterDimension;
        attr.val.clusterDim.x = 2;
        attr.val.clusterDim.y = 1;
        attr.val.clusterDim.z = 1;
        cfg.attrs = &attr;
        cfg.numAttrs = 1;
        CGB_CUDA(cudaLaunchKernelEx(&cfg, ozaki_gemm_pair_kernel, tmA, tmB, p));
        return COSMA_GPU_SUCCESS;
    }
    CGB_CUDA(cudaFuncSetAttribute(ozaki_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
    ozaki_gemm_kernel<<<grid, THREADS, SMEM_BYTES, st>>>(tmA, tmB, p);
    CGB_CUDA(cudaGetLastError());
    return COSMA_GPU_SUCCESS;
}

// One call with k <= MAX_K_PER_CALL.
int ozaki_chunk(const GemmDesc& g, int slices, cudaStream_t st, cosma_gpu_ozaki_info* info) {
    const int64_t m = g.m, n = g.n, k = g.k;
    const bool ta = g.opa != 0, tb = g.opb != 0;
    const double* A = (const double*)g.A;
    const double* B = (const double*)g.B;
    Workspace* w = workspace(st);
    if (!w->host_stats || !w->host_err) return set_error(COSMA_GPU_ERROR_OUT_OF_MEMORY, "ozaki: pinned staging");
    const GemmShape shape = gemm_shape(m, n);
    const int64_t m_pad = shape.m_pad, n_pad = shape.n_pad, k_pad = ceil_div(k, BK) * BK;

    // 1. scaling + spread statistics
    CGB_CHECK(w->stats.reserve(sizeof(Stats), st));
    CGB_CHECK(w->err.reserve(sizeof(unsigned), st));
    CGB_CHECK(w->expA.reserve((size_t)m_pad * 4, st));
    CGB_CHECK(w->expB.reserve((size_t)n_pad * 4, st));
    Stats* st_dev = (Stats*)w->stats.ptr;
    if (!w->ev[0] || !w->ev[3]) return set_error(COSMA_GPU_ERROR_CUDA, "ozaki: timing events");
    CGB_CUDA(cudaEventRecord(w->ev[0], st));
    CGB_CUDA(cudaMemsetAsync(st_dev, 0, sizeof(Stats), st));
    CGB_CUDA(cudaMemsetAsync(w->err.ptr, 0, sizeof(unsigned), st));
    CGB_CUDA(cudaMemsetAsync(w->expA.ptr, 0, (size_t)m_pad * 4, st));
    CGB_CUDA(cudaMemsetAsync(w->expB.ptr, 0, (size_t)n_pad * 4, st));
    // op(A) row i: elements contiguous along K when A is stored transposed
    CGB_CHECK(scale_rows(ta, A, g.lda, m, k, (int*)w->expA.ptr, w, st_dev, 0, st));
    // op(B) column j: contiguous along K when B is stored as is
    CGB_CHECK(scale_rows(!tb, B, g.ldb, n, k, (int*)w->expB.ptr, w, st_dev, 1, st));
    CGB_CUDA(cudaMemcpyAsync(w->host_stats, st_dev, sizeof(Stats), cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaStreamSynchronize(st));
    const Stats hs = *w->host_stats;
    const double spread = (double)hs.spread[0] + (double)hs.spread[1];
    if (hs.nonfinite) {  // Inf/NaN cannot be sliced: the native FP64 kernel propagates them
        if (info) info->fallback_native = 1;
        return native_gemm(g, st);
    }
    const int S = slices > 0 ? std::min(slices, MAX_SLICES) : choose_slices(spread, k);
    if (S < 2) return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "ozaki: at least 2 slices");

    // 2. slices
    CGB_CHECK(w->slicesA.reserve((size_t)S * m_pad * k_pad, st));
    CGB_CHECK(w->slicesB.reserve((size_t)S * n_pad * k_pad, st));
    split(S, ta, A, g.lda, m, k, (const int*)w->expA.ptr, k_pad, m_pad, (uint8_t*)w->slicesA.ptr, st);
    split(S, !tb, B, g.ldb, n, k, (const int*)w->expB.ptr, k_pad, n_pad, (uint8_t*)w->slicesB.ptr, st);
    CGB_CUDA(cudaGetLastError());
    CGB_CUDA(cudaEventRecord(w->ev[1], st));

    // 3. slice products + recombination
    GemmParams p;
    std::memset(&p, 0, sizeof(p));
    int L = 0;
    CGB_CHECK(build_schedule(S, k, k_pad, (int)m_pad, (int)n_pad, &p.sched, &L));
    set_tiles(shape, p);
    p.m = m; p.n = n; p.ldc = g.ldc;
    p.n_split = INT64_MAX;
    p.cs = 1;
    p.C = (double*)g.C;
    p.expA = (const int*)w->expA.ptr;
    p.expB = (const int*)w->expB.ptr;
    p.alpha = g.alpha[0];
    p.beta = g.beta[0];
    p.beta_zero = g.beta[0] == 0.0;
    p.alpha_one = g.alpha[0] == 1.0;
    p.L = L;
    int grid = 0;
    CGB_CHECK(gemm_grid(shape, p.num_tiles, &grid));
    CGB_CHECK(w->W.reserve((size_t)grid * BM * BN * sizeof(ulonglong2), st));
    p.W = (ulonglong2*)w->W.ptr;
    p.err = (unsigned*)w->err.ptr;
    CGB_CUDA(cudaEventRecord(w->ev[2], st));
    CGB_CHECK(launch_slice_gemm(shape, grid, w->slicesA.ptr, w->slicesB.ptr, S, k_pad, p, st));
    CGB_CUDA(cudaEventRecord(w->ev[3], st));
    CGB_CUDA(cudaMemcpyAsync(w->host_err, w->err.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaStreamSynchronize(st));
    if (*w->host_err)
        return set_error(COSMA_GPU_ERROR_DEVICE_TIMEOUT,
                         "ozaki gemm: a pipeline wait timed out (device code " + std::to_string(*w->host_err) + ")");
    if (info) {
        int products = 0;
        for (int i = 0; i < p.sched.n_groups; ++i) products += p.sched.gcount[i];
        float prep = 0.f, gemm = 0.f;
        cudaEventElapsedTime(&prep, w->ev[0], w->ev[1]);
        cudaEventElapsedTime(&gemm, w->ev[2], w->ev[3]);
        info->slices = S;
        info->fraction_bits = 4 + 5 * (S - 1);
        info->products = products;
        info->groups = p.sched.n_groups;
        info->spread_bits = spread;
        info->prep_ms += prep;
        info->gemm_ms += gemm;
    }
    return COSMA_GPU_SUCCESS;
}

template <int S>
void launch_split_cplx(bool kcontig, bool bside, const double2* X, int64_t ld, int64_t rows, int64_t k,
                       const int* exps, int64_t kh, int64_t rows_pad, int64_t slice_rows, uint32_t conj_mask,
                       uint8_t* out, cudaStream_t st) {
    dim3 grid((unsigned)(rows_pad / 64), (unsigned)(kh / 64));
#define CGB_SPLITC(KC, BS)                                                                                       \
    split_cplx_kernel<S, KC, BS><<<grid, 256, 0, st>>>(X, ld, rows, k, exps, kh, rows_pad, slice_rows, conj_mask, \
                                                       out)
    if (kcontig) {
        if (bside) CGB_SPLITC(true, true); else CGB_SPLITC(true, false);
    } else {
        if (bside) CGB_SPLITC(false, true); else CGB_SPLITC(false, false);
    }
#undef CGB_SPLITC
}

void split_cplx(int S, bool kcontig, bool bside, const double2* X, int64_t ld, int64_t rows, int64_t k,
                const int* exps, int64_t kh, int64_t rows_pad, int64_t slice_rows, bool conj, uint8_t* out,
                cudaStream_t st) {
    const uint32_t cm = conj ? 0x80808080u : 0u;
    switch (S) {
#define CGB_SPLIT_CASE(n) \
    case n: launch_split_cplx<n>(kcontig, bside, X, ld, rows, k, exps, kh, rows_pad, slice_rows, cm, out, st); break;
        CGB_SPLIT_CASE(2) CGB_SPLIT_CASE(3) CGB_SPLIT_CASE(4) CGB_SPLIT_CASE(5) CGB_SPLIT_CASE(6) CGB_SPLIT_CASE(7)
        CGB_SPLIT_CASE(8) CGB_SPLIT_CASE(9) CGB_SPLIT_CASE(10) CGB_SPLIT_CASE(11) CGB_SPLIT_CASE(12)
        CGB_SPLIT_CASE(13) CGB_SPLIT_CASE(14) CGB_SPLIT_CASE(15) CGB_SPLIT_CASE(16)
#undef CGB_SPLIT_CASE
        default: break;
    }
}

// Shape of the complex form: the GEMM has 2*nh columns (real parts, then
// imaginary parts), nh = n padded to 256, so both halves tile exactly.
GemmShape cplx_shape(int64_t m, int64_t n, int64_t* nh_out) {
    const int64_t nh = ceil_div(n, BN) * BN;
    *nh_out = nh;
    return gemm_shape(m, 2 * nh);
}

// One complex pass with 2k <= MAX_K_PER_CALL: the same pipeline on the
// concatenated real operands (4 real products per complex one, "4M").
int ozaki_zchunk(const GemmDesc& g, int slices, cudaStream_t st, cosma_gpu_ozaki_info* info) {
    const int64_t m = g.m, n = g.n, k = g.k;
    const bool a_kc = g.opa != 0, b_kc = g.opb == 0;
    const double2* A = (const double2*)g.A;
    const double2* B = (const double2*)g.B;
    Workspace* w = workspace(st);
    if (!w->host_stats || !w->host_err) return set_error(COSMA_GPU_ERROR_OUT_OF_MEMORY, "ozaki: pinned staging");
    int64_t nh = 0;
    const GemmShape shape = cplx_shape(m, n, &nh);
    const int64_t m_pad = shape.m_pad, kh = ceil_div(k, 64) * 64, k_pad = 2 * kh;

    // 1. scaling over both parts of every row / column
    CGB_CHECK(w->stats.reserve(sizeof(Stats), st));
    CGB_CHECK(w->err.reserve(sizeof(unsigned), st));
    CGB_CHECK(w->expA.reserve((size_t)m_pad * 4, st));
    CGB_CHECK(w->expB.reserve((size_t)nh * 4, st));
    Stats* st_dev = (Stats*)w->stats.ptr;
    if (!w->ev[0] || !w->ev[3]) return set_error(COSMA_GPU_ERROR_CUDA, "ozaki: timing events");
    CGB_CUDA(cudaEventRecord(w->ev[0], st));
    CGB_CUDA(cudaMemsetAsync(st_dev, 0, sizeof(Stats), st));
    CGB_CUDA(cudaMemsetAsync(w->err.ptr, 0, sizeof(unsigned), st));
    CGB_CUDA(cudaMemsetAsync(w->expA.ptr, 0, (size_t)m_pad * 4, st));
    CGB_CUDA(cudaMemsetAsync(w->expB.ptr, 0, (size_t)nh * 4, st));
    CGB_CHECK(scale_rows(a_kc, (const double*)A, g.lda, m, k, (int*)w->expA.ptr, w, st_dev, 0, st, 2));
    CGB_CHECK(scale_rows(b_kc, (const double*)B, g.ldb, n, k, (int*)w->expB.ptr, w, st_dev, 1, st, 2));
    CGB_CUDA(cudaMemcpyAsync(w->host_stats, st_dev, sizeof(Stats), cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaStreamSynchronize(st));
    const Stats hs = *w->host_stats;
    const double spread = (double)hs.spread[0] + (double)hs.spread[1];
    if (hs.nonfinite) {
        if (info) info->fallback_native = 1;
        return native_gemm(g, st);
    }
    const int S = slices > 0 ? std::min(slices, MAX_SLICES) : choose_slices(spread, 2 * k);
    if (S < 2) return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "ozaki: at least 2 slices");

    // 2. slices of [Re | Im] rows of op(A) and of the two stacked forms of op(B)
    CGB_CHECK(w->slicesA.reserve((size_t)S * m_pad * k_pad, st));
    CGB_CHECK(w->slicesB.reserve((size_t)S * 2 * nh * k_pad, st));
    split_cplx(S, a_kc, false, A, g.lda, m, k, (const int*)w->expA.ptr, kh, m_pad, m_pad, g.opa == 2,
               (uint8_t*)w->slicesA.ptr, st);
    split_cplx(S, b_kc, true, B, g.ldb, n, k, (const int*)w->expB.ptr, kh, nh, 2 * nh, g.opb == 2,
               (uint8_t*)w->slicesB.ptr, st);
    CGB_CUDA(cudaGetLastError());
    CGB_CUDA(cudaEventRecord(w->ev[1], st));

    // 3. slice products; real alpha and beta are applied in the epilogue,
    //    complex ones by alpha*T + beta*C afterwards
    const bool fused = g.alpha[1] == 0.0 && g.beta[1] == 0.0;
    GemmParams p;
    std::memset(&p, 0, sizeof(p));
    int L = 0;
    CGB_CHECK(build_schedule(S, 2 * k, k_pad, (int)m_pad, (int)(2 * nh), &p.sched, &L));
    set_tiles(shape, p);
    p.m = m;
    p.n = n;
    p.n_split = nh;
    p.cs = 2;
    if (fused) {
        p.C = (double*)g.C;
        p.ldc = g.ldc;
        p.alpha = g.alpha[0];
        p.beta = g.beta[0];
    } else {
        CGB_CHECK(w->T.reserve((size_t)m * n * 16, st));
        p.C = (double*)w->T.ptr;
        p.ldc = m;
        p.alpha = 1.0;
        p.beta = 0.0;
    }
    p.beta_zero = p.beta == 0.0;
    p.alpha_one = p.alpha == 1.0;
    p.expA = (const int*)w->expA.ptr;
    p.expB = (const int*)w->expB.ptr;
    p.L = L;
    int grid = 0;
    CGB_CHECK(gemm_grid(shape, p.num_tiles, &grid));
    CGB_CHECK(w->W.reserve((size_t)grid * BM * BN * sizeof(ulonglong2), st));
    p.W = (ulonglong2*)w->W.ptr;
    p.err = (unsigned*)w->err.ptr;
    CGB_CUDA(cudaEventRecord(w->ev[2], st));
    CGB_CHECK(launch_slice_gemm(shape, grid, w->slicesA.ptr, w->slicesB.ptr, S, k_pad, p, st));
    CGB_CUDA(cudaEventRecord(w->ev[3], st));
    CGB_CUDA(cudaMemcpyAsync(w->host_err, w->err.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaStreamSynchronize(st));
    if (*w->host_err)
        return set_error(COSMA_GPU_ERROR_DEVICE_TIMEOUT,
                         "ozaki gemm: a pipeline wait timed out (device code " + std::to_string(*w->host_err) + ")");
    if (!fused) CGB_CHECK(unpack_device(Scalar::Z, m, n, g.alpha, w->T.ptr, m, g.beta, g.C, g.ldc, st));
    if (info) {
        int products = 0;
        for (int i = 0; i < p.sched.n_groups; ++i) products += p.sched.gcount[i];
        float prep = 0.f, gemm = 0.f;
        cudaEventElapsedTime(&prep, w->ev[0], w->ev[1]);
        cudaEventElapsedTime(&gemm, w->ev[2], w->ev[3]);
        info->slices = S;
        info->fraction_bits = 4 + 5 * (S - 1);
        info->products = products;
        info->groups = p.sched.n_groups;
        info->spread_bits = spread;
        info->prep_ms += prep;
        info->gemm_ms += gemm;
    }
    return COSMA_GPU_SUCCESS;
}

}  // namespace oz

void ozaki_release_stream(cudaStream_t s) { oz::release_workspace(s); }

int ozaki_dgemm(const GemmDesc& g, int slices, cudaStream_t stream, cosma_gpu_ozaki_info* info) {
    if (g.scalar != Scalar::D) return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "ozaki: double only");
    if (((uintptr_t)g.A | (uintptr_t)g.B | (uintptr_t)g.C) % 8)
        return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "ozaki: buffers must be 8-byte aligned");
    if (g.m > (int64_t)1 << 24 || g.n > (int64_t)1 << 24)
        return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "ozaki: m and n are limited to 2^24");
    if (info) *info = cosma_gpu_ozaki_info{0, 0, 0, 0, 0.0, 0.0, 0.0, 0, 0};
    // K beyond one exact accumulator pass is cut into chunks accumulated
    // through C (beta = 1 after the first chunk).
    GemmDesc c = g;
    for (int64_t k0 = 0; k0 < g.k; k0 += oz::MAX_K_PER_CALL) {
        c.k = std::min<int64_t>(oz::MAX_K_PER_CALL, g.k - k0);
        c.A = (const double*)g.A + (g.opa == 0 ? k0 * g.lda : k0);
        c.B = (const double*)g.B + (g.opb == 0 ? k0 : k0 * g.ldb);
        if (k0 > 0) { c.beta[0] = 1.0; c.beta[1] = 0.0; }
        // a chunk holding Inf/NaN runs on the native kernel; the others stay split
        CGB_CHECK(oz::ozaki_chunk(c, slices, stream, info));
    }
    return COSMA_GPU_SUCCESS;
}

int ozaki_zgemm(const GemmDesc& g, int slices, cudaStream_t stream, cosma_gpu_ozaki_info* info) {
    if (g.scalar != Scalar::Z) return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "ozaki: complex double only");
    if (((uintptr_t)g.A | (uintptr_t)g.B | (uintptr_t)g.C) % 16)
        return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "ozaki: complex buffers must be 16-byte aligned");
    if (g.m > (int64_t)1 << 24 || g.n > (int64_t)1 << 23)
        return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "ozaki: m is limited to 2^24 and n to 2^23 (complex)");
    if (info) *info = cosma_gpu_ozaki_info{0, 0, 0, 0, 0.0, 0.0, 0.0, 0, 0};
    // each complex term is two real terms: half the real pass length per chunk
    const int64_t kmax = oz::MAX_K_PER_CALL / 2;
    GemmDesc c = g;
    for (int64_t k0 = 0; k0 < g.k; k0 += kmax) {
        c.k = std::min<int64_t>(kmax, g.k - k0);
        c.A = (const double2*)g.A + (g.opa == 0 ? k0 * g.lda : k0);
        c.B = (const double2*)g.B + (g.opb == 0 ? k0 : k0 * g.ldb);
        if (k0 > 0) { c.beta[0] = 1.0; c.beta[1] = 0.0; }
        CGB_CHECK(oz::ozaki_zchunk(c, slices, stream, info));
    }
    return COSMA_GPU_SUCCESS;
}

// ===========================================================================
// Ozaki DGEMM without any allocation.
//
// Who needs it: callers that cannot let a library call cudaMalloc or cudaFree.
// A solver or framework plugin that has handed all device memory to its own
// pool allocator has nothing left for a library to allocate, and code that
// keeps copies and kernels overlapping on several streams cannot afford the
// device-wide synchronisation that cudaMalloc and cudaFree imply.  For them
// the same kernels run with every scratch buffer (exponents, statistics,
// digit slices, partial sums) carved out of one statically sized device
// array, g_noalloc_scratch, which the module keeps on every GPU that loads
// the library until the process exits.
// ===========================================================================
namespace oz {

constexpr size_t kNoAllocScratchBytes = (size_t)COSMA_GPU_OZAKI_NOALLOC_SCRATCH_BYTES;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_addr[kNoAllocMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device, looked up once
// per device with that device current.  In host code the array's name only
// stands for a host-side shadow; a kernel handed it would fault or touch the
// wrong memory, so kernels only ever get the address returned here.
int noalloc_scratch_address(void** out) {
    int dev = 0;
    CGB_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices)
        return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "ozaki no-alloc: device index out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(no-alloc scratch)");
        if (!p) return set_error(COSMA_GPU_ERROR_CUDA, "ozaki no-alloc: null scratch address");
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return COSMA_GPU_SUCCESS;
}

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// K chunks of the row-exponent pass for rows contiguous in memory (the same
// split scale_rows uses, so both entry points pick the same slice count).
inline int mcontig_chunks(int64_t rows, int64_t k) {
    const int64_t row_blocks = ceil_div(rows, 256);
    int nchunks = (int)std::min<int64_t>(std::max<int64_t>(1, (16 * num_sms()) / row_blocks), 64);
    return (int)std::min<int64_t>(nchunks, std::max<int64_t>(1, k / 64));
}

// Byte offsets of the scratch buffers inside g_noalloc_scratch.
struct NoAllocLayout {
    size_t stats, err, expA, expB, part, head;  // slice-count independent part
    size_t slicesA, slicesB, W, total;
};

NoAllocLayout noalloc_layout(int64_t m, int64_t n, int64_t k, int S, bool a_kcontig, bool b_kcontig) {
    const GemmShape shape = gemm_shape(m, n);
    const int64_t m_pad = shape.m_pad, n_pad = shape.n_pad, k_pad = ceil_div(k, BK) * BK;
    NoAllocLayout L;
    size_t off = 0;
    L.stats = off; off += align256(sizeof(Stats));
    L.err = off; off += align256(sizeof(unsigned));
    L.expA = off; off += align256((size_t)m_pad * 4);
    L.expB = off; off += align256((size_t)n_pad * 4);
    size_t part = 0;
    if (!a_kcontig) part = std::max(part, (size_t)mcontig_chunks(m, k) * m * 8);
    if (!b_kcontig) part = std::max(part, (size_t)mcontig_chunks(n, k) * n * 8);
    L.part = off; off += align256(part);
    L.head = off;
    L.slicesA = off; off += align256((size_t)S * m_pad * k_pad);
    L.slicesB = off; off += align256((size_t)S * n_pad * k_pad);
    const int64_t tiles = (m_pad / BM) * (n_pad / BN);
    L.W = off; off += align256((size_t)std::min<int64_t>(tiles, num_sms()) * BM * BN * sizeof(ulonglong2));
    L.total = off;
    return L;
}

int too_large(size_t need) {
    return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT,
                     "ozaki no-alloc: the problem needs " + std::to_string(need) + " bytes of scratch, more than the " +
                         std::to_string(kNoAllocScratchBytes) +
                         "-byte static array (use cosma_gpu_dgemm_ozaki_device for larger problems)");
}

// One pass over K (k <= MAX_K_PER_CALL), the no-alloc twin of ozaki_chunk.
int noalloc_chunk(const GemmDesc& g, int slices, cudaStream_t st, cosma_gpu_ozaki_info* info) {
    const int64_t m = g.m, n = g.n, k = g.k;
    const bool ta = g.opa != 0, tb = g.opb != 0;
    const double* A = (const double*)g.A;
    const double* B = (const double*)g.B;
    const GemmShape shape = gemm_shape(m, n);
    const int64_t m_pad = shape.m_pad, n_pad = shape.n_pad, k_pad = ceil_div(k, BK) * BK;
    // Reject before touching the device: the smallest slice count must fit.
    const NoAllocLayout L2 = noalloc_layout(m, n, k, slices > 0 ? std::min(slices, MAX_SLICES) : 2, ta, !tb);
    if (L2.total > kNoAllocScratchBytes) return too_large(L2.total);
    void* base = nullptr;
    CGB_CHECK(noalloc_scratch_address(&base));
    char* sc = (char*)base;
    Stats* st_dev = (Stats*)(sc + L2.stats);
    unsigned* err_dev = (unsigned*)(sc + L2.err);
    int* expA = (int*)(sc + L2.expA);
    int* expB = (int*)(sc + L2.expB);
    char* part = sc + L2.part;

    // 1. scaling + spread statistics; the array keeps the previous call's
    //    contents, so everything read before being written is cleared first.
    CGB_CUDA(cudaMemsetAsync(st_dev, 0, sizeof(Stats), st));
    CGB_CUDA(cudaMemsetAsync(err_dev, 0, sizeof(unsigned), st));
    CGB_CUDA(cudaMemsetAsync(expA, 0, (size_t)m_pad * 4, st));
    CGB_CUDA(cudaMemsetAsync(expB, 0, (size_t)n_pad * 4, st));
    struct Operand { bool kcontig; const double* X; int64_t ld, rows; int* exps; int which; };
    const Operand ops[2] = {{ta, A, g.lda, m, expA, 0}, {!tb, B, g.ldb, n, expB, 1}};
    for (const Operand& o : ops) {
        if (o.rows == 0) continue;
        if (o.kcontig) {
            scale_kcontig_kernel<<<(unsigned)ceil_div(o.rows, 8), 256, 0, st>>>(o.X, o.ld, o.rows, k, o.exps, st_dev,
                                                                                 o.which);
        } else {
            const int64_t row_blocks = ceil_div(o.rows, 256);
            const int nchunks = mcontig_chunks(o.rows, k);
            const int64_t kchunk = ceil_div(k, nchunks);
            int* pe = (int*)part;
            float* pm = (float*)(part + (size_t)nchunks * o.rows * 4);
            scale_mcontig_partial_kernel<<<dim3((unsigned)row_blocks, (unsigned)nchunks), 256, 0, st>>>(
                o.X, o.ld, 1, o.rows, k, kchunk, pe, pm, nullptr, st_dev);
            scale_mcontig_combine_kernel<<<(unsigned)row_blocks, 256, 0, st>>>(pe, pm, nullptr, nchunks, o.rows, k,
                                                                                o.exps, st_dev, o.which);
        }
        CGB_CUDA(cudaGetLastError());
    }
    Stats hs;
    CGB_CUDA(cudaMemcpyAsync(&hs, st_dev, sizeof(Stats), cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaStreamSynchronize(st));
    const double spread = (double)hs.spread[0] + (double)hs.spread[1];
    if (hs.nonfinite) {
        if (info) info->fallback_native = 1;
        return native_gemm(g, st);  // the native kernel needs no scratch
    }
    const int S = slices > 0 ? std::min(slices, MAX_SLICES) : choose_slices(spread, k);
    if (S < 2) return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "ozaki: at least 2 slices");
    const NoAllocLayout L = noalloc_layout(m, n, k, S, ta, !tb);
    if (L.total > kNoAllocScratchBytes) return too_large(L.total);

    // 2. slices (every byte, padding included, is rewritten)
    uint8_t* slA = (uint8_t*)(sc + L.slicesA);
    uint8_t* slB = (uint8_t*)(sc + L.slicesB);
    split(S, ta, A, g.lda, m, k, expA, k_pad, m_pad, slA, st);
    split(S, !tb, B, g.ldb, n, k, expB, k_pad, n_pad, slB, st);
    CGB_CUDA(cudaGetLastError());

    // 3. slice products + recombination (the partial sums are written before
    //    they are read in every tile, so they need no clearing)
    GemmParams p;
    std::memset(&p, 0, sizeof(p));
    int Lw = 0;
    CGB_CHECK(build_schedule(S, k, k_pad, (int)m_pad, (int)n_pad, &p.sched, &Lw));
    set_tiles(shape, p);
    p.m = m; p.n = n; p.ldc = g.ldc;
    p.n_split = INT64_MAX;
    p.cs = 1;
    p.C = (double*)g.C;
    p.expA = expA;
    p.expB = expB;
    p.alpha = g.alpha[0];
    p.beta = g.beta[0];
    p.beta_zero = g.beta[0] == 0.0;
    p.alpha_one = g.alpha[0] == 1.0;
    p.L = Lw;
    p.W = (ulonglong2*)(sc + L.W);
    p.err = err_dev;
    int grid = 0;
    CGB_CHECK(gemm_grid(shape, p.num_tiles, &grid));  // <= num_sms(), the CTAs W was sized for
    CGB_CHECK(launch_slice_gemm(shape, grid, slA, slB, S, k_pad, p, st));
    unsigned herr = 0;
    CGB_CUDA(cudaMemcpyAsync(&herr, err_dev, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaStreamSynchronize(st));
    if (herr)
        return set_error(COSMA_GPU_ERROR_DEVICE_TIMEOUT,
                         "ozaki gemm: a pipeline wait timed out (device code " + std::to_string(herr) + ")");
    if (info) {
        int products = 0;
        for (int i = 0; i < p.sched.n_groups; ++i) products += p.sched.gcount[i];
        info->slices = S;
        info->fraction_bits = 4 + 5 * (S - 1);
        info->products = products;
        info->groups = p.sched.n_groups;
        info->spread_bits = spread;
    }
    return COSMA_GPU_SUCCESS;
}

}  // namespace oz
}  // namespace cgb

extern "C" int cosma_gpu_dgemm_ozaki_noalloc(char transa, char transb, int64_t m, int64_t n, int64_t k, double alpha,
                                             const double* A, int64_t lda, const double* B, int64_t ldb, double beta,
                                             double* C, int64_t ldc, int slices, void* stream,
                                             cosma_gpu_ozaki_info* info) {
    using namespace cgb;
    clear_error();
    if (info) *info = cosma_gpu_ozaki_info{0, 0, 0, 0, 0.0, 0.0, 0.0, 0, 0};
    const int opa = parse_op(transa), opb = parse_op(transb);
    if (opa < 0 || opb < 0) return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "ozaki no-alloc: op must be N, T or C");
    if (m < 0 || n < 0 || k < 0) return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "ozaki no-alloc: negative size");
    if (m == 0 || n == 0) return COSMA_GPU_SUCCESS;
    const int64_t a_rows = opa == 0 ? m : k, b_rows = opb == 0 ? k : n;
    if (ldc < std::max<int64_t>(1, m) ||
        (k > 0 && (lda < std::max<int64_t>(1, a_rows) || ldb < std::max<int64_t>(1, b_rows))))
        return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "ozaki no-alloc: leading dimension too small");
    if (((uintptr_t)A | (uintptr_t)B | (uintptr_t)C) % 8)
        return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "ozaki no-alloc: buffers must be 8-byte aligned");
    cudaStream_t st = (cudaStream_t)stream;
    double be[2] = {beta, 0.0};
    if (k == 0 || alpha == 0.0) return scale_matrix_device(Scalar::D, m, n, be, C, ldc, st);
    GemmDesc g;
    g.scalar = Scalar::D;
    g.opa = opa;
    g.opb = opb;
    g.m = m; g.n = n; g.k = k;
    g.alpha[0] = alpha; g.alpha[1] = 0.0;
    g.beta[0] = beta; g.beta[1] = 0.0;
    g.A = A; g.lda = lda; g.B = B; g.ldb = ldb; g.C = C; g.ldc = ldc;
    GemmDesc c = g;
    for (int64_t k0 = 0; k0 < k; k0 += oz::MAX_K_PER_CALL) {
        c.k = std::min<int64_t>(oz::MAX_K_PER_CALL, k - k0);
        c.A = A + (opa == 0 ? k0 * lda : k0);
        c.B = B + (opb == 0 ? k0 : k0 * ldb);
        if (k0 > 0) c.beta[0] = 1.0;
        CGB_CHECK(oz::noalloc_chunk(c, slices, st, info));
    }
    return COSMA_GPU_SUCCESS;
}
