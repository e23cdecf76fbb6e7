// Grouped Chinese-remainder FP64 GEMM: the batching form in the arithmetic of
// ozaki2.cu (Ozaki scheme II on the BF16 tensor cores).
//
// A batch of independent problems C_i = alpha_i op(A_i) op(B_i) + beta_i C_i
// (the reference runs such batches as a loop of local_multiply calls,
// src/cosma/multiply.cpp:476-587) runs as one CUDA graph of five launches
// over all problems at once:
//   1. row scaling of every op(A) row and op(B) column (one launch per memory
//      order), with per-problem statistics: exponent spread, the fraction
//      bits that keep every input bit, Inf/NaN;
//   2. a check of each problem's needed fraction bits against the P it was
//      planned with;
//   3. the residue split of every operand (one launch);
//   4. one persistent GEMM over the 128 x 128 tiles of all problems, each
//      tile running its problem's N modular BF16 products back to back
//      (tcgen05 kind::f16, TMA, accumulators in TMEM) and writing residue
//      bytes;
//   5. the reconstruction of every C entry from its N residues, rounded once.
// One modulus count N serves the batch (the most any problem needs); each
// problem gets the largest P that N admits at its depth k.  A problem whose
// data needs more bits than planned, or holds Inf/NaN, is skipped by steps
// 3-5, its C untouched, and recomputed by the host on the single-problem
// path, so a replay never returns a less accurate result.
//
// Residue matrices are stored without row padding, [t][rows][k_pad]: a tile
// that reaches past a problem's last row reads the next modulus' rows (or
// zeros past the last one, TMA's out-of-bounds fill), which only reach output
// rows / columns beyond m / n, and those are never reconstructed.
#include "common.cuh"
#include "ozaki2_common.cuh"
#include "ozaki_common.cuh"
#include "runtime.hpp"
#include "tc_common.cuh"
#include "tma_host.hpp"

#include <algorithm>
#include <climits>
#include <cstring>
#include <string>
#include <vector>

namespace cgb {
namespace oz2g {

using namespace oz2;
using oz::element_log2;
using oz::finish_row;
using oz::RowState;
using oz::state_add;
using oz::state_merge;
using oz::Stats;

constexpr int GBM = 128, GBN = 128, BKE = 64;  // tile rows, columns; BF16 elements per K block (128 bytes)
constexpr int KB_PER_CHUNK = 16;               // 1024-element K chunk: one exact FP32 accumulation
constexpr int CHUNKS_PER_REDUCE = 64;          // running sums reduced mod p after this many chunks
constexpr int64_t KMAX = 65536;                // deeper problems run on the single-problem path
constexpr int G_STAGES = 6;
constexpr int G_A = GBM * 128, G_B = GBN * 128, G_STAGE = G_A + G_B;
constexpr int G_ACC = 4;  // TMEM accumulators of GBN columns
static_assert(G_ACC * GBN <= 512, "TMEM columns");
constexpr int G_SMEM = G_STAGES * G_STAGE + 1024 + 256;
static_assert(G_SMEM <= 232448, "grouped GEMM shared memory");
constexpr int EPI_WARPS = 16;                 // four per TMEM lane quadrant
constexpr int EPI_GROUPS = EPI_WARPS / 4;     // column groups of a quadrant
constexpr int G_THREADS = 64 + 32 * EPI_WARPS;
constexpr int G_COLS = GBN / EPI_GROUPS;      // columns per epilogue thread
static_assert(G_COLS % 32 == 0, "epilogue TMEM loads of 32 columns");

// Device record of one problem (real data: op C is op T).
struct Prob {
    int m, n, k;
    int P;  // fraction bits; 0: not on the grouped path
    int m_pad, n_pad;  // multiples of the tile (residue output layout)
    int kb_count;      // 64-element K blocks
    int akc, bkc;      // op(A) rows / op(B) columns contiguous along K in memory
    int64_t k_pad;
    const double* A;
    int64_t lda;
    const double* B;
    int64_t ldb;
    double* C;
    int64_t ldc;
    double alpha, beta;
    int alpha_one, beta_zero;
    int* expA;
    int* expB;
    uint16_t* resA;  // [t][m][k_pad]
    uint16_t* resB;  // [t][n][k_pad]
    uint8_t* R;      // [t][n_pad / 16][m_pad][16]
};

// Moduli constants of the GEMM epilogue.
struct ModConst {
    int nmod;
    uint32_t p[MAX_MODULI], magic[MAX_MODULI], bias[MAX_MODULI];  // magic = floor(2^32/p); bias: multiple of p >= 2^30
};

// Items of the prep launches: {problem, operand (0 A, 1 B), block x, block y}.
using Item = int4;

__device__ __forceinline__ void operand_view(const Prob& p, int which, const double*& X, int64_t& ld, int64_t& rows,
                                             int*& exps) {
    if (which == 0) { X = p.A; ld = p.lda; rows = p.m; exps = p.expA; }
    else { X = p.B; ld = p.ldb; rows = p.n; exps = p.expB; }
}

// ---------------------------------------------------------------- scaling
// Rows contiguous along K: one warp per row, 8 rows per item.
__global__ void __launch_bounds__(256) gscale_kcontig_kernel(const Prob* __restrict__ P, const Item* __restrict__ items,
                                                             Stats* __restrict__ stats) {
    const Item it = items[blockIdx.x];
    const Prob& p = P[it.x];
    const double* X;
    int64_t ld, rows;
    int* exps;
    operand_view(p, it.y, X, ld, rows, exps);
    const int64_t row = (int64_t)it.z * 8 + threadIdx.x / 32;
    const int lane = threadIdx.x & 31;
    if (row >= rows) return;
    RowState s{-(1 << 30), 0.0f};
    unsigned bad = 0;
    const double* x = X + row * ld;
    for (int64_t l = lane; l < p.k; l += 32) {
        int lb, lsb;
        if (element_log2(x[l], &lb, &bad, &lsb)) state_add(s, lb, lsb);
    }
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
        if (bad) atomicOr(&stats[it.x].nonfinite, 1u);
        finish_row(s, p.k, exps + row, &stats[it.x], it.y);
    }
}

// Rows contiguous in memory: one thread per row over the whole of K, 256
// rows per item.
__global__ void __launch_bounds__(256) gscale_mcontig_kernel(const Prob* __restrict__ P, const Item* __restrict__ items,
                                                             Stats* __restrict__ stats) {
    const Item it = items[blockIdx.x];
    const Prob& p = P[it.x];
    const double* X;
    int64_t ld, rows;
    int* exps;
    operand_view(p, it.y, X, ld, rows, exps);
    const int64_t row = (int64_t)it.z * 256 + threadIdx.x;
    if (row >= rows) return;
    RowState s{-(1 << 30), 0.0f};
    unsigned bad = 0;
    for (int64_t l = 0; l < p.k; ++l) {
        int lb, lsb;
        if (element_log2(X[row + l * ld], &lb, &bad, &lsb)) state_add(s, lb, lsb);
    }
    if (bad) atomicOr(&stats[it.x].nonfinite, 1u);
    finish_row(s, p.k, exps + row, &stats[it.x], it.y);
}

// Fraction bits a problem needs: the fewer of the accuracy rule's (the rule
// of the single-problem path: max(60, 65 + 0.85 (spread - 3.3) - (log2 k -
// 8)) rounded up, plus `extra`) and those that keep every input bit.
// Evaluated on the device so that planning and checking agree.
__device__ __forceinline__ int need_bits(const Stats& s, int64_t k, int extra) {
    const double spread = (double)s.spread[0] + (double)s.spread[1];
    const double lk = log2((double)(k > 1 ? k : 1));
    const double F = fmax(60.0, 65.0 + 0.85 * (spread - 3.3) - (lk - 8.0));
    const int req = (int)ceil(F) + extra;
    const int ex = max(max(s.exact_bits[0], s.exact_bits[1]), 1);
    return min(req, ex);
}

// need[i]: fraction bits problem i needs (INT_MAX for Inf/NaN); ok[i] = need
// <= planned P; *bad counts the grouped problems that are not ok.
__global__ void gcheck_kernel(const Prob* __restrict__ P, const Stats* __restrict__ stats, int count, int extra,
                              int* __restrict__ need, int* __restrict__ ok, int* __restrict__ bad) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const Prob& p = P[i];
    if (p.P == 0) {  // not on the grouped path
        need[i] = 0;
        ok[i] = 0;
        return;
    }
    const Stats s = stats[i];
    const int nb = s.nonfinite ? INT_MAX : need_bits(s, p.k, extra);
    need[i] = nb;
    const int good = nb <= p.P;
    ok[i] = good;
    if (!good) atomicAdd(bad, 1);
}

// ------------------------------------------------------------------ split
template <int NL, bool NARROW>
__device__ __forceinline__ void gsplit_item(const Prob& p, const Item& it, const SplitParams& sp) {
    if (it.y == 0) {
        if (p.akc) split_block<true, NL, NARROW>(p.A, p.lda, p.m, p.k, p.expA, p.k_pad, p.m, p.resA, sp, p.P, it.z, it.w, true);
        else split_block<false, NL, NARROW>(p.A, p.lda, p.m, p.k, p.expA, p.k_pad, p.m, p.resA, sp, p.P, it.z, it.w, true);
    } else {
        if (p.bkc) split_block<true, NL, NARROW>(p.B, p.ldb, p.n, p.k, p.expB, p.k_pad, p.n, p.resB, sp, p.P, it.z, it.w, true);
        else split_block<false, NL, NARROW>(p.B, p.ldb, p.n, p.k, p.expB, p.k_pad, p.n, p.resB, sp, p.P, it.z, it.w, true);
    }
}

// One block of one problem's operand per CTA; a problem whose P is at most
// 63 takes the 64-bit scaled integers (the branch is uniform over the CTA).
template <int NL>
__global__ void __launch_bounds__(256) gsplit_kernel(const Prob* __restrict__ P, const Item* __restrict__ items,
                                                     const int* __restrict__ ok,
                                                     const __grid_constant__ SplitParams sp) {
    const Item it = items[blockIdx.x];
    if (!ok[it.x]) return;
    const Prob& p = P[it.x];
    if constexpr (NL <= 5) {
        if (p.P <= 63) {
            gsplit_item<NL, true>(p, it, sp);
            return;
        }
    }
    gsplit_item<NL, false>(p, it, sp);
}

// ------------------------------------------------------------------- GEMM
__device__ __forceinline__ void reduce_sums64(int (&s)[G_COLS], uint32_t p, uint32_t magic, uint32_t bias) {
#pragma unroll
    for (int j = 0; j < G_COLS; ++j) s[j] = (int)mod32((uint32_t)s[j] + bias, p, magic);  // s + bias in [0, 2^32)
}

// Persistent modular GEMM over the 128 x 128 tiles of every problem
// ({problem, m block, n block} in `units`, taken round-robin by the CTAs).
// Per tile the roles run the problem's N modular products in turn; per
// product and 1024-wide K chunk one TMEM accumulator (exact in FP32), which
// the epilogue adds into 32-bit running sums and finally reduces mod p_t to
// one residue byte per output.  Tiles of problems that failed the check are
// skipped by all three roles alike.
//   warp 0      TMA producer         warp 1   TMEM owner + MMA issuer
//   warps 2..17 epilogue (TMEM -> registers -> residue bytes), four per TMEM lane quadrant
__global__ void __launch_bounds__(G_THREADS, 1)
    oz2_grouped_gemm_kernel(const Prob* __restrict__ P, const CUtensorMap* __restrict__ maps,
                            const int4* __restrict__ units, int nunits, const int* __restrict__ okf, unsigned* err,
                            const __grid_constant__ ModConst mc) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* full = (uint64_t*)(smem + G_STAGES * G_STAGE);
    uint64_t* empty = full + G_STAGES;
    uint64_t* accf = empty + G_STAGES;
    uint64_t* acce = accf + G_ACC;
    uint64_t* drain = acce + G_ACC;
    uint32_t* tmem_slot = (uint32_t*)(drain + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nmod = mc.nmod;

    if (threadIdx.x == 0) {
        for (int s = 0; s < G_STAGES; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < G_ACC; ++b) {
            tc::mbar_init(&accf[b], 1);
            tc::mbar_init(&acce[b], EPI_WARPS);
        }
        tc::mbar_init(drain, 1);
        tc::fence_mbar_init();
    }
    if (warp == 1) tc::tmem_alloc(tmem_slot, 512);
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {  // ---------------------------------- TMA producer
            uint32_t it = 0;
            bool ok = true;
            for (int u = blockIdx.x; u < nunits && ok; u += gridDim.x) {
                const int4 tl = units[u];
                if (!okf[tl.x]) continue;
                // the tile's parameters in registers: the waits below clobber memory
                const Prob& p = P[tl.x];
                const int kbc = p.kb_count, rows_a = p.m, rows_b = p.n;
                const CUtensorMap* tmA = maps + 2 * tl.x;
                const CUtensorMap* tmB = tmA + 1;
                tc::prefetch_tmap(tmA);
                tc::prefetch_tmap(tmB);
                for (int t = 0; t < nmod && ok; ++t) {
                    const int arow = t * rows_a + tl.y * GBM;
                    const int brow = t * rows_b + tl.z * GBN;
                    for (int kb = 0; kb < kbc; ++kb, ++it) {
                        const int st = it % G_STAGES;
                        if (!tc::mbar_wait(&empty[st], ((it / G_STAGES) & 1) ^ 1, err, kDevTimeoutEmpty)) {
                            ok = false;
                            break;
                        }
                        tc::mbar_arrive_expect_tx(&full[st], G_STAGE);
                        uint8_t* sa = smem + st * G_STAGE;
                        tc::tma_load_2d(sa, tmA, kb * BKE, arow, &full[st]);
                        tc::tma_load_2d(sa + G_A, tmB, kb * BKE, brow, &full[st]);
                    }
                }
            }
            const uint32_t first = it > G_STAGES ? it - G_STAGES : 0;
            for (uint32_t j = first; j < it; ++j) tc::mbar_wait_drain(&full[j % G_STAGES], (j / G_STAGES) & 1);
        }
    } else if (warp == 1) {
        if (lane == 0) {  // ---------------------------------- MMA issuer
            constexpr uint32_t ID = tc::idesc(tc::kFmtBF16, tc::kFmtBF16, GBM, GBN);
            uint32_t it = 0, acc_it = 0;
            bool ok = true;
            for (int u = blockIdx.x; u < nunits && ok; u += gridDim.x) {
                const int4 tl = units[u];
                if (!okf[tl.x]) continue;
                const int kbc = P[tl.x].kb_count;
                const int nchunks = (kbc + KB_PER_CHUNK - 1) / KB_PER_CHUNK;
                for (int t = 0; t < nmod && ok; ++t) {
                    for (int c = 0; c < nchunks && ok; ++c, ++acc_it) {
                        const uint32_t buf = acc_it % G_ACC;
                        if (!tc::mbar_wait(&acce[buf], ((acc_it / G_ACC) & 1) ^ 1, err, kDevTimeoutAccEmpty)) {
                            ok = false;
                            break;
                        }
                        tc::tc_fence_after();
                        const uint32_t d_tmem = tmem + buf * GBN;
                        uint32_t accumulate = 0;
                        const int kb1 = min(kbc, (c + 1) * KB_PER_CHUNK);
                        for (int kb = c * KB_PER_CHUNK; kb < kb1; ++kb, ++it) {
                            const int st = it % G_STAGES;
                            if (!tc::mbar_wait(&full[st], (it / G_STAGES) & 1, err, kDevTimeoutFull)) {
                                ok = false;
                                break;
                            }
                            tc::tc_fence_after();
                            const uint32_t sa = tc::smem_u32(smem + st * G_STAGE);
                            const uint64_t ad = tc::sdesc_k_sw128(sa), bd = tc::sdesc_k_sw128(sa + G_A);
#pragma unroll
                            for (int kk = 0; kk < BKE / 16; ++kk) {  // K = 16 per MMA: 32 bytes
                                tc::mma_f16(d_tmem, ad + 2 * kk, bd + 2 * kk, ID, accumulate);
                                accumulate = 1;
                            }
                            tc::mma_commit(&empty[st]);
                        }
                        if (ok) tc::mma_commit(&accf[buf]);
                    }
                }
            }
            tc::mma_commit(drain);  // every MMA complete before TMEM is released
            tc::mbar_wait_drain(drain, 0);
        }
    } else {  // ------------------------------------------------ epilogue
        const int quad = warp & 3;          // TMEM lanes this warp may access
        const int grp = (warp - 2) >> 2;    // columns [grp * G_COLS, (grp + 1) * G_COLS) of the tile
        const int row = quad * 32 + lane;
        uint32_t acc_it = 0;
        bool ok = true;
        for (int u = blockIdx.x; u < nunits && ok; u += gridDim.x) {
            const int4 tl = units[u];
            if (!okf[tl.x]) continue;
            const Prob& pr = P[tl.x];
            const int kbc = pr.kb_count;
            const int nchunks = (kbc + KB_PER_CHUNK - 1) / KB_PER_CHUNK;
            const int64_t m_pad = pr.m_pad, nb16 = pr.n_pad / 16;
            uint8_t* const R = pr.R;
            const int64_t i = (int64_t)tl.y * GBM + row;
            for (int t = 0; t < nmod && ok; ++t) {
                const uint32_t pm = mc.p[t], mg = mc.magic[t], bias = mc.bias[t];
                int s[G_COLS];
#pragma unroll
                for (int j = 0; j < G_COLS; ++j) s[j] = 0;
                for (int c = 0; c < nchunks; ++c, ++acc_it) {
                    const uint32_t buf = acc_it % G_ACC;
                    // all lanes must agree before the warp-collective TMEM loads
                    if (!__all_sync(0xffffffffu,
                                    tc::mbar_wait(&accf[buf], (acc_it / G_ACC) & 1, err, kDevTimeoutAcc))) {
                        ok = false;
                        break;
                    }
                    tc::tc_fence_after();
                    const uint32_t base = tmem + ((uint32_t)(quad * 32) << 16) + buf * GBN + grp * G_COLS;
#pragma unroll
                    for (int q = 0; q < G_COLS / 32; ++q) {
                        uint32_t v[32];
                        tc::tmem_ld_32x32b_x32(base + q * 32, v);
                        tc::tmem_ld_wait();
#pragma unroll
                        for (int j = 0; j < 32; ++j) s[q * 32 + j] += __float2int_rn(__uint_as_float(v[j]));
                    }
                    tc::tc_fence_before();
                    __syncwarp();
                    if (lane == 0) tc::mbar_arrive(&acce[buf]);
                    if ((c + 1) % CHUNKS_PER_REDUCE == 0) reduce_sums64(s, pm, mg, bias);  // |s| < 2^30 for any K
                }
                if (!ok) break;
                reduce_sums64(s, pm, mg, bias);
                // the G_COLS residues of this thread's row, in groups of 16 columns
#pragma unroll
                for (int g = 0; g < G_COLS / 16; ++g) {
                    uint32_t w[4];
#pragma unroll
                    for (int b = 0; b < 4; ++b) {
                        const int j0 = g * 16 + b * 4;
                        w[b] = (uint32_t)s[j0] | ((uint32_t)s[j0 + 1] << 8) | ((uint32_t)s[j0 + 2] << 16) |
                               ((uint32_t)s[j0 + 3] << 24);
                    }
                    const int64_t jb = (int64_t)tl.z * (GBN / 16) + grp * (G_COLS / 16) + g;
                    *reinterpret_cast<uint4*>(R + (((int64_t)t * nb16 + jb) * m_pad + i) * 16) =
                        make_uint4(w[0], w[1], w[2], w[3]);
                }
            }
        }
    }
    __syncthreads();
    if (warp == 1) {
        __syncwarp();
        tc::tc_fence_after();
        tc::tmem_dealloc(tmem, 512);
    }
}

// --------------------------------------------------------- reconstruction
// Items {problem, row block of 32, column block of 16, 0}; four outputs per
// thread as in ozaki2.cu's combine_kernel: warp g takes columns 16 cb + 4 g
// .. + 3, lane the row 32 rb + lane, and one 32-bit load gives the thread its
// four residues of a modulus.
// SCALE: some problem of the batch has alpha != 1 or beta != 0 (otherwise
// the alpha / beta arithmetic is left out of the instantiation: predicated
// FP64 instructions would occupy GB300's narrow FP64 pipe).
template <int L, bool SCALE>
__global__ void __launch_bounds__(128) gcombine_kernel(const Prob* __restrict__ P, const Item* __restrict__ items,
                                                       const int* __restrict__ ok,
                                                       const __grid_constant__ CrtConst crt) {
    const Item it = items[blockIdx.x];
    if (!ok[it.x]) return;
    const Prob& p = P[it.x];
    const int lane = threadIdx.x & 31, g = threadIdx.x >> 5;
    const int64_t i = (int64_t)it.y * 32 + lane;
    const int64_t j0 = (int64_t)it.z * 16 + 4 * g;
    if (i >= p.m || j0 >= p.n) return;
    const int64_t m_pad = p.m_pad;
    const uint32_t* rp = reinterpret_cast<const uint32_t*>(p.R + ((int64_t)it.z * m_pad + i) * 16) + g;
    const int64_t stride = (int64_t)(p.n_pad / 16) * m_pad * 4;  // 32-bit words per modulus
    unsigned long long acc[4][L];
    crt_accumulate<L>(rp, stride, crt.nmod, crt, acc);
    const int Ei = p.expA[i];
    const int twoP = 2 * p.P;
    const double alpha = p.alpha, beta = p.beta;
    const bool alpha_one = p.alpha_one, beta_zero = p.beta_zero;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const int64_t j = j0 + c;
        if (j >= p.n) break;
        uint32_t x[L];
        const bool neg = reduce_crt<L>(acc[c], x, crt);
        double r = limbs_to_double<L>(x, neg, Ei + p.expB[j] - twoP);
        double* cp = p.C + i + j * p.ldc;
        if constexpr (SCALE) {
            if (!alpha_one) r = __dmul_rn(alpha, r);
            if (!beta_zero) r = __dadd_rn(r, __dmul_rn(beta, *cp));
        }
        *cp = r;
    }
}

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Rows of one operand's residue stack: nmod * rows, at least one TMA box.
inline int64_t stack_rows(int nmod, int rows) { return std::max<int64_t>((int64_t)nmod * rows, GBM); }

}  // namespace oz2g
}  // namespace cgb

using cgb::oz2g::Item;
using cgb::oz2g::Prob;

struct cosma_gpu_oz2_grouped_plan {
    int count = 0;
    int nmod = 0, limbs13 = 5, extra = 16;
    bool scale = false;  // some grouped problem has alpha != 1 or beta != 0
    std::vector<Prob> hp;
    std::vector<cosma_gpu_gemm_problem> orig;  // for the host-side recomputation of skipped problems
    std::vector<int> host_side;                // k == 0 or alpha == 0: C <- beta*C on every run
    std::vector<int> host_crt;                 // k beyond the grouped limit: the single-problem path
    cgb::DeviceBuffer probs, maps, units, kitems, mitems, sitems, citems, stats, need, ok, bad, err, exps, res, R;
    int n_kitems = 0, n_mitems = 0, n_sitems = 0, n_citems = 0;
    std::vector<int4> unit_list;
    int nunits = 0, grid = 0, order = 0;
    int* host_bad = nullptr;
    unsigned* host_err = nullptr;
    double useful = 0, padded = 0, tuned_ms = 0;
    cgb::oz2::SplitParams sp;
    cgb::oz2::CrtConst crt;
    cgb::oz2g::ModConst mc;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t cs = nullptr;
};

namespace cgb {
namespace oz2g {

using Plan = cosma_gpu_oz2_grouped_plan;

template <int NL>
void launch_gsplit_nl(int nitems, const Prob* P, const Item* items, const int* ok, const SplitParams& sp,
                      cudaStream_t st) {
    gsplit_kernel<NL><<<nitems, 256, 0, st>>>(P, items, ok, sp);
}

void launch_gsplit(const Plan* pl, cudaStream_t st) {
    const Prob* P = (const Prob*)pl->probs.ptr;
    const Item* it = (const Item*)pl->sitems.ptr;
    const int* ok = (const int*)pl->ok.ptr;
    switch (pl->limbs13) {  // P <= 64: 5 limbs; <= 77: 6; <= 90: 7; <= 103: 8; else 9
        case 1: case 2: case 3: case 4: case 5: launch_gsplit_nl<5>(pl->n_sitems, P, it, ok, pl->sp, st); break;
        case 6: launch_gsplit_nl<6>(pl->n_sitems, P, it, ok, pl->sp, st); break;
        case 7: launch_gsplit_nl<7>(pl->n_sitems, P, it, ok, pl->sp, st); break;
        case 8: launch_gsplit_nl<8>(pl->n_sitems, P, it, ok, pl->sp, st); break;
        default: launch_gsplit_nl<9>(pl->n_sitems, P, it, ok, pl->sp, st); break;
    }
}

template <bool SCALE>
void launch_gcombine_l(int limbs, unsigned g, const Prob* P, const Item* it, const int* ok, const CrtConst& crt,
                       cudaStream_t st) {
    switch (limbs) {
        case 4: gcombine_kernel<4, SCALE><<<g, 128, 0, st>>>(P, it, ok, crt); break;
        case 5: gcombine_kernel<5, SCALE><<<g, 128, 0, st>>>(P, it, ok, crt); break;
        case 6: gcombine_kernel<6, SCALE><<<g, 128, 0, st>>>(P, it, ok, crt); break;
        case 7: gcombine_kernel<7, SCALE><<<g, 128, 0, st>>>(P, it, ok, crt); break;
        default: gcombine_kernel<8, SCALE><<<g, 128, 0, st>>>(P, it, ok, crt); break;
    }
}

void launch_gcombine(const Plan* pl, cudaStream_t st) {
    const Prob* P = (const Prob*)pl->probs.ptr;
    const Item* it = (const Item*)pl->citems.ptr;
    const int* ok = (const int*)pl->ok.ptr;
    const unsigned g = (unsigned)pl->n_citems;
    if (pl->scale) launch_gcombine_l<true>(limbs_for(pl->nmod), g, P, it, ok, pl->crt, st);
    else launch_gcombine_l<false>(limbs_for(pl->nmod), g, P, it, ok, pl->crt, st);
}

// All launches of one run, in stream order (captured into the plan's graph).
// prep_only: scaling and the check (the planning pass).
int enqueue(Plan* pl, cudaStream_t st, bool prep_only) {
    const int cnt = std::max(pl->count, 1);
    CGB_CUDA(cudaMemsetAsync(pl->stats.ptr, 0, (size_t)cnt * sizeof(Stats), st));
    CGB_CUDA(cudaMemsetAsync(pl->bad.ptr, 0, sizeof(int), st));
    CGB_CUDA(cudaMemsetAsync(pl->err.ptr, 0, sizeof(unsigned), st));
    const Prob* P = (const Prob*)pl->probs.ptr;
    if (pl->n_kitems)
        gscale_kcontig_kernel<<<pl->n_kitems, 256, 0, st>>>(P, (const Item*)pl->kitems.ptr, (Stats*)pl->stats.ptr);
    if (pl->n_mitems)
        gscale_mcontig_kernel<<<pl->n_mitems, 256, 0, st>>>(P, (const Item*)pl->mitems.ptr, (Stats*)pl->stats.ptr);
    gcheck_kernel<<<(unsigned)ceil_div(cnt, 256), 256, 0, st>>>(P, (const Stats*)pl->stats.ptr, pl->count,
                                                                 pl->extra, (int*)pl->need.ptr, (int*)pl->ok.ptr,
                                                                 (int*)pl->bad.ptr);
    CGB_CUDA(cudaGetLastError());
    if (prep_only || pl->nunits == 0) return COSMA_GPU_SUCCESS;
    launch_gsplit(pl, st);
    CGB_CUDA(cudaGetLastError());
    oz2_grouped_gemm_kernel<<<pl->grid, G_THREADS, G_SMEM, st>>>(P, (const CUtensorMap*)pl->maps.ptr,
                                                                  (const int4*)pl->units.ptr, pl->nunits,
                                                                  (const int*)pl->ok.ptr, (unsigned*)pl->err.ptr,
                                                                  pl->mc);
    CGB_CUDA(cudaGetLastError());
    launch_gcombine(pl, st);
    CGB_CUDA(cudaGetLastError());
    return COSMA_GPU_SUCCESS;
}

// Tile order: 0 = deepest K first (problems of equal K together), 1 = the
// order of the batch.
int upload_units(Plan* pl, int order, cudaStream_t st) {
    std::vector<int4> t = pl->unit_list;
    if (order == 0)
        std::stable_sort(t.begin(), t.end(), [&](const int4& a, const int4& b) {
            return pl->hp[a.x].k > pl->hp[b.x].k;
        });
    pl->order = order;
    if (!t.empty())
        CGB_CUDA(cudaMemcpyAsync(pl->units.ptr, t.data(), t.size() * sizeof(int4), cudaMemcpyHostToDevice, st));
    CGB_CUDA(cudaStreamSynchronize(st));
    return COSMA_GPU_SUCCESS;
}

int capture(Plan* pl) {
    if (pl->exec) { cudaGraphExecDestroy(pl->exec); pl->exec = nullptr; }
    if (pl->graph) { cudaGraphDestroy(pl->graph); pl->graph = nullptr; }
    CGB_CUDA(cudaStreamBeginCapture(pl->cs, cudaStreamCaptureModeThreadLocal));
    int s = enqueue(pl, pl->cs, false);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(pl->cs, &g);
    if (s != COSMA_GPU_SUCCESS) { if (g) cudaGraphDestroy(g); return s; }
    if (e != cudaSuccess) return cuda_status(e, "cudaStreamEndCapture");
    pl->graph = g;
    CGB_CUDA(cudaGraphInstantiate(&pl->exec, g, 0));
    return COSMA_GPU_SUCCESS;
}

GemmDesc desc_of(const cosma_gpu_gemm_problem& q) {
    GemmDesc g;
    g.scalar = Scalar::D;
    g.opa = parse_op(q.transa);
    g.opb = parse_op(q.transb);
    g.m = q.m; g.n = q.n; g.k = q.k;
    g.alpha[0] = q.alpha; g.alpha[1] = 0.0;
    g.beta[0] = q.beta; g.beta[1] = 0.0;
    g.A = q.A; g.lda = q.lda; g.B = q.B; g.ldb = q.ldb; g.C = q.C; g.ldc = q.ldc;
    return g;
}

int run(Plan* pl, cudaStream_t st) {
    if (pl->exec) CGB_CUDA(cudaGraphLaunch(pl->exec, st));
    CGB_CUDA(cudaMemcpyAsync(pl->host_bad, pl->bad.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaMemcpyAsync(pl->host_err, pl->err.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaStreamSynchronize(st));
    if (*pl->host_err)
        return set_error(COSMA_GPU_ERROR_DEVICE_TIMEOUT,
                         "grouped ozaki2 gemm: a pipeline wait timed out (device code " +
                             std::to_string(*pl->host_err) + ")");
    for (int i : pl->host_side) CGB_CHECK(gemm_device(desc_of(pl->orig[i]), COSMA_GPU_METHOD_NATIVE, 0, st, nullptr));
    for (int i : pl->host_crt) CGB_CHECK(gemm_device(desc_of(pl->orig[i]), COSMA_GPU_METHOD_OZAKI2, 0, st, nullptr));
    if (*pl->host_bad > 0) {
        // problems whose data outgrew the planned fraction bits, or holding
        // Inf/NaN: their C is untouched; recompute them one by one
        std::vector<int> ok(pl->count);
        CGB_CUDA(cudaMemcpyAsync(ok.data(), pl->ok.ptr, (size_t)pl->count * sizeof(int), cudaMemcpyDeviceToHost, st));
        CGB_CUDA(cudaStreamSynchronize(st));
        for (int i = 0; i < pl->count; ++i)
            if (!ok[i] && pl->hp[i].P > 0)
                CGB_CHECK(gemm_device(desc_of(pl->orig[i]), COSMA_GPU_METHOD_OZAKI2, 0, st, nullptr));
    }
    return COSMA_GPU_SUCCESS;
}

// Times both tile orders on the batch (graph replays) and keeps the faster.
int autotune(Plan* pl, cudaStream_t st) {
    cudaEvent_t e0, e1;
    CGB_CUDA(cudaEventCreate(&e0));
    CGB_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    int best_order = 0;
    for (int order : {0, 1}) {
        CGB_CHECK(upload_units(pl, order, st));
        CGB_CHECK(capture(pl));
        CGB_CUDA(cudaGraphLaunch(pl->exec, st));
        CGB_CUDA(cudaEventRecord(e0, st));
        CGB_CUDA(cudaGraphLaunch(pl->exec, st));
        CGB_CUDA(cudaEventRecord(e1, st));
        CGB_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) { best = ms; best_order = order; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    pl->tuned_ms = best;
    if (best_order != pl->order) {
        CGB_CHECK(upload_units(pl, best_order, st));
        CGB_CHECK(capture(pl));
    }
    return COSMA_GPU_SUCCESS;
}

template <class T>
int upload(DeviceBuffer& buf, const std::vector<T>& v, cudaStream_t st) {
    CGB_CHECK(buf.reserve(std::max<size_t>(v.size(), 1) * sizeof(T), st));
    if (!v.empty()) CGB_CUDA(cudaMemcpyAsync(buf.ptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
    return COSMA_GPU_SUCCESS;
}

int build(Plan* pl, int count, const cosma_gpu_gemm_problem* in, int tune, cudaStream_t st) {
    pl->count = count;
    pl->extra = extra_fraction_bits();
    pl->orig.assign(in, in + count);
    pl->hp.assign(count, Prob{});
    CGB_CUDA(cudaStreamCreateWithFlags(&pl->cs, cudaStreamNonBlocking));
    if (pinned_alloc((void**)&pl->host_bad, sizeof(int)) != cudaSuccess ||
        pinned_alloc((void**)&pl->host_err, sizeof(unsigned)) != cudaSuccess)
        return set_error(COSMA_GPU_ERROR_OUT_OF_MEMORY, "grouped ozaki2: pinned staging");

    // 1. normalise; exponent arena offsets; scaling items
    std::vector<Item> kitems, mitems;
    size_t exp_ints = 0;
    std::vector<size_t> offA(count, 0), offB(count, 0);
    for (int i = 0; i < count; ++i) {
        const cosma_gpu_gemm_problem& q = in[i];
        Prob& p = pl->hp[i];
        const int oa = parse_op(q.transa), ob = parse_op(q.transb);
        if (oa < 0 || ob < 0)
            return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "grouped: problem " + std::to_string(i) + ": bad op");
        if (q.m < 0 || q.n < 0 || q.k < 0)
            return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT,
                             "grouped: problem " + std::to_string(i) + ": negative size");
        p.akc = oa ? 1 : 0;  // real data: C is T
        p.bkc = ob ? 0 : 1;
        p.m = q.m; p.n = q.n; p.k = q.k;
        p.A = q.A; p.lda = q.lda; p.B = q.B; p.ldb = q.ldb; p.C = q.C; p.ldc = q.ldc;
        p.alpha = q.alpha; p.beta = q.beta;
        p.alpha_one = q.alpha == 1.0;
        p.beta_zero = q.beta == 0.0;
        const int64_t ar = oa ? p.k : p.m, br = ob ? p.n : p.k;
        if (p.m > 0 && p.n > 0 &&
            (p.ldc < std::max(1, p.m) || (p.k > 0 && (p.lda < std::max<int64_t>(1, ar) ||
                                                      p.ldb < std::max<int64_t>(1, br)))))
            return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT,
                             "grouped: problem " + std::to_string(i) + ": leading dimension too small");
        if (((uintptr_t)p.A | (uintptr_t)p.B | (uintptr_t)p.C) % 8)
            return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "grouped: buffers must be 8-byte aligned");
        if (p.m == 0 || p.n == 0) continue;  // nothing to do
        if (p.k == 0 || q.alpha == 0.0) {    // C <- beta*C, on the host side of every run
            pl->host_side.push_back(i);
            continue;
        }
        if (p.k > KMAX || (int64_t)MAX_MODULI * std::max(p.m, p.n) >= (1ll << 31)) {
            pl->host_crt.push_back(i);  // deeper products: the single-problem path's K passes; taller
            continue;                   // residue stacks than 32-bit TMA row coordinates reach
        }
        p.P = 116;  // provisional: the planning pass measures what is needed
        p.m_pad = (int)(ceil_div(p.m, GBM) * GBM);
        p.n_pad = (int)(ceil_div(p.n, GBN) * GBN);
        p.k_pad = ceil_div(p.k, BKE) * BKE;
        p.kb_count = (int)(p.k_pad / BKE);
        offA[i] = exp_ints;
        exp_ints += (size_t)p.m_pad;
        offB[i] = exp_ints;
        exp_ints += (size_t)p.n_pad;
        pl->useful += 2.0 * p.m * p.n * p.k;
        auto add = [&](int which, int rows, bool kc) {
            const int per = kc ? 8 : 256;
            for (int z = 0; z * per < rows; ++z) (kc ? kitems : mitems).push_back(make_int4(i, which, z, 0));
        };
        add(0, p.m, p.akc == 1);
        add(1, p.n, p.bkc == 1);
    }
    const size_t cnt = std::max(count, 1);
    CGB_CHECK(pl->exps.reserve(std::max<size_t>(exp_ints, 1) * sizeof(int), st));
    for (int i = 0; i < count; ++i) {
        if (pl->hp[i].P == 0) continue;
        pl->hp[i].expA = (int*)pl->exps.ptr + offA[i];
        pl->hp[i].expB = (int*)pl->exps.ptr + offB[i];
    }
    CGB_CUDA(cudaMemsetAsync(pl->exps.ptr, 0, std::max<size_t>(exp_ints, 1) * sizeof(int), st));
    CGB_CHECK(pl->probs.reserve(cnt * sizeof(Prob), st));
    CGB_CHECK(pl->stats.reserve(cnt * sizeof(Stats), st));
    CGB_CHECK(pl->need.reserve(cnt * sizeof(int), st));
    CGB_CHECK(pl->ok.reserve(cnt * sizeof(int), st));
    CGB_CHECK(pl->bad.reserve(sizeof(int), st));
    CGB_CHECK(pl->err.reserve(sizeof(unsigned), st));
    CGB_CHECK(upload(pl->kitems, kitems, st));
    CGB_CHECK(upload(pl->mitems, mitems, st));
    pl->n_kitems = (int)kitems.size();
    pl->n_mitems = (int)mitems.size();
    CGB_CHECK(upload(pl->probs, pl->hp, st));

    // 2. planning pass: scaling and the check give each problem's needed bits
    pl->nunits = 0;
    CGB_CHECK(enqueue(pl, st, true));
    std::vector<int> need(count);
    if (count)
        CGB_CUDA(cudaMemcpyAsync(need.data(), pl->need.ptr, (size_t)count * sizeof(int), cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaStreamSynchronize(st));

    // 3. one modulus count for the batch, P per problem
    int nmod = 2;
    for (int i = 0; i < count; ++i) {
        const Prob& p = pl->hp[i];
        if (p.P == 0 || need[i] == INT_MAX) continue;  // Inf/NaN: recomputed on every run
        const int t = fewest_moduli(std::max(need[i], 1), p.k);
        if (t <= MAX_MODULI) nmod = std::max(nmod, t);  // beyond: fails the check, single-problem path
    }
    pl->nmod = nmod;
    int maxP = 1;
    for (int i = 0; i < count; ++i) {
        Prob& p = pl->hp[i];
        if (p.P == 0) continue;
        p.P = std::max(1, std::min(max_fraction_bits(nmod, p.k), 116));  // at most nine 13-bit limbs
        maxP = std::max(maxP, p.P);
    }
    pl->limbs13 = (maxP + 1 + 12) / 13;
    fill_split(pl->sp, nmod, maxP);
    fill_crt(pl->crt, nmod);
    std::memset(&pl->mc, 0, sizeof(pl->mc));
    pl->mc.nmod = nmod;
    for (int t = 0; t < nmod; ++t) {
        const uint32_t q = kModuli[t];
        pl->mc.p[t] = q;
        pl->mc.magic[t] = (uint32_t)((1ull << 32) / q);
        pl->mc.bias[t] = (uint32_t)((((1ull << 30) + q - 1) / q) * q);
    }

    // 4. residue and residue-byte arenas, tensor maps, items, tiles
    size_t res_bytes = 0, r_bytes = 0;
    std::vector<size_t> roffA(count, 0), roffB(count, 0), roffR(count, 0);
    for (int i = 0; i < count; ++i) {
        const Prob& p = pl->hp[i];
        if (p.P == 0) continue;
        roffA[i] = res_bytes;
        res_bytes += align256((size_t)stack_rows(nmod, p.m) * p.k_pad * 2);
        roffB[i] = res_bytes;
        res_bytes += align256((size_t)stack_rows(nmod, p.n) * p.k_pad * 2);
        roffR[i] = r_bytes;
        r_bytes += align256((size_t)nmod * p.m_pad * p.n_pad);
    }
    CGB_CHECK(pl->res.reserve(std::max<size_t>(res_bytes, 256), st));
    // rows past m (n) and K padding past k: the split never writes them
    CGB_CUDA(cudaMemsetAsync(pl->res.ptr, 0, std::max<size_t>(res_bytes, 256), st));
    CGB_CHECK(pl->R.reserve(std::max<size_t>(r_bytes, 256), st));
    std::vector<CUtensorMap> maps(2 * cnt);
    std::memset(maps.data(), 0, maps.size() * sizeof(CUtensorMap));
    std::vector<Item> sitems, citems;
    pl->unit_list.clear();
    for (int i = 0; i < count; ++i) {
        Prob& p = pl->hp[i];
        if (p.P == 0) continue;
        p.resA = (uint16_t*)((uint8_t*)pl->res.ptr + roffA[i]);
        p.resB = (uint16_t*)((uint8_t*)pl->res.ptr + roffB[i]);
        p.R = (uint8_t*)pl->R.ptr + roffR[i];
        CGB_CHECK(make_tmap_2d(&maps[2 * i], CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, p.resA, (uint64_t)p.k_pad,
                               (uint64_t)stack_rows(nmod, p.m), (uint64_t)p.k_pad * 2, BKE, GBM));
        CGB_CHECK(make_tmap_2d(&maps[2 * i + 1], CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, p.resB, (uint64_t)p.k_pad,
                               (uint64_t)stack_rows(nmod, p.n), (uint64_t)p.k_pad * 2, BKE, GBN));
        const int kbk = (int)(p.k_pad / 64);
        for (int bx = 0; bx < (int)ceil_div(p.m, 32); ++bx)
            for (int by = 0; by < kbk; ++by) sitems.push_back(make_int4(i, 0, bx, by));
        for (int bx = 0; bx < (int)ceil_div(p.n, 32); ++bx)
            for (int by = 0; by < kbk; ++by) sitems.push_back(make_int4(i, 1, bx, by));
        for (int mb = 0; mb < p.m_pad / GBM; ++mb)
            for (int nb = 0; nb < p.n_pad / GBN; ++nb) pl->unit_list.push_back(make_int4(i, mb, nb, 0));
        for (int cb = 0; cb < (int)ceil_div(p.n, 16); ++cb)
            for (int rb = 0; rb < (int)ceil_div(p.m, 32); ++rb) citems.push_back(make_int4(i, rb, cb, 0));
        pl->padded += 2.0 * nmod * (double)p.m_pad * p.n_pad * p.k_pad;
        pl->scale |= !p.alpha_one || !p.beta_zero;
    }
    if (sitems.size() > 0x7FFFFFFFu || citems.size() > 0x7FFFFFFFu)
        return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "grouped ozaki2: batch too large for one launch");
    CGB_CHECK(upload(pl->sitems, sitems, st));
    CGB_CHECK(upload(pl->citems, citems, st));
    pl->n_sitems = (int)sitems.size();
    pl->n_citems = (int)citems.size();
    CGB_CHECK(upload(pl->maps, maps, st));
    CGB_CHECK(upload(pl->probs, pl->hp, st));
    pl->nunits = (int)pl->unit_list.size();
    CGB_CHECK(pl->units.reserve(std::max<size_t>(pl->unit_list.size(), 1) * sizeof(int4), st));
    pl->grid = std::max(1, std::min(pl->nunits, device_sm_count()));
    CGB_CUDA(cudaFuncSetAttribute(oz2_grouped_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, G_SMEM));
    CGB_CHECK(upload_units(pl, 0, st));
    CGB_CHECK(capture(pl));
    // tuning replays the batch: only when that cannot change C (beta == 0 everywhere)
    bool beta_free = true;
    for (const Prob& p : pl->hp) beta_free &= p.P == 0 || p.beta_zero;
    if (tune && beta_free && pl->nunits > 0) CGB_CHECK(autotune(pl, st));
    return COSMA_GPU_SUCCESS;
}

void destroy(Plan* pl) {
    if (!pl) return;
    if (pl->exec) cudaGraphExecDestroy(pl->exec);
    if (pl->graph) cudaGraphDestroy(pl->graph);
    if (pl->cs) cudaStreamDestroy(pl->cs);
    if (pl->host_bad) cudaFreeHost(pl->host_bad);
    if (pl->host_err) cudaFreeHost(pl->host_err);
    cudaGetLastError();
    delete pl;
}

}  // namespace oz2g

// Entry points used by the grouped plan (grouped.cu).
cosma_gpu_oz2_grouped_plan* oz2_grouped_create(int count, const cosma_gpu_gemm_problem* problems, int autotune,
                                               cudaStream_t st, int* status) {
    auto* pl = new cosma_gpu_oz2_grouped_plan();
    *status = oz2g::build(pl, count, problems, autotune, st);
    if (*status != COSMA_GPU_SUCCESS) {
        oz2g::destroy(pl);
        return nullptr;
    }
    return pl;
}
int oz2_grouped_run(cosma_gpu_oz2_grouped_plan* pl, cudaStream_t st) { return oz2g::run(pl, st); }
void oz2_grouped_destroy(cosma_gpu_oz2_grouped_plan* pl) { oz2g::destroy(pl); }
void oz2_grouped_info(const cosma_gpu_oz2_grouped_plan* pl, cosma_gpu_grouped_info* info) {
    info->tiles = pl->nunits;
    info->tile_policy = 4;  // 128 x 128 BF16 tensor-core tiles, every modulus per tile
    info->dynamic_schedule = 0;
    info->warps_per_cta = oz2g::G_THREADS / 32;
    info->useful_flops = pl->useful;
    info->padded_flops = pl->padded;
    info->tuned_ms = pl->tuned_ms;
}
int oz2_grouped_slices(const cosma_gpu_oz2_grouped_plan* pl, int* out) {
    for (int i = 0; i < pl->count; ++i) out[i] = pl->hp[i].P > 0 ? pl->nmod : 0;
    return COSMA_GPU_SUCCESS;
}
int oz2_grouped_fraction_bits(const cosma_gpu_oz2_grouped_plan* pl, int* out) {
    for (int i = 0; i < pl->count; ++i) out[i] = pl->hp[i].P;
    return COSMA_GPU_SUCCESS;
}

}  // namespace cgb
