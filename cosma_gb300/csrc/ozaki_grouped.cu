// Grouped Ozaki-split FP64 GEMM: the batching form in the precision arithmetic.
//
// A batch of independent problems C_i = alpha_i op(A_i) op(B_i) + beta_i C_i
// (the many uneven local GEMMs a strategy or a caller produces; the reference
// runs them as a loop of local_multiply calls, src/cosma/multiply.cpp:476-587)
// runs as one CUDA graph of a handful of launches over all problems at once:
//   1. row scaling of every op(A) row and op(B) column (one launch per memory
//      order), with per-problem exponent-spread statistics;
//   2. a check that recomputes each problem's slice count from its spread and
//      compares it with the count the plan was built for;
//   3. digit slicing (one launch per slice count and memory order);
//   4. one persistent slice-product GEMM over the 128 x 64 tiles of all
//      problems: the warp-specialised tcgen05 kind::f8f6f4 pipeline of
//      ozaki.cu with the 128-bit partial sums held in TMEM, and a tensor map,
//      schedule and output description per problem.
// A problem whose data needs more slices than planned (or holds Inf/NaN) is
// skipped by steps 3-4, its C untouched, and recomputed by the host on the
// single-problem path, so a replay never returns a less accurate result.
#include "common.cuh"
#include "ozaki_common.cuh"
#include "runtime.hpp"
#include "tc_common.cuh"
#include "tma_host.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace cgb {
namespace ozg {

using namespace oz;

// Device record of one problem (real data: op C is op T).
struct Prob {
    int m, n, k;
    int S;         // planned slice count
    int kb_count;  // K blocks of 128 bytes
    int m_pad, n_pad;
    int sched;     // index into the schedule table
    int L;
    int opa, opb;  // 0 N, 1 T
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
    uint8_t* slA;
    uint8_t* slB;
};


// Items of the prep launches: {problem, operand (0 A, 1 B), block x, block y}.
using Item = int4;

__device__ __forceinline__ void operand_view(const Prob& p, int which, const double*& X, int64_t& ld, int64_t& rows,
                                             int*& exps) {
    if (which == 0) { X = p.A; ld = p.lda; rows = p.m; exps = p.expA; }
    else { X = p.B; ld = p.ldb; rows = p.n; exps = p.expB; }
}

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
        int lb;
        if (element_log2(x[l], &lb, &bad)) state_add(s, lb);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        RowState t;
        t.emax = __shfl_xor_sync(0xffffffffu, s.emax, o);
        t.mass = __shfl_xor_sync(0xffffffffu, s.mass, o);
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
        int lb;
        if (element_log2(X[row + l * ld], &lb, &bad)) state_add(s, lb);
    }
    if (bad) atomicOr(&stats[it.x].nonfinite, 1u);
    finish_row(s, p.k, exps + row, &stats[it.x], it.y);
}

// The slice count a problem needs, from its spread: the rule of
// oz::choose_slices, evaluated on the device so that planning and checking
// use the same arithmetic.
__device__ __forceinline__ int slices_needed(double spread_bits, int64_t k) {
    const double lk = log2((double)(k > 1 ? k : 1));
    const double F = fmax(60.0, 65.0 + 0.85 * (spread_bits - 3.3) - (lk - 8.0));
    const int S = (int)ceil((F - 4.0) / 5.0) + 1;
    return min(max(S, 2), MAX_SLICES);
}

// need[i]: slices problem i needs (MAX_SLICES + 1 for Inf/NaN); ok[i] = need
// <= planned; *bad counts the problems that are not ok.
__global__ void gcheck_kernel(const Prob* __restrict__ P, const Stats* __restrict__ stats, int count,
                              int* __restrict__ need, int* __restrict__ ok, int* __restrict__ bad) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const Prob& p = P[i];
    if (p.S == 0) {  // empty, k == 0 or alpha == 0: handled by the host (C <- beta*C)
        need[i] = 0;
        ok[i] = 0;
        return;
    }
    const Stats s = stats[i];
    const int n = s.nonfinite ? MAX_SLICES + 1 : slices_needed((double)s.spread[0] + (double)s.spread[1], p.k);
    need[i] = n;
    const int good = n <= p.S;
    ok[i] = good;
    if (!good) atomicAdd(bad, 1);
}

template <int S, bool KCONTIG>
__global__ void __launch_bounds__(256) gsplit_kernel(const Prob* __restrict__ P, const Item* __restrict__ items,
                                                     const int* __restrict__ ok) {
    const Item it = items[blockIdx.x];
    if (!ok[it.x]) return;
    const Prob& p = P[it.x];
    if (it.y == 0) split_block<S, KCONTIG>(p.A, p.lda, p.m, p.k, p.expA, p.k_pad, p.m_pad, p.slA, it.z, it.w);
    else split_block<S, KCONTIG>(p.B, p.ldb, p.n, p.k, p.expB, p.k_pad, p.n_pad, p.slB, it.z, it.w);
}

// Tiles of the grouped GEMM: 128 x 64.  Batches hold many small problems,
// for which a 128 x 256 tile wastes work on padding and, above all, spends
// its time draining accumulators into 128-bit partial sums in global memory
// (one drain per accumulator group, ~14 per tile, each a round trip to L2).
// At N = 64 each of the eight epilogue threads of a row owns 32 of the tile's
// columns, and their 128-bit partial sums fit in its registers (128 of them)
// for the whole tile: a drain is two TMEM loads and integer adds, and the
// accumulator goes back to the MMA issuer as soon as it has been read.  TMEM
// holds only accumulators, G_ACC of them, so the issuer can run several
// groups ahead of the drains.
constexpr int GBN = 64;
constexpr int G_ACC = 4;
static_assert(G_ACC * GBN <= 512, "TMEM columns");
// A stage carries three consecutive 128-byte K blocks of one slice product
// (12 MMAs of 128 x 64 x 32): the wait / commit round trip of a stage costs
// ~300 cycles that the MMAs of the stage must cover, and the 4 MMAs of one
// K block (48 cycles each at N = 64) do not.  Layout of a stage: A blocks
// 0..2 | B blocks 0..2, every part 1024-byte aligned.
constexpr int G_STAGES = 3;
constexpr int G_KB_PER_STAGE = 3;
constexpr int G_KB_CHUNK = 6;  // K blocks per chunk of the group loop: two stages
constexpr int G_A = BM * BK, G_B = GBN * BK, G_STAGE = G_KB_PER_STAGE * (G_A + G_B);
constexpr int G_SMEM = G_STAGES * G_STAGE + 1024 + 256;
static_assert(G_SMEM <= 232448, "grouped GEMM shared memory");
// Eight epilogue warps, two per TMEM lane quadrant, each draining 32 of the
// tile's 64 columns.
constexpr int G_EPI_WARPS = 16;                   // four per TMEM lane quadrant
constexpr int G_THREADS = 64 + 32 * G_EPI_WARPS;
constexpr int G_COLS = GBN / (G_EPI_WARPS / 4);  // columns per epilogue thread
static_assert(G_COLS % 16 == 0, "epilogue TMEM loads of 16 columns");

// Drains the accumulator groups of one tile (rows mb*128.., this thread's 32
// columns of nb*64..) into 128-bit partial sums held in registers and, after
// the last group, rounds them to FP64 and writes alpha*r + beta*C.
template <class Release>
__device__ __forceinline__ bool gepilogue_tile(const Prob& p, const Schedule& sc, int mb, int nb, uint32_t tmem,
                                               int quad, int half, int lane, uint64_t* accf, uint32_t& acc_it,
                                               uint64_t pol_stream, unsigned* err, Release release) {
    const int row = quad * 32 + lane;
    const int64_t gi = (int64_t)mb * BM + row;
    const int Ei = p.expA[gi];
    const uint32_t lanes = (uint32_t)(quad * 32) << 16;
    const int last = sc.n_groups - 1;
    // output description in registers (the TMEM accesses clobber memory)
    const int64_t m = p.m, n = p.n, ldc = p.ldc;
    double* const C = p.C;
    const int* const expB = p.expB;
    const int L = p.L;
    const double alpha = p.alpha, beta = p.beta;
    const bool alpha_one = p.alpha_one, beta_zero = p.beta_zero;
    const int c0 = half * G_COLS;
    unsigned long long lo[G_COLS], hi[G_COLS];
#pragma unroll
    for (int j = 0; j < G_COLS; ++j) lo[j] = hi[j] = 0ull;
    for (int g = 0; g <= last; ++g, ++acc_it) {
        const uint32_t buf = acc_it % G_ACC;
        if (!__all_sync(0xffffffffu, tc::mbar_wait(&accf[buf], (acc_it / G_ACC) & 1, err, kDevTimeoutAcc)))
            return false;
        tc::tc_fence_after();
        const int sh = sc.gshift[g];
        uint32_t v[16];
#pragma unroll
        for (int q = 0; q < G_COLS / 16; ++q) {
            tc::tmem_ld_32x32b_x16(tmem + lanes + buf * GBN + c0 + 16 * q, v);
            tc::tmem_ld_wait();
            if (q == G_COLS / 16 - 1) {
                tc::tc_fence_before();
                release(buf);  // the values are in registers: the issuer may reuse the accumulator
            }
#pragma unroll
            for (int j = 0; j < 16; ++j)
                add_shifted(lo[16 * q + j], hi[16 * q + j], __float2int_rn(__uint_as_float(v[j])), sh);
        }
    }
#pragma unroll
    for (int j = 0; j < G_COLS; ++j) {
        const int64_t gj = (int64_t)nb * GBN + c0 + j;
        if (gi < m && gj < n) {
            double r = i128_to_double(lo[j], hi[j], Ei + expB[gj] - L);
            double* cp = C + gi + gj * ldc;
            if (!alpha_one) r = __dmul_rn(alpha, r);
            if (!beta_zero) r = __dadd_rn(r, __dmul_rn(beta, *cp));
            tc::st_f64_hint(cp, r, pol_stream);
        }
    }
    return true;
}

// Persistent slice-product GEMM over the 128 x 64 tiles of every problem
// ({problem, m block, n block} in `tiles`, taken round-robin by the CTAs).
// The roles are those of ozaki_gemm_kernel<1>; per tile they switch to the
// problem's tensor maps (maps[2i], maps[2i+1] in global memory), schedule
// and output description.  Tiles of problems that failed the check are
// skipped by all three roles alike.
__global__ void __launch_bounds__(G_THREADS, 1)
    ozaki_grouped_gemm_kernel(const Prob* __restrict__ P, const CUtensorMap* __restrict__ maps,
                              const Schedule* __restrict__ scheds, const int4* __restrict__ tiles, int ntiles,
                              const int* __restrict__ okf, unsigned* err) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* full = (uint64_t*)(smem + G_STAGES * G_STAGE);
    uint64_t* empty = full + G_STAGES;
    uint64_t* accf = empty + G_STAGES;
    uint64_t* acce = accf + G_ACC;
    uint64_t* drain = acce + G_ACC;
    uint32_t* tmem_slot = (uint32_t*)(drain + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        for (int s = 0; s < G_STAGES; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < G_ACC; ++b) {
            tc::mbar_init(&accf[b], 1);
            tc::mbar_init(&acce[b], 32 * G_EPI_WARPS);
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
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
                const int4 tl = tiles[t];
                if (!okf[tl.x]) continue;
                // the tile's parameters in registers: the waits below clobber
                // memory, and reloading them from global memory on every K
                // block would cost more than the MMAs of a short K block
                const Prob& p = P[tl.x];
                const int kbc = p.kb_count, mpad = p.m_pad, npad = p.n_pad;
                const Schedule* scp = scheds + p.sched;
                const int ng = scp->n_groups;
                const CUtensorMap* tmA = maps + 2 * tl.x;
                const CUtensorMap* tmB = tmA + 1;
                tc::prefetch_tmap(tmA);
                tc::prefetch_tmap(tmB);
                for (int g = 0; g < ng && ok; ++g) {
                    const int u0 = scp->gfirst[g], u1 = u0 + scp->gcount[g];
                    for (int kc = 0; kc < kbc && ok; kc += G_KB_CHUNK) {
                        const int kc1 = min(kbc, kc + G_KB_CHUNK);
                        for (int u = u0; u < u1 && ok; ++u) {
                            const int arow = scp->us[u] * mpad + tl.y * BM;
                            const int brow = scp->ut[u] * npad + tl.z * GBN;
                            for (int kb = kc; kb < kc1; kb += G_KB_PER_STAGE, ++it) {
                                const int st = it % G_STAGES;
                                const int nkb = min(G_KB_PER_STAGE, kc1 - kb);
                                if (!tc::mbar_wait(&empty[st], ((it / G_STAGES) & 1) ^ 1, err, kDevTimeoutEmpty)) {
                                    ok = false;
                                    break;
                                }
                                tc::mbar_arrive_expect_tx(&full[st], nkb * (G_A + G_B));
                                uint8_t* sa = smem + st * G_STAGE;
                                for (int j = 0; j < nkb; ++j) {
                                    tc::tma_load_2d(sa + j * G_A, tmA, (kb + j) * BK, arow, &full[st]);
                                    tc::tma_load_2d(sa + G_KB_PER_STAGE * G_A + j * G_B, tmB, (kb + j) * BK, brow,
                                                    &full[st]);
                                }
                            }
                        }
                    }
                }
            }
            const uint32_t first = it > G_STAGES ? it - G_STAGES : 0;
            for (uint32_t j = first; j < it; ++j) tc::mbar_wait_drain(&full[j % G_STAGES], (j / G_STAGES) & 1);
        }
    } else if (warp == 1) {
        if (lane == 0) {  // ---------------------------------- MMA issuer
            constexpr uint32_t ID = tc::idesc(tc::kFmtE4M3, tc::kFmtE4M3, BM, GBN);
            uint32_t it = 0, acc_it = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
                const int4 tl = tiles[t];
                if (!okf[tl.x]) continue;
                const Prob& p = P[tl.x];
                const int kbc = p.kb_count;
                const Schedule* scp = scheds + p.sched;
                const int ng = scp->n_groups;
                for (int g = 0; g < ng && ok; ++g, ++acc_it) {
                    const int u0 = scp->gfirst[g], u1 = u0 + scp->gcount[g];
                    const uint32_t buf = acc_it % G_ACC;
                    if (!tc::mbar_wait(&acce[buf], ((acc_it / G_ACC) & 1) ^ 1, err, kDevTimeoutAccEmpty)) {
                        ok = false;
                        break;
                    }
                    tc::tc_fence_after();
                    const uint32_t d_tmem = tmem + buf * GBN;
                    uint32_t accumulate = 0;
                    for (int kc = 0; kc < kbc && ok; kc += G_KB_CHUNK) {
                        const int kc1 = min(kbc, kc + G_KB_CHUNK);
                        for (int u = u0; u < u1 && ok; ++u) {
                            for (int kb = kc; kb < kc1; kb += G_KB_PER_STAGE, ++it) {
                                const int st = it % G_STAGES;
                                const int nkb = min(G_KB_PER_STAGE, kc1 - kb);
                                if (!tc::mbar_wait(&full[st], (it / G_STAGES) & 1, err, kDevTimeoutFull)) {
                                    ok = false;
                                    break;
                                }
                                tc::tc_fence_after();
                                const uint32_t sa = tc::smem_u32(smem + st * G_STAGE);
                                for (int j = 0; j < nkb; ++j) {
                                    const uint64_t ad = tc::sdesc_k_sw128(sa + j * G_A);
                                    const uint64_t bd = tc::sdesc_k_sw128(sa + G_KB_PER_STAGE * G_A + j * G_B);
#pragma unroll
                                    for (int kk = 0; kk < BK / 32; ++kk) {
                                        tc::mma_f8f6f4(d_tmem, ad + 2 * kk, bd + 2 * kk, ID, accumulate);
                                        accumulate = 1;
                                    }
                                }
                                tc::mma_commit(&empty[st]);
                            }
                        }
                    }
                    if (ok) tc::mma_commit(&accf[buf]);
                }
            }
            tc::mma_commit(drain);
            tc::mbar_wait_drain(drain, 0);
        }
    } else {  // ------------------------------------------------ epilogue
        const int quad = warp & 3;         // TMEM lanes this warp may access
        const int half = (warp - 2) / 4;  // which G_COLS of the 64 columns
        const uint64_t pol_stream = tc::policy_evict_first();
        uint32_t acc_it = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
            const int4 tl = tiles[t];
            if (!okf[tl.x]) continue;
            const Prob& p = P[tl.x];
            if (!gepilogue_tile(p, scheds[p.sched], tl.y, tl.z, tmem, quad, half, lane, accf, acc_it, pol_stream, err,
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

// ------------------------------------------------------------------ host
template <int S, bool KC>
void launch_gsplit(int nitems, const Prob* P, const Item* items, const int* ok, cudaStream_t st) {
    gsplit_kernel<S, KC><<<nitems, 256, 0, st>>>(P, items, ok);
}

void gsplit(int S, bool kcontig, int nitems, const Prob* P, const Item* items, const int* ok, cudaStream_t st) {
    switch (S) {
#define CGB_GSPLIT(n)                                                                   \
    case n:                                                                             \
        if (kcontig) launch_gsplit<n, true>(nitems, P, items, ok, st);                  \
        else launch_gsplit<n, false>(nitems, P, items, ok, st);                         \
        break;
        CGB_GSPLIT(2) CGB_GSPLIT(3) CGB_GSPLIT(4) CGB_GSPLIT(5) CGB_GSPLIT(6) CGB_GSPLIT(7) CGB_GSPLIT(8)
        CGB_GSPLIT(9) CGB_GSPLIT(10) CGB_GSPLIT(11) CGB_GSPLIT(12) CGB_GSPLIT(13) CGB_GSPLIT(14)
        CGB_GSPLIT(15) CGB_GSPLIT(16)
#undef CGB_GSPLIT
        default: break;
    }
}

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace ozg
}  // namespace cgb

using cgb::ozg::Prob;
using cgb::ozg::Item;

struct cosma_gpu_oz_grouped_plan {
    int count = 0;
    std::vector<Prob> hp;
    std::vector<cosma_gpu_gemm_problem> orig;  // for the host-side recomputation of skipped problems
    std::vector<int> host_side;                // k == 0 or alpha == 0: C <- beta*C on every run
    std::vector<int> host_ozaki;               // k beyond one exact pass: the single-problem path
    cgb::DeviceBuffer probs, maps, scheds, tiles, kitems, mitems, sitems, stats, need, ok, bad, err, exps, slices;
    int n_kitems = 0, n_mitems = 0;
    struct SplitLaunch { int S; bool kcontig; int first, count; };
    std::vector<SplitLaunch> splits;
    std::vector<int4> tile_list;
    int ntiles = 0, grid = 0, order = 0;
    int* host_bad = nullptr;
    unsigned* host_err = nullptr;
    double useful = 0, padded = 0, tuned_ms = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t cs = nullptr;
};

namespace cgb {
namespace ozg {

using Plan = cosma_gpu_oz_grouped_plan;

// All launches of one run, in stream order (captured into the plan's graph).
int enqueue(Plan* pl, cudaStream_t st) {
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
                                                                 (int*)pl->need.ptr, (int*)pl->ok.ptr,
                                                                 (int*)pl->bad.ptr);
    CGB_CUDA(cudaGetLastError());
    for (const auto& sl : pl->splits)
        gsplit(sl.S, sl.kcontig, sl.count, P, (const Item*)pl->sitems.ptr + sl.first, (const int*)pl->ok.ptr, st);
    CGB_CUDA(cudaGetLastError());
    if (pl->ntiles) {
        ozaki_grouped_gemm_kernel<<<pl->grid, G_THREADS, G_SMEM, st>>>(
            P, (const CUtensorMap*)pl->maps.ptr, (const Schedule*)pl->scheds.ptr, (const int4*)pl->tiles.ptr,
            pl->ntiles, (const int*)pl->ok.ptr, (unsigned*)pl->err.ptr);
        CGB_CUDA(cudaGetLastError());
    }
    return COSMA_GPU_SUCCESS;
}

// Tile order: 0 = longest K first (problems of equal K together), 1 = the
// order of the batch.
int upload_tiles(Plan* pl, int order, cudaStream_t st) {
    std::vector<int4> t = pl->tile_list;
    if (order == 0)
        std::stable_sort(t.begin(), t.end(), [&](const int4& a, const int4& b) {
            return pl->hp[a.x].k > pl->hp[b.x].k;
        });
    pl->order = order;
    if (!t.empty())
        CGB_CUDA(cudaMemcpyAsync(pl->tiles.ptr, t.data(), t.size() * sizeof(int4), cudaMemcpyHostToDevice, st));
    CGB_CUDA(cudaStreamSynchronize(st));
    return COSMA_GPU_SUCCESS;
}

int capture(Plan* pl) {
    if (pl->exec) { cudaGraphExecDestroy(pl->exec); pl->exec = nullptr; }
    if (pl->graph) { cudaGraphDestroy(pl->graph); pl->graph = nullptr; }
    CGB_CUDA(cudaStreamBeginCapture(pl->cs, cudaStreamCaptureModeThreadLocal));
    int s = enqueue(pl, pl->cs);
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
                         "grouped ozaki gemm: a pipeline wait timed out (device code " +
                             std::to_string(*pl->host_err) + ")");
    for (int i : pl->host_side) CGB_CHECK(gemm_device(desc_of(pl->orig[i]), COSMA_GPU_METHOD_NATIVE, 0, st, nullptr));
    for (int i : pl->host_ozaki) CGB_CHECK(gemm_device(desc_of(pl->orig[i]), COSMA_GPU_METHOD_OZAKI, 0, st, nullptr));
    if (*pl->host_bad > 0) {
        // problems whose spread outgrew the planned slice count, or holding
        // Inf/NaN: their C is untouched; recompute them one by one
        std::vector<int> ok(pl->count);
        CGB_CUDA(cudaMemcpyAsync(ok.data(), pl->ok.ptr, (size_t)pl->count * sizeof(int), cudaMemcpyDeviceToHost, st));
        CGB_CUDA(cudaStreamSynchronize(st));
        for (int i = 0; i < pl->count; ++i)
            if (!ok[i] && pl->hp[i].S > 0)
                CGB_CHECK(gemm_device(desc_of(pl->orig[i]), COSMA_GPU_METHOD_OZAKI, 0, st, nullptr));
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
        CGB_CHECK(upload_tiles(pl, order, st));
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
        CGB_CHECK(upload_tiles(pl, best_order, st));
        CGB_CHECK(capture(pl));
    }
    return COSMA_GPU_SUCCESS;
}

int build(Plan* pl, int count, const cosma_gpu_gemm_problem* in, int tune, cudaStream_t st) {
    pl->count = count;
    pl->orig.assign(in, in + count);
    pl->hp.assign(count, Prob{});
    CGB_CUDA(cudaStreamCreateWithFlags(&pl->cs, cudaStreamNonBlocking));
    if (pinned_alloc((void**)&pl->host_bad, sizeof(int)) != cudaSuccess ||
        pinned_alloc((void**)&pl->host_err, sizeof(unsigned)) != cudaSuccess)
        return set_error(COSMA_GPU_ERROR_OUT_OF_MEMORY, "grouped ozaki: pinned staging");

    // 1. normalise; exponent arena offsets; scaling items
    std::vector<Item> kitems, mitems;
    size_t exp_ints = 0;
    std::vector<size_t> offA(count, 0), offB(count, 0);
    for (int i = 0; i < count; ++i) {
        const cosma_gpu_gemm_problem& q = in[i];
        Prob& p = pl->hp[i];
        int oa = parse_op(q.transa), ob = parse_op(q.transb);
        if (oa < 0 || ob < 0)
            return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "grouped: problem " + std::to_string(i) + ": bad op");
        if (q.m < 0 || q.n < 0 || q.k < 0)
            return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT,
                             "grouped: problem " + std::to_string(i) + ": negative size");
        p.opa = oa ? 1 : 0;  // real data: C is T
        p.opb = ob ? 1 : 0;
        p.m = q.m; p.n = q.n; p.k = q.k;
        p.A = q.A; p.lda = q.lda; p.B = q.B; p.ldb = q.ldb; p.C = q.C; p.ldc = q.ldc;
        p.alpha = q.alpha; p.beta = q.beta;
        p.alpha_one = q.alpha == 1.0;
        p.beta_zero = q.beta == 0.0;
        const int64_t ar = p.opa ? p.k : p.m, br = p.opb ? p.n : p.k;
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
        if (p.k > MAX_K_PER_CALL) {  // one accumulator pass is exact up to 65536 terms: the
            pl->host_ozaki.push_back(i);  // single-problem path cuts K into exact passes
            continue;
        }
        p.S = MAX_SLICES;  // provisional: the planning pass measures what is needed
        p.m_pad = (int)(ceil_div(p.m, BM) * BM);
        p.n_pad = (int)(ceil_div(p.n, GBN) * GBN);
        p.k_pad = ceil_div(p.k, BK) * BK;
        p.kb_count = (int)(p.k_pad / BK);
        p.L = 8 + 5 * (p.S - 1);
        offA[i] = exp_ints;
        exp_ints += (size_t)p.m_pad;
        offB[i] = exp_ints;
        exp_ints += (size_t)p.n_pad;
        pl->useful += 2.0 * p.m * p.n * p.k;
        // op(A) rows run along K in memory when A is stored transposed; op(B)
        // columns when B is stored as is
        auto add = [&](int which, int rows, bool kc) {
            const int per = kc ? 8 : 256;
            for (int z = 0; z * per < rows; ++z) (kc ? kitems : mitems).push_back(make_int4(i, which, z, 0));
        };
        add(0, p.m, p.opa == 1);
        add(1, p.n, p.opb == 0);
    }
    const size_t cnt = std::max(count, 1);
    CGB_CHECK(pl->exps.reserve(std::max<size_t>(exp_ints, 1) * sizeof(int), st));
    for (int i = 0; i < count; ++i) {
        if (pl->hp[i].S == 0) continue;
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
    CGB_CHECK(pl->kitems.reserve(std::max<size_t>(kitems.size(), 1) * sizeof(Item), st));
    CGB_CHECK(pl->mitems.reserve(std::max<size_t>(mitems.size(), 1) * sizeof(Item), st));
    pl->n_kitems = (int)kitems.size();
    pl->n_mitems = (int)mitems.size();
    if (!kitems.empty())
        CGB_CUDA(cudaMemcpyAsync(pl->kitems.ptr, kitems.data(), kitems.size() * sizeof(Item), cudaMemcpyHostToDevice, st));
    if (!mitems.empty())
        CGB_CUDA(cudaMemcpyAsync(pl->mitems.ptr, mitems.data(), mitems.size() * sizeof(Item), cudaMemcpyHostToDevice, st));
    if (count)
        CGB_CUDA(cudaMemcpyAsync(pl->probs.ptr, pl->hp.data(), (size_t)count * sizeof(Prob), cudaMemcpyHostToDevice, st));

    // 2. planning pass: scaling and the check give each problem's slice count
    pl->ntiles = 0;  // no slices yet: run the prep launches only
    CGB_CHECK(enqueue(pl, st));
    std::vector<int> need(count);
    if (count)
        CGB_CUDA(cudaMemcpyAsync(need.data(), pl->need.ptr, (size_t)count * sizeof(int), cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaStreamSynchronize(st));

    // 3. slice arena, tensor maps, schedules, split items, tiles
    size_t slice_bytes = 0;
    std::vector<size_t> soffA(count, 0), soffB(count, 0);
    std::map<std::pair<int, int>, int> sched_index;
    std::vector<Schedule> scheds;
    for (int i = 0; i < count; ++i) {
        Prob& p = pl->hp[i];
        if (p.S == 0) continue;
        p.S = std::min(std::max(need[i], 2), MAX_SLICES);  // Inf/NaN now: planned at the maximum
        p.L = 8 + 5 * (p.S - 1);
        soffA[i] = slice_bytes;
        slice_bytes += align256((size_t)p.S * p.m_pad * p.k_pad);
        soffB[i] = slice_bytes;
        slice_bytes += align256((size_t)p.S * p.n_pad * p.k_pad);
        const int per_group = (int)std::max<int64_t>(1, MAX_K_PER_CALL / std::max<int64_t>(p.k, 1));
        const auto key = std::make_pair(p.S, std::min(per_group, p.S));
        auto it = sched_index.find(key);
        if (it == sched_index.end()) {
            Schedule sc;
            int L = 0;
            CGB_CHECK(build_schedule(p.S, p.k, p.k_pad, p.m_pad, p.n_pad, &sc, &L));
            it = sched_index.emplace(key, (int)scheds.size()).first;
            scheds.push_back(sc);
        }
        p.sched = it->second;
    }
    CGB_CHECK(pl->slices.reserve(std::max<size_t>(slice_bytes, 256), st));
    std::vector<CUtensorMap> maps(2 * cnt);
    std::memset(maps.data(), 0, maps.size() * sizeof(CUtensorMap));
    std::map<std::pair<int, int>, std::vector<Item>> sitems;  // (S, kcontig) -> items
    for (int i = 0; i < count; ++i) {
        Prob& p = pl->hp[i];
        if (p.S == 0) continue;
        p.slA = (uint8_t*)pl->slices.ptr + soffA[i];
        p.slB = (uint8_t*)pl->slices.ptr + soffB[i];
        CGB_CHECK(make_tmap_2d(&maps[2 * i], CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, p.slA, (uint64_t)p.k_pad,
                               (uint64_t)p.S * p.m_pad, (uint64_t)p.k_pad, BK, BM));
        CGB_CHECK(make_tmap_2d(&maps[2 * i + 1], CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, p.slB, (uint64_t)p.k_pad,
                               (uint64_t)p.S * p.n_pad, (uint64_t)p.k_pad, BK, GBN));
        const int kbk = (int)(p.k_pad / 64);
        auto& ia = sitems[{p.S, p.opa == 1 ? 1 : 0}];
        for (int bx = 0; bx < p.m_pad / 64; ++bx)
            for (int by = 0; by < kbk; ++by) ia.push_back(make_int4(i, 0, bx, by));
        auto& ib = sitems[{p.S, p.opb == 0 ? 1 : 0}];
        for (int bx = 0; bx < p.n_pad / 64; ++bx)
            for (int by = 0; by < kbk; ++by) ib.push_back(make_int4(i, 1, bx, by));
        for (int mb = 0; mb < p.m_pad / BM; ++mb)
            for (int nb = 0; nb < p.n_pad / GBN; ++nb) pl->tile_list.push_back(make_int4(i, mb, nb, 0));
        pl->padded += 2.0 * p.S * (p.S + 1) / 2 * (double)p.m_pad * p.n_pad * p.k_pad;
    }
    std::vector<Item> all_items;
    pl->splits.clear();
    for (auto& kv : sitems) {
        Plan::SplitLaunch sl{kv.first.first, kv.first.second != 0, (int)all_items.size(), (int)kv.second.size()};
        all_items.insert(all_items.end(), kv.second.begin(), kv.second.end());
        pl->splits.push_back(sl);
    }
    CGB_CHECK(pl->sitems.reserve(std::max<size_t>(all_items.size(), 1) * sizeof(Item), st));
    if (!all_items.empty())
        CGB_CUDA(cudaMemcpyAsync(pl->sitems.ptr, all_items.data(), all_items.size() * sizeof(Item),
                                 cudaMemcpyHostToDevice, st));
    CGB_CHECK(pl->maps.reserve(maps.size() * sizeof(CUtensorMap), st));
    CGB_CUDA(cudaMemcpyAsync(pl->maps.ptr, maps.data(), maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice, st));
    CGB_CHECK(pl->scheds.reserve(std::max<size_t>(scheds.size(), 1) * sizeof(Schedule), st));
    if (!scheds.empty())
        CGB_CUDA(cudaMemcpyAsync(pl->scheds.ptr, scheds.data(), scheds.size() * sizeof(Schedule),
                                 cudaMemcpyHostToDevice, st));
    if (count)
        CGB_CUDA(cudaMemcpyAsync(pl->probs.ptr, pl->hp.data(), (size_t)count * sizeof(Prob), cudaMemcpyHostToDevice, st));
    pl->ntiles = (int)pl->tile_list.size();
    CGB_CHECK(pl->tiles.reserve(std::max<size_t>(pl->tile_list.size(), 1) * sizeof(int4), st));
    pl->grid = std::max(1, std::min(pl->ntiles, num_sms()));
    CGB_CUDA(cudaFuncSetAttribute(ozaki_grouped_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, G_SMEM));
    CGB_CHECK(upload_tiles(pl, 0, st));
    CGB_CHECK(capture(pl));
    // tuning replays the batch: only when that cannot change C (beta == 0 everywhere)
    bool beta_free = true;
    for (const Prob& p : pl->hp) beta_free &= p.S == 0 || p.beta_zero;
    if (tune && beta_free && pl->ntiles > 0) CGB_CHECK(autotune(pl, st));
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

}  // namespace ozg

// Entry points used by the grouped plan (grouped.cu).
cosma_gpu_oz_grouped_plan* oz_grouped_create(int count, const cosma_gpu_gemm_problem* problems, int autotune,
                                             cudaStream_t st, int* status) {
    auto* pl = new cosma_gpu_oz_grouped_plan();
    *status = ozg::build(pl, count, problems, autotune, st);
    if (*status != COSMA_GPU_SUCCESS) {
        ozg::destroy(pl);
        return nullptr;
    }
    return pl;
}
int oz_grouped_run(cosma_gpu_oz_grouped_plan* pl, cudaStream_t st) { return ozg::run(pl, st); }
void oz_grouped_destroy(cosma_gpu_oz_grouped_plan* pl) { ozg::destroy(pl); }
void oz_grouped_info(const cosma_gpu_oz_grouped_plan* pl, cosma_gpu_grouped_info* info) {
    info->tiles = pl->ntiles;
    info->tile_policy = 3;  // 128 x 64 tensor-core tiles, partial sums in TMEM
    info->dynamic_schedule = 0;
    info->warps_per_cta = ozg::G_THREADS / 32;
    info->useful_flops = pl->useful;
    info->padded_flops = pl->padded;
    info->tuned_ms = pl->tuned_ms;
}
int oz_grouped_slices(const cosma_gpu_oz_grouped_plan* pl, int* out) {
    for (int i = 0; i < pl->count; ++i) out[i] = pl->hp[i].S;
    return COSMA_GPU_SUCCESS;
}

}  // namespace cgb
