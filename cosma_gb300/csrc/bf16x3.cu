// Single-precision GEMM from three BF16 slices per operand on the BF16
// tensor cores (the FP32 precision form).
//
// Splitting: every FP32 value a is written exactly as a = h + m + l with
// h = bf16(a), m = bf16(a - h), l = bf16(a - h - m) (round to nearest; each
// residual is exact in FP32 and carries 8 fewer bits, so 3 x 8 bits cover
// the 24-bit significand).  The product keeps the six slice products of
// weight >= 2^-16 relative to h*h - l*h, m*m, h*l, m*h, h*m, h*h, issued in
// that order (smallest first) - and drops m*l, l*m, l*l (<= 2^-24 relative).
//
// Accumulation: the tensor core's FP32 accumulator loses low bits on every
// addition in a biased way, so a long chain (all of K in one accumulator)
// ends several times less accurate than an FP32 GEMM.  Each TMEM accumulation
// therefore spans only a 512-wide K chunk (all six products of the chunk),
// and the epilogue adds the chunk results with round-to-nearest FP32
// additions in registers; the result is as accurate as an FP32 GEMM.
//
// Kernel: persistent, warp-specialised like the Ozaki GEMM: 128 x 256 tile,
// 64-element (128-byte) K blocks of BF16 through a 4-stage TMA ring with
// 128-byte swizzle, tcgen05.mma kind::f16 (K = 16 per instruction), two TMEM
// accumulators alternating between chunks so the epilogue's drain of one
// overlaps the MMAs of the next; 8 epilogue warps hold the running sums.
#include "common.cuh"
#include "runtime.hpp"
#include "tc_common.cuh"
#include "tma_host.hpp"

#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <string>

namespace cgb {
namespace b3 {

constexpr int BM = 128, BN = 256, BKE = 64;  // BKE: BF16 elements per K block (128 bytes)
constexpr int STAGES = 4;
constexpr int A_STAGE = BM * 128, B_STAGE = BN * 128, STAGE_BYTES = A_STAGE + B_STAGE;
constexpr int EPI_THREADS = 256;            // 8 epilogue warps
constexpr int THREADS = 64 + EPI_THREADS;   // + TMA warp + MMA warp
constexpr int KB_PER_CHUNK = 8;            // K chunk of 512 per TMEM accumulation
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 256;
constexpr int NPROD = 6;
// slice pairs (A slice, B slice), smallest weight first
__constant__ int8_t kPairA[NPROD] = {2, 1, 0, 1, 0, 0};
__constant__ int8_t kPairB[NPROD] = {0, 1, 2, 0, 1, 0};

struct Params {
    int num_m_tiles, num_n_tiles, num_tiles;
    int kb_count;
    int a_rows_pad, b_rows_pad;
    int64_t m, n, ldc;
    float* C;
    float alpha, beta;
    int beta_zero;
    unsigned* err;
};

// Three BF16 slices of a (rows x k) FP32 operand, row-major with row pitch
// k_pad elements, zero padded to rows_pad x k_pad.  Each thread handles 8
// consecutive K elements of one row.  kcontig: element (r, l) at X[l + r*ld],
// else at X[r + l*ld].
template <bool KCONTIG>
__global__ void __launch_bounds__(256) split3_kernel(const float* __restrict__ X, int64_t ld, int64_t rows,
                                                     int64_t k, int64_t k_pad, int64_t rows_pad,
                                                     __nv_bfloat16* __restrict__ out) {
    const int t = threadIdx.x;
    int64_t r;
    int kc;
    if (KCONTIG) { r = (int64_t)blockIdx.x * 32 + t / 8; kc = t % 8; }
    else { r = (int64_t)blockIdx.x * 32 + t % 32; kc = t / 32; }
    const int64_t l0 = (int64_t)blockIdx.y * 64 + kc * 8;
    if (r >= rows_pad || l0 >= k_pad) return;
    __align__(16) __nv_bfloat16 s[3][8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        const int64_t l = l0 + e;
        float a = 0.0f;
        if (r < rows && l < k) a = KCONTIG ? X[l + r * ld] : X[r + l * ld];
        const __nv_bfloat16 h = __float2bfloat16_rn(a);
        const float r1 = __fsub_rn(a, __bfloat162float(h));
        const __nv_bfloat16 m = __float2bfloat16_rn(r1);
        const float r2 = __fsub_rn(r1, __bfloat162float(m));
        s[0][e] = h;
        s[1][e] = m;
        s[2][e] = __float2bfloat16_rn(r2);
    }
#pragma unroll
    for (int q = 0; q < 3; ++q)
        *reinterpret_cast<uint4*>(out + (int64_t)q * rows_pad * k_pad + r * k_pad + l0) =
            *reinterpret_cast<const uint4*>(s[q]);
}

__device__ __forceinline__ void tile_coords(int tile, int num_m, int num_n, int& mb, int& nb) {
    constexpr int kStripM = 16;  // see the Ozaki GEMM: strips keep a wave's panels in L2
    const int strip = tile / (kStripM * num_n);
    const int r = tile - strip * kStripM * num_n;
    const int h = min(kStripM, num_m - strip * kStripM);
    nb = r / h;
    mb = strip * kStripM + r % h;
}

__global__ void __launch_bounds__(THREADS, 1)
    bf16x3_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                       const __grid_constant__ Params p) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* full = (uint64_t*)(smem + STAGES * STAGE_BYTES);
    uint64_t* empty = full + STAGES;
    uint64_t* accf = empty + STAGES;
    uint64_t* acce = accf + 2;
    uint64_t* drain = acce + 2;
    uint32_t* tmem_slot = (uint32_t*)(drain + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nchunks = (p.kb_count + KB_PER_CHUNK - 1) / KB_PER_CHUNK;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&accf[b], 1);
            tc::mbar_init(&acce[b], EPI_THREADS);
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
        if (lane == 0) {  // TMA producer
            uint32_t it = 0;
            bool ok = true;
            for (int tile = blockIdx.x; tile < p.num_tiles && ok; tile += gridDim.x) {
                int mb, nb;
                tile_coords(tile, p.num_m_tiles, p.num_n_tiles, mb, nb);
                for (int c = 0; c < nchunks && ok; ++c) {
                    const int kb0 = c * KB_PER_CHUNK, kb1 = min(p.kb_count, kb0 + KB_PER_CHUNK);
                    for (int u = 0; u < NPROD && ok; ++u) {
                        const int arow = kPairA[u] * p.a_rows_pad + mb * BM;
                        const int brow = kPairB[u] * p.b_rows_pad + nb * BN;
                        for (int kb = kb0; kb < kb1; ++kb, ++it) {
                            const int st = it % STAGES;
                            if (!tc::mbar_wait(&empty[st], ((it / STAGES) & 1) ^ 1, p.err, kDevTimeoutEmpty)) {
                                ok = false;
                                break;
                            }
                            tc::mbar_arrive_expect_tx(&full[st], STAGE_BYTES);
                            uint8_t* sa = smem + st * STAGE_BYTES;
                            tc::tma_load_2d(sa, &tmA, kb * BKE, arow, &full[st]);
                            tc::tma_load_2d(sa + A_STAGE, &tmB, kb * BKE, brow, &full[st]);
                        }
                    }
                }
            }
            const uint32_t first = it > STAGES ? it - STAGES : 0;
            for (uint32_t j = first; j < it; ++j) tc::mbar_wait_drain(&full[j % STAGES], (j / STAGES) & 1);
        }
    } else if (warp == 1) {
        if (lane == 0) {  // MMA issuer: one accumulator per K chunk, buffers alternate
            constexpr uint32_t ID = tc::idesc(tc::kFmtBF16, tc::kFmtBF16, BM, BN);
            uint32_t it = 0, acc_it = 0;
            bool ok = true;
            for (int tile = blockIdx.x; tile < p.num_tiles && ok; tile += gridDim.x) {
                for (int c = 0; c < nchunks && ok; ++c, ++acc_it) {
                    const int kb0 = c * KB_PER_CHUNK, kb1 = min(p.kb_count, kb0 + KB_PER_CHUNK);
                    const uint32_t buf = acc_it & 1;
                    if (!tc::mbar_wait(&acce[buf], ((acc_it >> 1) & 1) ^ 1, p.err, kDevTimeoutAccEmpty)) {
                        ok = false;
                        break;
                    }
                    tc::tc_fence_after();
                    const uint32_t d_tmem = tmem + buf * BN;
                    uint32_t accumulate = 0;
                    for (int u = 0; u < NPROD && ok; ++u) {
                        for (int kb = kb0; kb < kb1; ++kb, ++it) {
                            const int st = it % STAGES;
                            if (!tc::mbar_wait(&full[st], (it / STAGES) & 1, p.err, kDevTimeoutFull)) {
                                ok = false;
                                break;
                            }
                            tc::tc_fence_after();
                            const uint32_t sa = tc::smem_u32(smem + st * STAGE_BYTES);
                            const uint64_t ad = tc::sdesc_k_sw128(sa), bd = tc::sdesc_k_sw128(sa + A_STAGE);
#pragma unroll
                            for (int kk = 0; kk < 4; ++kk) {  // 4 x K=16 BF16 = 128 bytes
                                tc::mma_f16(d_tmem, ad + 2 * kk, bd + 2 * kk, ID, accumulate);
                                accumulate = 1;
                            }
                            tc::mma_commit(&empty[st]);
                        }
                    }
                    if (ok) tc::mma_commit(&accf[buf]);
                }
            }
            tc::mma_commit(drain);
            tc::mbar_wait_drain(drain, 0);
        }
    } else {
        // Epilogue, 8 warps: two per TMEM lane quadrant, each owning 128 of the
        // tile's 256 columns.  Chunk results are summed in registers with
        // round-to-nearest FP32 additions; C = alpha*sum + beta*C at the end.
        const int quad = warp & 3;
        const int half = (warp - 2) >> 2;
        const int row = quad * 32 + lane;
        uint32_t acc_it = 0;
        bool ok = true;
        for (int tile = blockIdx.x; tile < p.num_tiles && ok; tile += gridDim.x) {
            int mb, nb;
            tile_coords(tile, p.num_m_tiles, p.num_n_tiles, mb, nb);
            float sum[128];
            for (int c = 0; c < nchunks && ok; ++c, ++acc_it) {
                const uint32_t buf = acc_it & 1;
                ok = __all_sync(0xffffffffu, tc::mbar_wait(&accf[buf], (acc_it >> 1) & 1, p.err, kDevTimeoutAcc));
                if (!ok) break;
                tc::tc_fence_after();
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    uint32_t v[16];
                    tc::tmem_ld_32x32b_x16(tmem + ((uint32_t)(quad * 32) << 16) + buf * BN + half * 128 + q * 16, v);
                    tc::tmem_ld_wait();
#pragma unroll
                    for (int j = 0; j < 16; ++j)
                        sum[q * 16 + j] = c == 0 ? __uint_as_float(v[j]) : __fadd_rn(sum[q * 16 + j], __uint_as_float(v[j]));
                }
                tc::tc_fence_before();
                tc::mbar_arrive(&acce[buf]);
            }
            if (!ok) break;
            const int64_t gi = (int64_t)mb * BM + row;
            if (gi < p.m) {
#pragma unroll
                for (int j = 0; j < 128; ++j) {
                    const int64_t gj = (int64_t)nb * BN + half * 128 + j;
                    if (gj < p.n) {
                        float* cp = p.C + gi + gj * p.ldc;
                        float r = __fmul_rn(p.alpha, sum[j]);
                        if (!p.beta_zero) r = __fadd_rn(r, __fmul_rn(p.beta, *cp));
                        *cp = r;
                    }
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

struct Workspace {
    DeviceBuffer slicesA, slicesB, err;
    unsigned* host_err = nullptr;
};
std::mutex g_mu;
std::map<std::pair<int, cudaStream_t>, Workspace*> g_ws;

Workspace* workspace(cudaStream_t s) {
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lock(g_mu);
    auto& w = g_ws[{dev, s}];
    if (!w) w = new Workspace();
    // (re)tried until it exists: a failed allocation fails this call only
    if (!w->host_err && pinned_alloc((void**)&w->host_err, sizeof(unsigned)) != cudaSuccess) w->host_err = nullptr;
    cudaGetLastError();
    return w;
}

int num_sms() { return device_sm_count(); }

}  // namespace b3

int bf16x3_sgemm(const GemmDesc& g, cudaStream_t st) {
    using namespace b3;
    if (g.scalar != Scalar::S) return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "bf16x3: float only");
    if (((uintptr_t)g.A | (uintptr_t)g.B | (uintptr_t)g.C) % 4)
        return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "bf16x3: buffers must be 4-byte aligned");
    const int64_t m = g.m, n = g.n, k = g.k;
    if (m > (int64_t)1 << 24 || n > (int64_t)1 << 24 || k > (int64_t)1 << 26)
        return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "bf16x3: size limits exceeded");
    const bool ta = g.opa != 0, tb = g.opb != 0;
    Workspace* w = workspace(st);
    if (!w->host_err) return set_error(COSMA_GPU_ERROR_OUT_OF_MEMORY, "bf16x3: pinned staging");
    const int64_t m_pad = ceil_div(m, BM) * BM, n_pad = ceil_div(n, BN) * BN, k_pad = ceil_div(k, BKE) * BKE;
    CGB_CHECK(w->slicesA.reserve((size_t)3 * m_pad * k_pad * 2, st));
    CGB_CHECK(w->slicesB.reserve((size_t)3 * n_pad * k_pad * 2, st));
    CGB_CHECK(w->err.reserve(sizeof(unsigned), st));
    CGB_CUDA(cudaMemsetAsync(w->err.ptr, 0, sizeof(unsigned), st));
    auto* sa = (__nv_bfloat16*)w->slicesA.ptr;
    auto* sb = (__nv_bfloat16*)w->slicesB.ptr;
    const float* A = (const float*)g.A;
    const float* B = (const float*)g.B;
    {
        dim3 gA((unsigned)(m_pad / 32), (unsigned)(k_pad / 64)), gB((unsigned)(n_pad / 32), (unsigned)(k_pad / 64));
        if (ta) split3_kernel<true><<<gA, 256, 0, st>>>(A, g.lda, m, k, k_pad, m_pad, sa);
        else split3_kernel<false><<<gA, 256, 0, st>>>(A, g.lda, m, k, k_pad, m_pad, sa);
        if (!tb) split3_kernel<true><<<gB, 256, 0, st>>>(B, g.ldb, n, k, k_pad, n_pad, sb);
        else split3_kernel<false><<<gB, 256, 0, st>>>(B, g.ldb, n, k, k_pad, n_pad, sb);
        CGB_CUDA(cudaGetLastError());
    }
    Params p;
    std::memset(&p, 0, sizeof(p));
    p.num_m_tiles = (int)(m_pad / BM);
    p.num_n_tiles = (int)(n_pad / BN);
    p.num_tiles = p.num_m_tiles * p.num_n_tiles;
    p.kb_count = (int)(k_pad / BKE);
    p.a_rows_pad = (int)m_pad;
    p.b_rows_pad = (int)n_pad;
    p.m = m; p.n = n; p.ldc = g.ldc;
    p.C = (float*)g.C;
    p.alpha = (float)g.alpha[0];
    p.beta = (float)g.beta[0];
    p.beta_zero = g.beta[0] == 0.0;
    p.err = (unsigned*)w->err.ptr;
    CUtensorMap tmA, tmB;
    CGB_CHECK(make_tmap_2d(&tmA, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, sa, (uint64_t)k_pad, (uint64_t)(3 * m_pad),
                           (uint64_t)k_pad * 2, BKE, BM));
    CGB_CHECK(make_tmap_2d(&tmB, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, sb, (uint64_t)k_pad, (uint64_t)(3 * n_pad),
                           (uint64_t)k_pad * 2, BKE, BN));
    static PerDevice<bool> attr;  // the attribute is set once per device
    bool done = false;
    CGB_CHECK(attr.get(
        [](bool& v) {
            CGB_CUDA(cudaFuncSetAttribute(bf16x3_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          SMEM_BYTES));
            v = true;
            return COSMA_GPU_SUCCESS;
        },
        &done));
    const int grid = std::min(p.num_tiles, num_sms());
    bf16x3_gemm_kernel<<<grid, THREADS, SMEM_BYTES, st>>>(tmA, tmB, p);
    CGB_CUDA(cudaGetLastError());
    CGB_CUDA(cudaMemcpyAsync(w->host_err, w->err.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaStreamSynchronize(st));
    if (*w->host_err)
        return set_error(COSMA_GPU_ERROR_DEVICE_TIMEOUT,
                         "bf16x3 gemm: a pipeline wait timed out (device code " + std::to_string(*w->host_err) + ")");
    return COSMA_GPU_SUCCESS;
}

}  // namespace cgb
