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
#include "pipeline.hpp"

#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

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

// The GEMM kernel's shared-memory attribute, set once per device.
int gemm_attr() {
    static PerDevice<bool> attr;
    bool done = false;
    return attr.get(
        [](bool& v) {
            CGB_CUDA(cudaFuncSetAttribute(bf16x3_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          SMEM_BYTES));
            v = true;
            return COSMA_GPU_SUCCESS;
        },
        &done);
}

// The GEMM over slice stacks sa (3 x a_rows_pad rows) and sb (3 x b_rows_pad
// rows) of K depth k_pad, into C (m x n, ldc).
int launch_gemm(const __nv_bfloat16* sa, int64_t a_rows_pad, const __nv_bfloat16* sb, int64_t b_rows_pad,
                int64_t k_pad, int64_t m, int64_t n, float* C, int64_t ldc, float alpha, float beta, unsigned* err,
                cudaStream_t st) {
    Params p;
    std::memset(&p, 0, sizeof(p));
    p.num_m_tiles = (int)(a_rows_pad / BM);
    p.num_n_tiles = (int)(b_rows_pad / BN);
    p.num_tiles = p.num_m_tiles * p.num_n_tiles;
    p.kb_count = (int)(k_pad / BKE);
    p.a_rows_pad = (int)a_rows_pad;
    p.b_rows_pad = (int)b_rows_pad;
    p.m = m; p.n = n; p.ldc = ldc;
    p.C = C;
    p.alpha = alpha;
    p.beta = beta;
    p.beta_zero = beta == 0.0f;
    p.err = err;
    CUtensorMap tmA, tmB;
    CGB_CHECK(make_tmap_2d(&tmA, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, sa, (uint64_t)k_pad, (uint64_t)(3 * a_rows_pad),
                           (uint64_t)k_pad * 2, BKE, BM));
    CGB_CHECK(make_tmap_2d(&tmB, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, sb, (uint64_t)k_pad, (uint64_t)(3 * b_rows_pad),
                           (uint64_t)k_pad * 2, BKE, BN));
    CGB_CHECK(gemm_attr());
    const int grid = std::min(p.num_tiles, num_sms());
    bf16x3_gemm_kernel<<<grid, THREADS, SMEM_BYTES, st>>>(tmA, tmB, p);
    CGB_CUDA(cudaGetLastError());
    return COSMA_GPU_SUCCESS;
}

void launch_split3(bool kcontig, const float* X, int64_t ld, int64_t rows, int64_t k, int64_t k_pad, int64_t rows_pad,
                   __nv_bfloat16* out, cudaStream_t st) {
    const dim3 grid((unsigned)(rows_pad / 32), (unsigned)(k_pad / 64));
    if (kcontig) split3_kernel<true><<<grid, 256, 0, st>>>(X, ld, rows, k, k_pad, rows_pad, out);
    else split3_kernel<false><<<grid, 256, 0, st>>>(X, ld, rows, k, k_pad, rows_pad, out);
}

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
    launch_split3(ta, A, g.lda, m, k, k_pad, m_pad, sa, st);
    launch_split3(!tb, B, g.ldb, n, k, k_pad, n_pad, sb, st);
    CGB_CUDA(cudaGetLastError());
    CGB_CHECK(launch_gemm(sa, m_pad, sb, n_pad, k_pad, m, n, (float*)g.C, g.ldc, (float)g.alpha[0], (float)g.beta[0],
                          (unsigned*)w->err.ptr, st));
    CGB_CUDA(cudaMemcpyAsync(w->host_err, w->err.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaStreamSynchronize(st));
    if (*w->host_err)
        return set_error(COSMA_GPU_ERROR_DEVICE_TIMEOUT,
                         "bf16x3 gemm: a pipeline wait timed out (device code " + std::to_string(*w->host_err) + ")");
    return COSMA_GPU_SUCCESS;
}

namespace b3 {

// ------------------------------------------------------ host operands, overlapped
// One-step SGEMM on host A, B and C (C = alpha op(A) op(B) + beta C) with the
// host link's copies overlapped with the work: op(A) arrives in row panels
// and op(B) in column panels, each
// panel's three BF16 slices are split on a second stream as it lands, block
// (i, j)'s GEMM runs once both its panels are split, and its C block leaves
// while later blocks compute.  Nothing is chosen from the data, so no block
// waits for a check, and every output's K loop is the one-step call's: the
// same bits.  The first panel of each operand is copied by the calling
// thread (a pageable one by the device copy kernel, before any kernel of the
// call runs), every later copy by the copy thread through the copy engines.
constexpr int kRing = 4;            // C slots in flight
constexpr int kMaxPanels = 8;
constexpr int kEvents = 2 * kMaxPanels + 3 * kRing;

struct PipeWS {
    DeviceBuffer a, b, sa, sb, C[kRing], err;
    unsigned* host_err = nullptr;
    std::vector<cudaEvent_t> ev;
    cudaStream_t ss = nullptr;  // the slice splits, beside the GEMMs
    std::unique_ptr<CopyWorker> worker;
};
std::mutex g_pipe_mu;
std::map<std::pair<int, cudaStream_t>, PipeWS*> g_pipe;

PipeWS* pipe_ws(cudaStream_t s) {
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lock(g_pipe_mu);
    auto& w = g_pipe[{dev, s}];
    if (!w) w = new PipeWS();
    if (!w->host_err && pinned_alloc((void**)&w->host_err, sizeof(unsigned)) != cudaSuccess) w->host_err = nullptr;
    if (w->ev.empty()) {
        w->ev.assign(kEvents, nullptr);
        for (auto& e : w->ev)
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) e = nullptr;
    }
    if (!w->ss && cudaStreamCreateWithFlags(&w->ss, cudaStreamNonBlocking) != cudaSuccess) w->ss = nullptr;
    if (!w->worker) {
        try {
            w->worker.reset(new CopyWorker(dev));
        } catch (...) {
            w->worker.reset();
        }
    }
    cudaGetLastError();
    return w;
}

void release_stream(cudaStream_t s) {
    int dev = 0;
    cudaGetDevice(&dev);
    PipeWS* pw = nullptr;
    Workspace* w = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_pipe_mu);
        auto it = g_pipe.find({dev, s});
        if (it != g_pipe.end()) {
            pw = it->second;
            g_pipe.erase(it);
        }
    }
    {
        std::lock_guard<std::mutex> lock(g_mu);
        auto it = g_ws.find({dev, s});
        if (it != g_ws.end()) {
            w = it->second;
            g_ws.erase(it);
        }
    }
    if (pw) {
        pw->worker.reset();  // runs what is queued, then joins
        if (pw->host_err) cudaFreeHost(pw->host_err);
        for (auto e : pw->ev)
            if (e) cudaEventDestroy(e);
        if (pw->ss) {
            cudaStreamSynchronize(pw->ss);
            cudaStreamDestroy(pw->ss);
        }
        delete pw;
    }
    if (w) {
        if (w->host_err) cudaFreeHost(w->host_err);
        delete w;
    }
    cudaGetLastError();
}

int sgemm_host_body(const GemmDesc& g, cudaStream_t cs, cudaStream_t hs, cudaStream_t ds, int64_t* h2d_bytes,
                    int64_t* d2h_bytes, bool* taken) {
    *taken = false;
    const int64_t m = g.m, n = g.n, k = g.k;
    if (g.scalar != Scalar::S || m < 1 || n < 1 || k < 1) return COSMA_GPU_SUCCESS;
    if (m > (int64_t)1 << 24 || n > (int64_t)1 << 24 || k > (int64_t)64 * 65535) return COSMA_GPU_SUCCESS;
    const bool a_kc = g.opa != 0, b_kc = g.opb == 0;  // op(A) rows / op(B) columns contiguous along K
    // op(A) in 2 row panels and op(B) in up to 4 column panels, without a
    // shorter lead panel: the GEMM of a 2048-row block leaves more of its
    // last wave idle than the earlier start gains (16384^3 from pinned
    // buffers: 34.9 ms per call against 38.6 with the lead panel).
    const Panels PA = make_panels(m, m >= 2048 ? 2 : 1, m);
    const Panels PB = make_panels(n, n >= 4096 ? 4 : (n >= 2048 ? 2 : 1), n);
    const int MA = PA.count, NB = PB.count, NP = MA + NB;
    if (MA * NB < 2 || MA > kMaxPanels / 2 || NB > kMaxPanels / 2) return COSMA_GPU_SUCCESS;
    PipeWS* w = pipe_ws(cs);
    if (!w->host_err || !w->ss || !w->worker) return COSMA_GPU_SUCCESS;  // the regular path
    for (auto e : w->ev)
        if (!e) return COSMA_GPU_SUCCESS;
    cudaStream_t ss = w->ss;
    CopyWorker& cw = *w->worker;
    const int64_t k_pad = ceil_div(k, BKE) * BKE;
    const float* A = (const float*)g.A;
    const float* B = (const float*)g.B;
    float* C = (float*)g.C;
    const bool beta_zero = g.beta[0] == 0.0;

    // panel geometry: compact device copies, slice stacks of 3 x rows_pad rows
    int64_t offA[kMaxPanels], offB[kMaxPanels], soffA[kMaxPanels], soffB[kMaxPanels];
    int64_t a_elems = 0, b_elems = 0, sa_elems = 0, sb_elems = 0;
    for (int i = 0; i < MA; ++i) {
        offA[i] = a_elems; a_elems += PA.rows(i, m) * k;
        soffA[i] = sa_elems; sa_elems += 3 * ceil_div(PA.rows(i, m), BM) * BM * k_pad;
    }
    for (int j = 0; j < NB; ++j) {
        offB[j] = b_elems; b_elems += PB.rows(j, n) * k;
        soffB[j] = sb_elems; sb_elems += 3 * ceil_div(PB.rows(j, n), BN) * BN * k_pad;
    }
    const int NBLK = MA * NB, NR = std::min(NBLK, kRing);
    // everything that could allocate is reserved before the first copy
    CGB_CHECK(w->a.reserve((size_t)a_elems * 4, cs));
    CGB_CHECK(w->b.reserve((size_t)b_elems * 4, cs));
    CGB_CHECK(w->sa.reserve((size_t)sa_elems * 2, cs));
    CGB_CHECK(w->sb.reserve((size_t)sb_elems * 2, cs));
    for (int r = 0; r < NR; ++r) CGB_CHECK(w->C[r].reserve((size_t)PA.largest() * PB.largest() * 4, cs));
    CGB_CHECK(w->err.reserve(sizeof(unsigned), cs));
    CGB_CUDA(cudaMemsetAsync(w->err.ptr, 0, sizeof(unsigned), cs));
    CGB_CUDA(cudaStreamSynchronize(cs));
    float* dA = (float*)w->a.ptr;
    float* dB = (float*)w->b.ptr;
    auto* sa = (__nv_bfloat16*)w->sa.ptr;
    auto* sb = (__nv_bfloat16*)w->sb.ptr;
    int evi = 0;
    auto next_event = [&]() { return w->ev[evi++]; };
    cudaEvent_t ev_copy[kMaxPanels], ev_split[kMaxPanels];
    uint64_t tk_copy[kMaxPanels] = {};
    bool split_issued[kMaxPanels] = {};
    *taken = true;  // from here the call owns C
    *h2d_bytes = 0;
    *d2h_bytes = 0;

    auto copy_task = [](void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t cols,
                        cudaMemcpyKind kind, cudaStream_t st, cudaEvent_t wait_ev, cudaEvent_t done_ev) {
        return [=]() -> int {
            if (wait_ev) CGB_CUDA(cudaStreamWaitEvent(st, wait_ev, 0));
            CGB_CHECK(copy_2d_from_thread(dst, dpitch, src, spitch, width, cols, kind, st));
            CGB_CUDA(cudaEventRecord(done_ev, st));
            return COSMA_GPU_SUCCESS;
        };
    };
    auto copy_panel = [&](int p) -> int {
        ev_copy[p] = next_event();
        void* dst;
        const void* src;
        size_t dpitch, spitch, width, cols;
        if (p < MA) {
            const int64_t i0 = PA.first(p), mi = PA.rows(p, m);
            dst = dA + offA[p];
            if (!a_kc) { dpitch = mi * 4; src = A + i0; spitch = g.lda * 4; width = mi * 4; cols = k; }
            else { dpitch = k * 4; src = A + i0 * g.lda; spitch = g.lda * 4; width = k * 4; cols = mi; }
            *h2d_bytes += mi * k * 4;
        } else {
            const int j = p - MA;
            const int64_t j0 = PB.first(j), nj = PB.rows(j, n);
            dst = dB + offB[j];
            if (b_kc) { dpitch = k * 4; src = B + j0 * g.ldb; spitch = g.ldb * 4; width = k * 4; cols = nj; }
            else { dpitch = nj * 4; src = B + j0; spitch = g.ldb * 4; width = nj * 4; cols = k; }
            *h2d_bytes += nj * k * 4;
        }
        if (p == 0 || p == MA) {  // before any kernel of the call: the calling thread
            CGB_CHECK(copy_2d_overlapped(dst, dpitch, src, spitch, width, cols, cudaMemcpyHostToDevice, hs));
            CGB_CUDA(cudaEventRecord(ev_copy[p], hs));
            tk_copy[p] = 0;
        } else {
            tk_copy[p] = cw.post(copy_task(dst, dpitch, src, spitch, width, cols, cudaMemcpyHostToDevice, hs,
                                           nullptr, ev_copy[p]));
        }
        return COSMA_GPU_SUCCESS;
    };
    // the slices of panel p, on ss once it has landed
    auto split_panel = [&](int p) -> int {
        if (split_issued[p]) return COSMA_GPU_SUCCESS;
        split_issued[p] = true;
        CGB_CHECK(cw.wait(tk_copy[p]));  // its event is recorded
        CGB_CUDA(cudaStreamWaitEvent(ss, ev_copy[p], 0));
        if (p < MA) {
            const int64_t mi = PA.rows(p, m);
            launch_split3(a_kc, dA + offA[p], a_kc ? k : mi, mi, k, k_pad, ceil_div(mi, BM) * BM, sa + soffA[p], ss);
        } else {
            const int j = p - MA;
            const int64_t nj = PB.rows(j, n);
            launch_split3(b_kc, dB + offB[j], b_kc ? k : nj, nj, k, k_pad, ceil_div(nj, BN) * BN, sb + soffB[j], ss);
        }
        CGB_CUDA(cudaGetLastError());
        ev_split[p] = next_event();
        CGB_CUDA(cudaEventRecord(ev_split[p], ss));
        return COSMA_GPU_SUCCESS;
    };

    // copies: the lead panels, then op(B)'s (block row 0 uses them), then op(A)'s
    CGB_CHECK(copy_panel(0));
    CGB_CHECK(copy_panel(MA));
    for (int p = MA + 1; p < NP; ++p) CGB_CHECK(copy_panel(p));
    for (int p = 1; p < MA; ++p) CGB_CHECK(copy_panel(p));

    cudaEvent_t ev_gemm[kRing], ev_out[kRing], ev_cin[kRing];
    for (int r = 0; r < NR; ++r) {
        ev_gemm[r] = next_event();
        ev_out[r] = next_event();
        ev_cin[r] = next_event();
    }
    bool out_used[kRing] = {};
    uint64_t tk_out[kRing] = {};
    const float alpha = (float)g.alpha[0], beta = (float)g.beta[0];
    for (int b = 0; b < NBLK; ++b) {
        const int i = b / NB, j = b % NB, slot = b % NR;
        const int64_t i0 = PA.first(i), mi = PA.rows(i, m), j0 = PB.first(j), nj = PB.rows(j, n);
        CGB_CHECK(split_panel(i));
        CGB_CHECK(split_panel(MA + j));
        CGB_CUDA(cudaStreamWaitEvent(cs, ev_split[i], 0));
        CGB_CUDA(cudaStreamWaitEvent(cs, ev_split[MA + j], 0));
        float* cdev = (float*)w->C[slot].ptr;
        float* chost = C + i0 + j0 * g.ldc;
        if (!beta_zero) {  // the old C block comes in once its slot has been drained
            const uint64_t t = cw.post(copy_task(cdev, mi * 4, chost, g.ldc * 4, mi * 4, nj, cudaMemcpyHostToDevice,
                                                 hs, out_used[slot] ? ev_out[slot] : nullptr, ev_cin[slot]));
            *h2d_bytes += mi * nj * 4;
            CGB_CHECK(cw.wait(t));
            CGB_CUDA(cudaStreamWaitEvent(cs, ev_cin[slot], 0));
        } else if (out_used[slot]) {
            CGB_CHECK(cw.wait(tk_out[slot]));
            CGB_CUDA(cudaStreamWaitEvent(cs, ev_out[slot], 0));
        }
        const int64_t mi_pad = ceil_div(mi, BM) * BM, nj_pad = ceil_div(nj, BN) * BN;
        CGB_CHECK(launch_gemm(sa + soffA[i], mi_pad, sb + soffB[j], nj_pad, k_pad, mi, nj, cdev, mi, alpha, beta,
                              (unsigned*)w->err.ptr, cs));
        CGB_CUDA(cudaEventRecord(ev_gemm[slot], cs));
        tk_out[slot] = cw.post(copy_task(chost, g.ldc * 4, cdev, mi * 4, mi * 4, nj, cudaMemcpyDeviceToHost, ds,
                                         ev_gemm[slot], ev_out[slot]));
        *d2h_bytes += mi * nj * 4;
        out_used[slot] = true;
    }
    CGB_CHECK(cw.drain());
    for (cudaStream_t s : {cs, hs, ds, ss}) CGB_CUDA(cudaStreamSynchronize(s));
    CGB_CUDA(cudaMemcpy(w->host_err, w->err.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost));
    if (*w->host_err)
        return set_error(COSMA_GPU_ERROR_DEVICE_TIMEOUT,
                         "bf16x3 gemm: a pipeline wait timed out (device code " + std::to_string(*w->host_err) + ")");
    return COSMA_GPU_SUCCESS;
}

}  // namespace b3

int bf16x3_sgemm_host(const GemmDesc& g, cudaStream_t cs, cudaStream_t hs, cudaStream_t ds, int64_t* h2d_bytes,
                      int64_t* d2h_bytes, bool* taken) {
    const int st = b3::sgemm_host_body(g, cs, hs, ds, h2d_bytes, d2h_bytes, taken);
    if (st != COSMA_GPU_SUCCESS) {  // nothing left in flight
        b3::PipeWS* w = b3::pipe_ws(cs);
        if (w->worker) w->worker->drain();
        for (cudaStream_t s : {cs, hs, ds, w->ss})
            if (s) cudaStreamSynchronize(s);
        cudaGetLastError();
        if (st == COSMA_GPU_ERROR_OUT_OF_MEMORY && !*taken) {
            for (DeviceBuffer* b : {&w->a, &w->b, &w->sa, &w->sb}) b->release();
            for (auto& c : w->C) c.release();
        }
    }
    return st;
}

void bf16x3_release_stream(cudaStream_t s) { b3::release_stream(s); }

}  // namespace cgb
