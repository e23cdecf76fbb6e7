// Grouped FP64 GEMM: many independent, uneven C_i = alpha_i op(A_i) op(B_i)
// + beta_i C_i in one persistent launch (the batching form).
//
// The reference runs such batches as a loop of local_multiply calls, one per
// sub-problem (src/cosma/multiply.cpp:476-587).  Here a single persistent
// kernel walks a tile list that spans all problems.
//
// GB300's FP64 pipe (~1 TFLOP/s, a few flops per clock per SM) is so much
// slower than its memory system that a tile needs no shared-memory staging:
// each warp owns one tile of up to 32 x 32, streams its DMMA fragments
// straight from L1/L2, and the only thing that matters is keeping the FP64
// pipe busy with useful work.  That is decided by
//  * tile shapes: per problem one of 32x32, 32x16, 16x32, 16x16, chosen to
//    cut the padding of small m / n (the autotuner picks the policy);
//  * schedule: tiles ordered by decreasing K (longest first), fetched
//    dynamically by warps through an atomic counter, or dealt statically;
//  * CTA size (warps per CTA), which sets how many warps share an SM.
// The autotuner times the candidate (policy, schedule, CTA size) triples on
// the actual batch, keeps the fastest per batch signature, and the plan
// captures memset-of-counter + launch in a CUDA graph for replay.
#include "common.cuh"
#include "runtime.hpp"

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

namespace cgb {
namespace grp {

struct Problem {  // device copy of cosma_gpu_gemm_problem, normalised
    int m, n, k, opa, opb;
    double alpha, beta;
    const double* A; int64_t lda;
    const double* B; int64_t ldb;
    double* C; int64_t ldc;
};

struct Tile {
    int problem;
    int m0, n0;
    uint8_t fm, fn;  // fragments: rows = 16*fm (1..2), cols = 8*fn (1..4)
    uint16_t pad;
};

__device__ __forceinline__ void dmma(double (&c)[4], double a0, double a1, double b0) {
    asm volatile("mma.sync.aligned.m16n8k4.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5}, {%6}, {%0,%1,%2,%3};\n"
                 : "+d"(c[0]), "+d"(c[1]), "+d"(c[2]), "+d"(c[3])
                 : "d"(a0), "d"(a1), "d"(b0));
}

__device__ __forceinline__ double ldA(const Problem& P, int i, int l) {
    if (i >= P.m || l >= P.k) return 0.0;
    return P.opa ? __ldg(P.A + l + (int64_t)i * P.lda) : __ldg(P.A + i + (int64_t)l * P.lda);
}
__device__ __forceinline__ double ldB(const Problem& P, int l, int j) {
    if (l >= P.k || j >= P.n) return 0.0;
    return P.opb ? __ldg(P.B + j + (int64_t)l * P.ldb) : __ldg(P.B + l + (int64_t)j * P.ldb);
}

// One warp computes one tile.  Fragment layouts of mma.m16n8k4.f64 (g = lane/4,
// t = lane%4): a0/a1 = A[g][t] / A[g+8][t], b0 = B[t][g], c[r] = C[g + 8(r/2)][2t + r%2].
__device__ __forceinline__ void tile_gemm(const Problem& P, const Tile& T, int lane) {
    const int g = lane >> 2, t = lane & 3;
    double acc[2][4][4];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b)
#pragma unroll
            for (int r = 0; r < 4; ++r) acc[a][b][r] = 0.0;
    const int fm = T.fm, fn = T.fn;
    for (int l0 = 0; l0 < P.k; l0 += 4) {
        double a[2][2], b[4];
#pragma unroll
        for (int mi = 0; mi < 2; ++mi) {
            const int i = T.m0 + mi * 16 + g;
            a[mi][0] = mi < fm ? ldA(P, i, l0 + t) : 0.0;
            a[mi][1] = mi < fm ? ldA(P, i + 8, l0 + t) : 0.0;
        }
#pragma unroll
        for (int ni = 0; ni < 4; ++ni) b[ni] = ni < fn ? ldB(P, l0 + t, T.n0 + ni * 8 + g) : 0.0;
#pragma unroll
        for (int mi = 0; mi < 2; ++mi)
            if (mi < fm)
#pragma unroll
                for (int ni = 0; ni < 4; ++ni)
                    if (ni < fn) dmma(acc[mi][ni], a[mi][0], a[mi][1], b[ni]);
    }
    const bool beta_zero = P.beta == 0.0;
#pragma unroll
    for (int mi = 0; mi < 2; ++mi)
#pragma unroll
        for (int ni = 0; ni < 4; ++ni)
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                if (mi >= fm || ni >= fn) continue;
                const int i = T.m0 + mi * 16 + g + 8 * (r >> 1);
                const int j = T.n0 + ni * 8 + 2 * t + (r & 1);
                if (i >= P.m || j >= P.n) continue;
                double* cp = P.C + i + (int64_t)j * P.ldc;
                double v = P.alpha * acc[mi][ni][r];
                if (!beta_zero) v += P.beta * *cp;
                *cp = v;
            }
}

__global__ void grouped_dmma_kernel(const Problem* __restrict__ probs, const Tile* __restrict__ tiles, int ntiles,
                                    int* counter, int dynamic_sched) {
    const int lane = threadIdx.x & 31;
    const int warps_per_cta = blockDim.x >> 5;
    const int gwarp = blockIdx.x * warps_per_cta + (threadIdx.x >> 5);
    const int nwarps = gridDim.x * warps_per_cta;
    int idx = dynamic_sched ? 0 : gwarp;
    if (dynamic_sched) {
        int v = 0;
        if (lane == 0) v = atomicAdd(counter, 1);
        idx = __shfl_sync(0xffffffffu, v, 0);
    }
    while (idx < ntiles) {
        const Tile T = tiles[idx];
        const Problem P = probs[T.problem];
        tile_gemm(P, T, lane);
        if (dynamic_sched) {
            int v = 0;
            if (lane == 0) v = atomicAdd(counter, 1);
            idx = __shfl_sync(0xffffffffu, v, 0);
        } else {
            idx += nwarps;
        }
    }
}

// ------------------------------------------------------------------ host
struct Config {
    int policy;       // 0: all 32x32, 1: per-problem smallest padded work, 2: 16-row tiles for m <= 16
    int dynamic_sched;
    int warps_per_cta;
};

// Tiles of one problem under a policy.
void problem_tiles(const Problem& P, int pi, int policy, std::vector<Tile>& out) {
    int tm = 32, tn = 32;
    if (policy == 1) {
        static const int shapes[4][2] = {{32, 32}, {32, 16}, {16, 32}, {16, 16}};
        double best = 1e300;
        for (auto& s : shapes) {
            // padded work plus a per-tile overhead worth ~64 K-steps of a 16x16 tile
            const double tiles = (double)ceil_div(P.m, s[0]) * (double)ceil_div(P.n, s[1]);
            const double work = tiles * s[0] * s[1] * (double)P.k + tiles * 16.0 * 16.0 * 64.0;
            if (work < best) { best = work; tm = s[0]; tn = s[1]; }
        }
    } else if (policy == 2) {
        tm = P.m <= 16 ? 16 : 32;
        tn = P.n <= 16 ? 16 : 32;
    }
    for (int j = 0; j < P.n; j += tn)
        for (int i = 0; i < P.m; i += tm) {
            Tile t;
            t.problem = pi;
            t.m0 = i;
            t.n0 = j;
            t.fm = (uint8_t)(tm / 16);
            t.fn = (uint8_t)(tn / 8);
            t.pad = 0;
            out.push_back(t);
        }
}

}  // namespace grp
}  // namespace cgb

struct cosma_gpu_grouped_plan {
    int device = 0;
    int count = 0;
    std::vector<cgb::grp::Problem> host_probs;
    cgb::DeviceBuffer probs, tiles, counter;
    int ntiles = 0;
    cgb::grp::Config cfg{0, 1, 4};
    double useful_flops = 0, padded_flops = 0;
    double tuned_ms = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t capture_stream = nullptr;
    cosma_gpu_oz_grouped_plan* oz = nullptr;    // the Ozaki-split form, when chosen
    cosma_gpu_oz2_grouped_plan* oz2 = nullptr;  // the Chinese-remainder form, when chosen
};

namespace cgb {
namespace grp {

std::mutex g_cache_mu;
std::map<std::string, Config> g_cache;  // batch signature -> tuned configuration

// Signature of a batch for the tuning cache: count plus a histogram of
// (log2 m, log2 n, log2 k, ops) buckets.
std::string signature(const std::vector<Problem>& ps) {
    std::map<int, int> h;
    auto lg = [](int x) { int r = 0; while ((1 << (r + 1)) <= x) ++r; return r; };
    for (auto& p : ps) h[((lg(p.m) * 16 + lg(p.n)) * 16 + lg(p.k)) * 4 + p.opa * 2 + p.opb]++;
    std::string s = std::to_string(ps.size()) + ":";
    for (auto& kv : h) s += std::to_string(kv.first) + "x" + std::to_string(kv.second) + ",";
    return s;
}

int build_tiles(cosma_gpu_grouped_plan* pl, const Config& cfg, cudaStream_t st) {
    std::vector<Tile> tiles;
    tiles.reserve(pl->count * 64);
    for (int i = 0; i < pl->count; ++i) problem_tiles(pl->host_probs[i], i, cfg.policy, tiles);
    // longest K first (largest tiles first on ties)
    std::stable_sort(tiles.begin(), tiles.end(), [&](const Tile& a, const Tile& b) {
        const int ka = pl->host_probs[a.problem].k, kb = pl->host_probs[b.problem].k;
        if (ka != kb) return ka > kb;
        return a.fm * a.fn > b.fm * b.fn;
    });
    pl->padded_flops = 0;
    for (auto& t : tiles) pl->padded_flops += 2.0 * 16 * t.fm * 8 * t.fn * pl->host_probs[t.problem].k;
    pl->ntiles = (int)tiles.size();
    CGB_CHECK(pl->tiles.reserve(std::max<size_t>(tiles.size(), 1) * sizeof(Tile), st));
    if (!tiles.empty())
        CGB_CUDA(cudaMemcpyAsync(pl->tiles.ptr, tiles.data(), tiles.size() * sizeof(Tile), cudaMemcpyHostToDevice, st));
    CGB_CUDA(cudaStreamSynchronize(st));
    pl->cfg = cfg;
    return COSMA_GPU_SUCCESS;
}

int grid_for(const Config& cfg) {
    int dev = 0, sms = kNumSMs;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, grouped_dmma_kernel, cfg.warps_per_cta * 32, 0);
    if (per_sm < 1) per_sm = 1;
    return sms * per_sm;
}

int launch(cosma_gpu_grouped_plan* pl, cudaStream_t st) {
    if (pl->ntiles == 0) return COSMA_GPU_SUCCESS;
    if (pl->cfg.dynamic_sched) CGB_CUDA(cudaMemsetAsync(pl->counter.ptr, 0, sizeof(int), st));
    const int grid = grid_for(pl->cfg);
    grouped_dmma_kernel<<<grid, pl->cfg.warps_per_cta * 32, 0, st>>>(
        (const Problem*)pl->probs.ptr, (const Tile*)pl->tiles.ptr, pl->ntiles, (int*)pl->counter.ptr,
        pl->cfg.dynamic_sched);
    CGB_CUDA(cudaGetLastError());
    return COSMA_GPU_SUCCESS;
}

int capture(cosma_gpu_grouped_plan* pl) {
    if (pl->exec) { cudaGraphExecDestroy(pl->exec); pl->exec = nullptr; }
    if (pl->graph) { cudaGraphDestroy(pl->graph); pl->graph = nullptr; }
    cudaStream_t cs = pl->capture_stream;
    CGB_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    int st = launch(pl, cs);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(cs, &g);
    if (st != COSMA_GPU_SUCCESS) { if (g) cudaGraphDestroy(g); return st; }
    if (e != cudaSuccess) return cuda_status(e, "cudaStreamEndCapture");
    pl->graph = g;
    CGB_CUDA(cudaGraphInstantiate(&pl->exec, g, 0));
    return COSMA_GPU_SUCCESS;
}

// Times each candidate configuration on the batch itself (two launches each,
// the second timed) and keeps the fastest.  C is overwritten during tuning,
// so problems whose beta != 0 are tuned on a scratch copy of their C.
int autotune(cosma_gpu_grouped_plan* pl, cudaStream_t st) {
    // beta != 0 problems would accumulate into C across trial runs: tune with
    // beta forced to 0 on the device copy, then restore.
    std::vector<Problem> tune = pl->host_probs;
    for (auto& p : tune) p.beta = 0.0;
    bool any_beta = false;
    for (auto& p : pl->host_probs) any_beta |= p.beta != 0.0;
    // C of beta != 0 problems must not be clobbered: save and restore it
    std::vector<DeviceBuffer> saved(any_beta ? pl->count : 0);
    if (any_beta) {
        for (int i = 0; i < pl->count; ++i) {
            const Problem& p = pl->host_probs[i];
            if (p.beta == 0.0 || p.m == 0 || p.n == 0) continue;
            CGB_CHECK(saved[i].reserve((size_t)p.m * p.n * 8, st));
            CGB_CUDA(cudaMemcpy2DAsync(saved[i].ptr, (size_t)p.m * 8, p.C, (size_t)p.ldc * 8, (size_t)p.m * 8, p.n,
                                       cudaMemcpyDeviceToDevice, st));
        }
    }
    CGB_CUDA(cudaMemcpyAsync(pl->probs.ptr, tune.data(), tune.size() * sizeof(Problem), cudaMemcpyHostToDevice, st));
    cudaEvent_t e0, e1;
    CGB_CUDA(cudaEventCreate(&e0));
    CGB_CUDA(cudaEventCreate(&e1));
    static const Config candidates[] = {
        {0, 1, 4}, {1, 1, 4}, {2, 1, 4}, {1, 0, 4}, {1, 1, 2}, {1, 1, 8},
    };
    float best = 1e30f;
    Config best_cfg = candidates[0];
    for (const Config& c : candidates) {
        CGB_CHECK(build_tiles(pl, c, st));
        CGB_CHECK(launch(pl, st));
        CGB_CUDA(cudaEventRecord(e0, st));
        CGB_CHECK(launch(pl, st));
        CGB_CUDA(cudaEventRecord(e1, st));
        CGB_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) { best = ms; best_cfg = c; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    pl->tuned_ms = best;
    CGB_CUDA(cudaMemcpyAsync(pl->probs.ptr, pl->host_probs.data(), pl->host_probs.size() * sizeof(Problem),
                             cudaMemcpyHostToDevice, st));
    if (any_beta) {
        for (int i = 0; i < pl->count; ++i) {
            const Problem& p = pl->host_probs[i];
            if (!saved[i].ptr) continue;
            CGB_CUDA(cudaMemcpy2DAsync(p.C, (size_t)p.ldc * 8, saved[i].ptr, (size_t)p.m * 8, (size_t)p.m * 8, p.n,
                                       cudaMemcpyDeviceToDevice, st));
        }
    }
    CGB_CUDA(cudaStreamSynchronize(st));
    return build_tiles(pl, best_cfg, st);
}

int normalise(int count, const cosma_gpu_gemm_problem* in, std::vector<Problem>& out, double* useful) {
    out.resize(count);
    *useful = 0;
    for (int i = 0; i < count; ++i) {
        const cosma_gpu_gemm_problem& q = in[i];
        Problem& p = out[i];
        p.opa = parse_op(q.transa);
        p.opb = parse_op(q.transb);
        if (p.opa < 0 || p.opb < 0)
            return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "grouped: problem " + std::to_string(i) + ": bad op");
        if (p.opa == 2) p.opa = 1;  // real data: conjugate transpose is a transpose
        if (p.opb == 2) p.opb = 1;
        if (q.m < 0 || q.n < 0 || q.k < 0)
            return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "grouped: problem " + std::to_string(i) + ": negative size");
        p.m = q.m; p.n = q.n; p.k = q.k;
        p.alpha = q.alpha; p.beta = q.beta;
        p.A = q.A; p.lda = q.lda; p.B = q.B; p.ldb = q.ldb; p.C = q.C; p.ldc = q.ldc;
        const int64_t ar = p.opa ? p.k : p.m, br = p.opb ? p.n : p.k;
        if (p.m > 0 && p.n > 0 &&
            (p.ldc < std::max(1, p.m) || (p.k > 0 && (p.lda < std::max<int64_t>(1, ar) || p.ldb < std::max<int64_t>(1, br)))))
            return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT,
                             "grouped: problem " + std::to_string(i) + ": leading dimension too small");
        if (((uintptr_t)p.A | (uintptr_t)p.B | (uintptr_t)p.C) % 8)
            return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "grouped: buffers must be 8-byte aligned");
        if (p.m > 0 && p.n > 0 && p.k == 0) p.alpha = 0.0;  // k == 0: C <- beta*C through the same kernel
        *useful += 2.0 * p.m * p.n * p.k;
    }
    return COSMA_GPU_SUCCESS;
}

}  // namespace grp
}  // namespace cgb

extern "C" {

cosma_gpu_grouped_plan* cosma_gpu_grouped_plan_create(int method, int count, const cosma_gpu_gemm_problem* problems,
                                                      int autotune, void* stream) {
    using namespace cgb;
    clear_error();
    if (method != COSMA_GPU_METHOD_AUTO && method != COSMA_GPU_METHOD_NATIVE && method != COSMA_GPU_METHOD_OZAKI &&
        method != COSMA_GPU_METHOD_OZAKI2) {
        set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "grouped: the native FP64 and the two Ozaki methods are implemented");
        return nullptr;
    }
    if (count < 0 || (count > 0 && !problems)) {
        set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "grouped: bad problem array");
        return nullptr;
    }
    if (method == COSMA_GPU_METHOD_OZAKI || method == COSMA_GPU_METHOD_OZAKI2) {
        auto* pl = new cosma_gpu_grouped_plan();
        pl->count = count;
        int s = COSMA_GPU_SUCCESS;
        if (method == COSMA_GPU_METHOD_OZAKI) pl->oz = oz_grouped_create(count, problems, autotune, (cudaStream_t)stream, &s);
        else pl->oz2 = oz2_grouped_create(count, problems, autotune, (cudaStream_t)stream, &s);
        if (!pl->oz && !pl->oz2) {
            delete pl;
            return nullptr;
        }
        return pl;
    }
    auto* pl = new cosma_gpu_grouped_plan();
    cudaStream_t st = (cudaStream_t)stream;
    int s = COSMA_GPU_SUCCESS;
    auto fail = [&](int code) { (void)code; cosma_gpu_grouped_plan_destroy(pl); return (cosma_gpu_grouped_plan*)nullptr; };
    if (cudaGetDevice(&pl->device) != cudaSuccess) { cuda_status(cudaGetLastError(), "cudaGetDevice"); return fail(0); }
    pl->count = count;
    if ((s = grp::normalise(count, problems, pl->host_probs, &pl->useful_flops))) return fail(s);
    if ((s = pl->probs.reserve(std::max<size_t>((size_t)count, 1) * sizeof(grp::Problem), st))) return fail(s);
    if ((s = pl->counter.reserve(sizeof(int), st))) return fail(s);
    if (count > 0 &&
        cudaMemcpyAsync(pl->probs.ptr, pl->host_probs.data(), (size_t)count * sizeof(grp::Problem),
                        cudaMemcpyHostToDevice, st) != cudaSuccess) {
        cuda_status(cudaGetLastError(), "cudaMemcpyAsync(problems)");
        return fail(0);
    }
    grp::Config cfg{1, 1, 4};  // default: per-problem shapes, dynamic longest-K-first
    bool tuned = false;
    const std::string sig = grp::signature(pl->host_probs);
    {
        std::lock_guard<std::mutex> lock(grp::g_cache_mu);
        auto it = grp::g_cache.find(sig);
        if (it != grp::g_cache.end()) { cfg = it->second; tuned = true; }
    }
    if (autotune && !tuned && count > 0) {
        if ((s = grp::autotune(pl, st))) return fail(s);
        std::lock_guard<std::mutex> lock(grp::g_cache_mu);
        grp::g_cache[sig] = pl->cfg;
    } else {
        if ((s = grp::build_tiles(pl, cfg, st))) return fail(s);
    }
    if (cudaStreamCreateWithFlags(&pl->capture_stream, cudaStreamNonBlocking) != cudaSuccess) {
        cuda_status(cudaGetLastError(), "cudaStreamCreate");
        return fail(0);
    }
    if ((s = grp::capture(pl))) return fail(s);
    return pl;
}

int cosma_gpu_grouped_plan_run(cosma_gpu_grouped_plan* pl, void* stream) {
    cgb::clear_error();
    if (!pl) return cgb::set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "grouped: null plan");
    if (pl->oz) return cgb::oz_grouped_run(pl->oz, (cudaStream_t)stream);
    if (pl->oz2) return cgb::oz2_grouped_run(pl->oz2, (cudaStream_t)stream);
    if (pl->ntiles == 0) return COSMA_GPU_SUCCESS;
    CGB_CUDA(cudaGraphLaunch(pl->exec, (cudaStream_t)stream));
    return COSMA_GPU_SUCCESS;
}

int cosma_gpu_grouped_plan_info(cosma_gpu_grouped_plan* pl, cosma_gpu_grouped_info* info) {
    if (!pl || !info) return cgb::set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "grouped: null argument");
    if (pl->oz) {
        cgb::oz_grouped_info(pl->oz, info);
        return COSMA_GPU_SUCCESS;
    }
    if (pl->oz2) {
        cgb::oz2_grouped_info(pl->oz2, info);
        return COSMA_GPU_SUCCESS;
    }
    info->tiles = pl->ntiles;
    info->tile_policy = pl->cfg.policy;
    info->dynamic_schedule = pl->cfg.dynamic_sched;
    info->warps_per_cta = pl->cfg.warps_per_cta;
    info->useful_flops = pl->useful_flops;
    info->padded_flops = pl->padded_flops;
    info->tuned_ms = pl->tuned_ms;
    return COSMA_GPU_SUCCESS;
}

int cosma_gpu_grouped_plan_slices(cosma_gpu_grouped_plan* pl, int* slices) {
    if (!pl || !slices) return cgb::set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "grouped: null argument");
    if (pl->oz) return cgb::oz_grouped_slices(pl->oz, slices);
    if (pl->oz2) return cgb::oz2_grouped_slices(pl->oz2, slices);
    for (int i = 0; i < pl->count; ++i) slices[i] = 0;
    return COSMA_GPU_SUCCESS;
}

void cosma_gpu_grouped_plan_destroy(cosma_gpu_grouped_plan* pl) {
    if (!pl) return;
    if (pl->oz) cgb::oz_grouped_destroy(pl->oz);
    if (pl->oz2) cgb::oz2_grouped_destroy(pl->oz2);
    if (pl->exec) cudaGraphExecDestroy(pl->exec);
    if (pl->graph) cudaGraphDestroy(pl->graph);
    if (pl->capture_stream) cudaStreamDestroy(pl->capture_stream);
    cudaGetLastError();
    delete pl;
}

int cosma_gpu_dgemm_grouped_device(int method, int count, const cosma_gpu_gemm_problem* problems, void* stream) {
    cosma_gpu_grouped_plan* pl = cosma_gpu_grouped_plan_create(method, count, problems, 0, stream);
    if (!pl) return cosma_gpu_last_error();
    int s = cosma_gpu_grouped_plan_run(pl, stream);
    if (s == COSMA_GPU_SUCCESS && cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess)
        s = cgb::cuda_status(cudaGetLastError(), "cudaStreamSynchronize");
    cosma_gpu_grouped_plan_destroy(pl);
    return s;
}

}  // extern "C"
