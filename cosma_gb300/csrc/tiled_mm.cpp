// Tiled-MM-compatible GEMM engine: the handle, the host<->HBM tile streamer
// and the COSMA local_multiply entry points.
//
// Reference behaviour (Tiled-MM v2.3.2 as used by COSMA):
//  * gpu::make_context<T>(streams, tile_m, tile_n, tile_k) creates a handle
//    owning device tile buffers and streams (src/cosma/context.cpp:24-25,45);
//    device memory streams*(tm*tk + tk*tn + tm*tn) elements (README.md:362-365).
//  * gpu::gemm(handle, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc,
//    pin, copy_c_back) computes C = alpha*op(A)*op(B) + beta*C on host
//    matrices: C is cut into tm x tn tiles and K into tk slabs, tiles are
//    dealt round-robin to the streams, each tile copies its A/B slabs in,
//    multiplies (beta on the first K slab, 1 afterwards) and copies C back
//    (call site src/cosma/local_multiply.cpp:245-260).
//  * cosma::local_multiply pins A, B, C once (memory_pool::pin ->
//    cudaHostRegister, re-registered when a buffer grows;
//    src/cosma/pinned_buffers.cpp:6-35) and calls gpu::gemm with 'N','N'
//    and ld = m, k, m (src/cosma/local_multiply.cpp:300-381).
//
// GB300 design: one process drives one GPU with 280 GB of HBM, so the
// default tile covers any in-core problem up to 32768 in a single piece and
// the matrices cross the C2C link exactly once; larger problems stream tiles
// over several streams so that copies of one tile overlap the GEMM of
// another.  Device pointers are detected and used in place (no copies).
// On a Grace host the GPU reaches pageable memory through the host's page
// tables: tiles of pageable matrices are then copied in place by a device
// kernel and the pin flag registers nothing.
#include "common.cuh"
#include "runtime.hpp"

#include <algorithm>
#include <map>
#include <mutex>
#include <vector>

struct cosma_gpu_mm_handle {
    cgb::Scalar scalar = cgb::Scalar::D;
    int n_streams = 3, tile_m = 0, tile_n = 0, tile_k = 0;
    int method = COSMA_GPU_METHOD_AUTO, slices = 0;
    int device = 0;
    std::vector<cudaStream_t> streams;
    std::vector<cgb::DeviceBuffer> bufA, bufB, bufC;
    cgb::DeviceBuffer full_c;
    void* last_device_c = nullptr;
    std::map<uintptr_t, size_t> pinned;  // registered host ranges (base -> bytes)
    std::mutex mu;
    cosma_gpu_ozaki_info last_info{0, 0, 0, 0, 0.0, 0.0, 0.0};
    int64_t last_h2d_bytes = 0, last_d2h_bytes = 0;
    int last_overlapped = 0;  // the last call ran in an overlapped one-step form
    cudaEvent_t ev_ready[2] = {}, ev_free[2] = {}, ev_cin[2] = {}, ev_cdone[2] = {}, ev_cout[2] = {};
};

namespace cgb {
namespace {

bool is_device_ptr(const void* p) {
    if (!p) return false;
    cudaPointerAttributes at;
    cudaError_t e = cudaPointerGetAttributes(&at, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// Page-locks [ptr, ptr+bytes) for the copies of one call.
//
// The reference keeps registrations until its context is destroyed and
// re-registers a pointer only when it grows (pinned_buffers::add,
// src/cosma/pinned_buffers.cpp:6-35).  That is safe for COSMA's own memory
// pool, which owns the buffers, but not for callers that free a buffer and
// get a new one at the same address: the driver would keep the stale
// registration.  So registrations are scoped to the call by default
// (registered ranges are recorded in `scoped` and released by the caller of
// pin_range); COSMA_GPU_PIN_CACHE=ON restores the reference's
// keep-until-destroyed policy for callers whose buffers outlive the handle.
// Memory that its owner already page-locked is used as it is.
int pin_range(cosma_gpu_mm_handle* h, const void* ptr, size_t bytes, std::vector<void*>& scoped) {
    if (!ptr || bytes == 0) return COSMA_GPU_SUCCESS;
    static const bool cache = env_bool("COSMA_GPU_PIN_CACHE", false);
    uintptr_t key = (uintptr_t)ptr;
    if (cache) {
        auto it = h->pinned.find(key);
        if (it != h->pinned.end()) {
            if (it->second >= bytes) return COSMA_GPU_SUCCESS;
            cudaHostUnregister((void*)ptr);
            cudaGetLastError();
            h->pinned.erase(it);
        }
    }
    cudaError_t e =
        inject_fault(kFaultHostRegister) ? cudaErrorMemoryAllocation : cudaHostRegister((void*)ptr, bytes, cudaHostRegisterDefault);
    if (e == cudaErrorHostMemoryAlreadyRegistered) {  // page-locked by its owner
        cudaGetLastError();
        return COSMA_GPU_SUCCESS;
    }
    if (e != cudaSuccess) {
        // Pinning is an optimisation: memory that cannot be registered still
        // moves through staged pageable copies.
        cudaGetLastError();
        if (env_verbose()) std::fprintf(stderr, "[cosma_gb300] cudaHostRegister failed: %s\n", cudaGetErrorString(e));
        return COSMA_GPU_SUCCESS;
    }
    if (cache) h->pinned[key] = bytes;
    else scoped.push_back((void*)ptr);
    return COSMA_GPU_SUCCESS;
}

void unpin_scoped(std::vector<void*>& scoped) {
    for (void* p : scoped) cudaHostUnregister(p);
    scoped.clear();
    cudaGetLastError();
}

size_t span_bytes(int64_t rows, int64_t cols, int64_t ld, size_t es) {
    if (rows <= 0 || cols <= 0) return 0;
    return ((size_t)(cols - 1) * (size_t)ld + (size_t)rows) * es;
}

// Tile copies run beside the GEMMs of other steps: page-locked host memory
// goes through the copy engines (copy kernels would hold SMs the persistent
// GEMMs wait for), pageable memory through the in-place copy kernel.
int copy2d(void* dst, int64_t dld, const void* src, int64_t sld, int64_t rows, int64_t cols, size_t es,
           cudaMemcpyKind kind, cudaStream_t s) {
    if (rows == 0 || cols == 0) return COSMA_GPU_SUCCESS;
    return copy_2d_overlapped(dst, (size_t)dld * es, src, (size_t)sld * es, (size_t)rows * es, (size_t)cols, kind, s);
}

bool is_zero(const double* v, Scalar s) { return v[0] == 0.0 && (!scalar_complex(s) || v[1] == 0.0); }
bool is_one(const double* v, Scalar s) { return v[0] == 1.0 && (!scalar_complex(s) || v[1] == 0.0); }

}  // namespace

int handle_init(cosma_gpu_mm_handle* h) {
    CGB_CUDA(cudaGetDevice(&h->device));
    h->streams.resize(h->n_streams);
    for (auto& s : h->streams) CGB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    // two operand slots and two C slots (sized once: DeviceBuffer is not movable)
    h->bufA.resize(2);
    h->bufB.resize(2);
    h->bufC.resize(2);
    for (int i = 0; i < 2; ++i)
        for (cudaEvent_t* e : {&h->ev_ready[i], &h->ev_free[i], &h->ev_cin[i], &h->ev_cdone[i], &h->ev_cout[i]})
            CGB_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    return COSMA_GPU_SUCCESS;
}

int tmm_stream_tiles(cosma_gpu_mm_handle* h, Scalar sc, char ta, char tb, int opa, int opb, int64_t m, int64_t n,
                     int64_t k, const double* alpha, const void* A, int64_t lda, const void* B, int64_t ldb,
                     const double* beta, void* C, int64_t ldc, bool dA, bool dB, bool dC, bool trivial,
                     bool copy_c_back, cosma_gpu_ozaki_info* info);

// C = alpha*op(A)*op(B) + beta*C with any mix of host and device pointers.
int tmm_gemm(cosma_gpu_mm_handle* h, Scalar sc, char ta, char tb, int64_t m, int64_t n, int64_t k,
             const double* alpha, const void* A, int64_t lda, const void* B, int64_t ldb, const double* beta,
             void* C, int64_t ldc, bool pin, bool copy_c_back) {
    if (!h) return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "gemm: null handle");
    if (h->scalar != sc) return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "gemm: handle scalar type mismatch");
    const int opa = parse_op(ta), opb = parse_op(tb);
    if (opa < 0 || opb < 0) return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "gemm: op must be N, T or C");
    if (m < 0 || n < 0 || k < 0) return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "gemm: negative size");
    if (m == 0 || n == 0) return COSMA_GPU_SUCCESS;
    const int64_t a_rows = opa == 0 ? m : k, a_cols = opa == 0 ? k : m;
    const int64_t b_rows = opb == 0 ? k : n, b_cols = opb == 0 ? n : k;
    if (ldc < std::max<int64_t>(1, m) || (k > 0 && (lda < std::max<int64_t>(1, a_rows) || ldb < std::max<int64_t>(1, b_rows))))
        return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "gemm: leading dimension too small");

    std::lock_guard<std::mutex> lock(h->mu);
    CGB_CUDA(cudaSetDevice(h->device));
    const size_t es = scalar_bytes(sc);
    const bool dA = is_device_ptr(A), dB = is_device_ptr(B), dC = is_device_ptr(C);
    const bool trivial = (k == 0) || is_zero(alpha, sc);
    cosma_gpu_ozaki_info* info = &h->last_info;
    *info = cosma_gpu_ozaki_info{0, 0, 0, 0, 0.0, 0.0, 0.0, 0, 0};
    h->last_overlapped = 0;

    if (trivial && is_one(beta, sc)) return COSMA_GPU_SUCCESS;  // C unchanged
    if (dC && (trivial || (dA && dB))) {  // everything already in HBM
        GemmDesc g = make_gemm_desc(sc, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
        CGB_CHECK(gemm_device(g, h->method, h->slices, h->streams[0], info));
        CGB_CUDA(cudaStreamSynchronize(h->streams[0]));
        h->last_device_c = C;
        return COSMA_GPU_SUCCESS;
    }

    std::vector<void*> scoped;
    // Where kernels copy pageable memory in place, registering it only adds
    // cost: cudaHostRegister of 6 GB took 70 to 800 ms per call, while the
    // in-place copies run at the link's rate (16384^3 Ozaki DGEMM from
    // pageable arrays: 315 ms unregistered against 354 to 1083 ms registered).
    if (pin && !host_direct_available()) {
        if (!dA && !trivial) pin_range(h, A, span_bytes(a_rows, a_cols, lda, es), scoped);
        if (!dB && !trivial) pin_range(h, B, span_bytes(b_rows, b_cols, ldb, es), scoped);
        if (!dC) pin_range(h, C, span_bytes(m, n, ldc, es), scoped);
    }
    int status = tmm_stream_tiles(h, sc, ta, tb, opa, opb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, dA, dB, dC,
                                  trivial, copy_c_back, info);
    unpin_scoped(scoped);
    return status;
}

// The host<->HBM streamer behind tmm_gemm (host or mixed pointers).
//
// Work is a sequence of steps (C tile, K slab).  Three streams play fixed
// roles - H2D copies, GEMMs, D2H copies - and two rings of device buffers
// (operand slots for A/B slabs, C slots for C tiles) are chained with events:
// the copies of step i+1 are enqueued before the GEMM of step i is called, so
// they run while it computes even when the GEMM call itself blocks the host
// (the Ozaki path reads its slice statistics back), and the D2H of a finished
// C tile overlaps the next tile.  Tiles never exceed the handle's limits and
// shrink until the rings fit in 60% of free HBM.
int tmm_stream_tiles(cosma_gpu_mm_handle* h, Scalar sc, char ta, char tb, int opa, int opb, int64_t m, int64_t n,
                     int64_t k, const double* alpha, const void* A, int64_t lda, const void* B, int64_t ldb,
                     const double* beta, void* C, int64_t ldc, bool dA, bool dB, bool dC, bool trivial,
                     bool copy_c_back, cosma_gpu_ozaki_info* info) {
    const size_t es = scalar_bytes(sc);
    constexpr int R = 2;  // operand slots and C slots
    int64_t tm = std::min<int64_t>(m, h->tile_m), tn = std::min<int64_t>(n, h->tile_n);
    int64_t tk = std::min<int64_t>(std::max<int64_t>(k, 1), h->tile_k);
    size_t free_b = 0, total_b = 0;
    CGB_CUDA(cudaMemGetInfo(&free_b, &total_b));
    size_t have = 0;
    for (int s = 0; s < R; ++s) have += h->bufA[s].bytes + h->bufB[s].bytes + h->bufC[s].bytes;
    for (;;) {
        const size_t per = (R * ((dA || trivial ? 0 : (size_t)tm * tk) + (dB || trivial ? 0 : (size_t)tk * tn)) +
                            R * (dC ? 0 : (size_t)tm * tn)) * es;
        if (per <= (size_t)(0.6 * (double)(free_b + have)) || (tm <= 256 && tn <= 256 && tk <= 256)) break;
        if (tk >= tm && tk >= tn) tk = (tk + 1) / 2;
        else if (tm >= tn) tm = (tm + 1) / 2;
        else tn = (tn + 1) / 2;
    }
    const int64_t ntm = ceil_div(m, tm), ntn = ceil_div(n, tn), ntk = trivial ? 1 : ceil_div(k, tk);
    const int64_t ntiles = ntm * ntn, nsteps = ntiles * ntk;
    const bool keep_on_device = !dC && !copy_c_back;
    const bool crt = h->method == COSMA_GPU_METHOD_OZAKI2 && (sc == Scalar::D || sc == Scalar::Z);
    // One step on host operands with the Chinese-remainder method (double, or
    // complex with real alpha and beta): the overlapped form (op(A) / op(B) panels copied by the copy engines while
    // earlier blocks compute, C blocks copied out while later ones do) where
    // it applies; 16384^3 from page-locked arrays took 97 to 99 ms per call in
    // it against 116 ms in the one-step form.  Its copies are issued by a
    // worker thread, so pageable arrays (whose copies return only once done)
    // overlap too.
    const bool overlap = env_bool("COSMA_GPU_OZAKI2_OVERLAP", true);
    // With two streams the C blocks leave on the copy stream, behind every
    // panel copy (those end long before the first block is reconstructed).
    if (overlap && crt && !dA && !dB && !dC && !trivial && !keep_on_device && nsteps == 1 && h->streams.size() >= 2) {
        const GemmDesc g = make_gemm_desc(sc, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
        cosma_gpu_ozaki_info oi{0, 0, 0, 0, 0.0, 0.0, 0.0, 0, 0};
        int64_t h2d = 0, d2h = 0;
        bool taken = false;
        const size_t S = h->streams.size();
        const int st = ozaki2_gemm_host(g, h->slices, h->streams[0], h->streams[1],
                                         h->streams[std::min<size_t>(2, S - 1)], &oi, &h2d, &d2h, &taken);
        // a refused allocation before C is touched: the one-step form below
        // needs less memory
        if (st != COSMA_GPU_SUCCESS && (taken || st != COSMA_GPU_ERROR_OUT_OF_MEMORY)) return st;
        if (st != COSMA_GPU_SUCCESS) clear_error();
        if (taken && st == COSMA_GPU_SUCCESS) {
            *info = oi;
            h->last_h2d_bytes = h2d;
            h->last_d2h_bytes = d2h;
            h->last_device_c = nullptr;
            h->last_overlapped = 1;
            return COSMA_GPU_SUCCESS;
        }
    }
    // One step on host operands with 3xBF16 (float under the AUTO or BF16X3
    // method): the same overlapped form around the slice splits and block
    // GEMMs (16384^3 from pinned buffers: 34.9 to 35.6 ms per call against 44
    // ms with the copies before and after the GEMM).
    const bool b3 = sc == Scalar::S && (h->method == COSMA_GPU_METHOD_AUTO || h->method == COSMA_GPU_METHOD_BF16X3);
    if (b3 && env_bool("COSMA_GPU_BF16X3_OVERLAP", true) && !dA && !dB && !dC && !trivial && !keep_on_device &&
        nsteps == 1 && h->streams.size() >= 2) {
        const GemmDesc g = make_gemm_desc(sc, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
        int64_t h2d = 0, d2h = 0;
        bool taken = false;
        const size_t S = h->streams.size();
        const int st = bf16x3_sgemm_host(g, h->streams[0], h->streams[1], h->streams[std::min<size_t>(2, S - 1)],
                                         &h2d, &d2h, &taken);
        if (st != COSMA_GPU_SUCCESS && (taken || st != COSMA_GPU_ERROR_OUT_OF_MEMORY)) return st;
        if (st != COSMA_GPU_SUCCESS) clear_error();
        if (taken && st == COSMA_GPU_SUCCESS) {
            h->last_h2d_bytes = h2d;
            h->last_d2h_bytes = d2h;
            h->last_device_c = nullptr;
            h->last_overlapped = 1;
            return COSMA_GPU_SUCCESS;
        }
    }
    // One step with the Chinese-remainder method: its reconstruction kernel
    // writes (and, for beta != 0, reads) C in host memory directly where the
    // device reaches it, so the write-back overlaps that kernel instead of
    // following it as a separate copy, and no C slot is needed.
    const bool direct_c = crt && !dC && !keep_on_device && !trivial && nsteps == 1 &&
                          prepare_direct_host(C, (size_t)ldc * es, (size_t)m * es, (size_t)n, true);
    for (int s = 0; s < R; ++s) {
        if (!dA && !trivial) CGB_CHECK(h->bufA[s].reserve((size_t)tm * tk * es, h->streams[0]));
        if (!dB && !trivial) CGB_CHECK(h->bufB[s].reserve((size_t)tk * tn * es, h->streams[0]));
        if (!dC && !direct_c) CGB_CHECK(h->bufC[s].reserve((size_t)tm * tn * es, h->streams[0]));
    }
    if (keep_on_device) CGB_CHECK(h->full_c.reserve((size_t)m * n * es, h->streams[0]));
    CGB_CUDA(cudaDeviceSynchronize());  // buffers from any earlier call are idle

    const int S = (int)h->streams.size();
    cudaStream_t cs = h->streams[0], hs = h->streams[std::min(1, S - 1)], ds = h->streams[std::min(2, S - 1)];
    cudaEvent_t* ev_ready = h->ev_ready;    // operand slot filled
    cudaEvent_t* ev_free = h->ev_free;      // operand slot read by its GEMM
    cudaEvent_t* ev_cin = h->ev_cin;        // C slot filled (beta != 0) / free to overwrite
    cudaEvent_t* ev_cdone = h->ev_cdone;    // C slot final
    cudaEvent_t* ev_cout = h->ev_cout;      // C slot drained to its destination
    bool slot_used[R] = {false, false}, cslot_used[R] = {false, false};
    h->last_h2d_bytes = 0;
    h->last_overlapped = 0;
    h->last_d2h_bytes = 0;
    const double one[2] = {1.0, 0.0};
    const bool beta_zero = is_zero(beta, sc);

    auto tile_of = [&](int64_t step, int64_t& i0, int64_t& j0, int64_t& mi, int64_t& nj, int64_t& l0, int64_t& kk) {
        const int64_t t = step / ntk, kt = step % ntk;
        const int64_t ti = t % ntm, tj = t / ntm;
        i0 = ti * tm; j0 = tj * tn;
        mi = std::min(tm, m - i0); nj = std::min(tn, n - j0);
        l0 = kt * tk; kk = trivial ? 0 : std::min(tk, k - l0);
    };
    auto cdev_of = [&](int64_t step, int64_t i0, int64_t j0, int64_t& cld) -> char* {
        if (dC || direct_c) { cld = ldc; return (char*)C + (i0 + j0 * ldc) * es; }
        const int64_t t = step / ntk;
        int64_t mi = std::min(tm, m - i0);
        cld = mi;
        return (char*)h->bufC[t % R].ptr;
    };
    // device pointers of the op(A) / op(B) slabs of a step (issuing the H2D copies when host-resident)
    auto issue_copies = [&](int64_t step) -> int {
        int64_t i0, j0, mi, nj, l0, kk;
        tile_of(step, i0, j0, mi, nj, l0, kk);
        const int r = (int)(step % R);
        const int64_t t = step / ntk, kt = step % ntk;
        const int c = (int)(t % R);
        if (kt == 0 && !dC && !direct_c && !beta_zero) {  // C tile comes in once, before its first K slab
            if (cslot_used[c]) CGB_CUDA(cudaStreamWaitEvent(hs, ev_cout[c], 0));
            CGB_CHECK(copy2d(h->bufC[c].ptr, mi, (const char*)C + (i0 + j0 * ldc) * es, ldc, mi, nj, es,
                             cudaMemcpyHostToDevice, hs));
            h->last_h2d_bytes += mi * nj * es;
            CGB_CUDA(cudaEventRecord(ev_cin[c], hs));
        }
        if (trivial) return COSMA_GPU_SUCCESS;
        if (slot_used[r] && (!dA || !dB)) CGB_CUDA(cudaStreamWaitEvent(hs, ev_free[r], 0));
        if (!dA) {
            if (opa == 0) CGB_CHECK(copy2d(h->bufA[r].ptr, mi, (const char*)A + (i0 + l0 * lda) * es, lda, mi, kk, es,
                                           cudaMemcpyHostToDevice, hs));
            else CGB_CHECK(copy2d(h->bufA[r].ptr, kk, (const char*)A + (l0 + i0 * lda) * es, lda, kk, mi, es,
                                  cudaMemcpyHostToDevice, hs));
            h->last_h2d_bytes += mi * kk * es;
        }
        if (!dB) {
            if (opb == 0) CGB_CHECK(copy2d(h->bufB[r].ptr, kk, (const char*)B + (l0 + j0 * ldb) * es, ldb, kk, nj, es,
                                           cudaMemcpyHostToDevice, hs));
            else CGB_CHECK(copy2d(h->bufB[r].ptr, nj, (const char*)B + (j0 + l0 * ldb) * es, ldb, nj, kk, es,
                                  cudaMemcpyHostToDevice, hs));
            h->last_h2d_bytes += kk * nj * es;
        }
        CGB_CUDA(cudaEventRecord(ev_ready[r], hs));
        slot_used[r] = true;
        return COSMA_GPU_SUCCESS;
    };
    auto compute = [&](int64_t step) -> int {
        int64_t i0, j0, mi, nj, l0, kk;
        tile_of(step, i0, j0, mi, nj, l0, kk);
        const int r = (int)(step % R);
        const int64_t t = step / ntk, kt = step % ntk;
        const int c = (int)(t % R);
        int64_t cld;
        char* cdev = cdev_of(step, i0, j0, cld);
        if (kt == 0 && !dC && !direct_c) {
            if (!beta_zero) CGB_CUDA(cudaStreamWaitEvent(cs, ev_cin[c], 0));
            else if (cslot_used[c]) CGB_CUDA(cudaStreamWaitEvent(cs, ev_cout[c], 0));  // slot drained before overwrite
        }
        if (trivial) {
            CGB_CHECK(scale_matrix_device(sc, mi, nj, beta, cdev, cld, cs));
        } else {
            if (!dA || !dB) CGB_CUDA(cudaStreamWaitEvent(cs, ev_ready[r], 0));
            const char* adev;
            int64_t ald;
            if (dA) { adev = (const char*)A + (opa == 0 ? (i0 + l0 * lda) : (l0 + i0 * lda)) * es; ald = lda; }
            else { adev = (const char*)h->bufA[r].ptr; ald = opa == 0 ? mi : kk; }
            const char* bdev;
            int64_t bld;
            if (dB) { bdev = (const char*)B + (opb == 0 ? (l0 + j0 * ldb) : (j0 + l0 * ldb)) * es; bld = ldb; }
            else { bdev = (const char*)h->bufB[r].ptr; bld = opb == 0 ? kk : nj; }
            GemmDesc g = make_gemm_desc(sc, ta, tb, mi, nj, kk, alpha, adev, ald, bdev, bld, kt == 0 ? beta : one,
                                        cdev, cld);
            cosma_gpu_ozaki_info ti_info;
            CGB_CHECK(gemm_device(g, h->method, h->slices, cs, &ti_info));
            if (ti_info.slices || ti_info.fallback_native) *info = ti_info;
            CGB_CUDA(cudaEventRecord(ev_free[r], cs));
        }
        if (kt == ntk - 1 && direct_c) h->last_d2h_bytes += mi * nj * es;  // written in place by the GEMM
        if (kt == ntk - 1 && !dC && !direct_c) {  // tile final: drain it on the D2H stream
            CGB_CUDA(cudaEventRecord(ev_cdone[c], cs));
            CGB_CUDA(cudaStreamWaitEvent(ds, ev_cdone[c], 0));
            if (keep_on_device) {
                CGB_CHECK(copy2d((char*)h->full_c.ptr + (i0 + j0 * m) * es, m, cdev, cld, mi, nj, es,
                                 cudaMemcpyDeviceToDevice, ds));
            } else {
                CGB_CHECK(copy2d((char*)C + (i0 + j0 * ldc) * es, ldc, cdev, cld, mi, nj, es, cudaMemcpyDeviceToHost,
                                 ds));
                h->last_d2h_bytes += mi * nj * es;
            }
            CGB_CUDA(cudaEventRecord(ev_cout[c], ds));
            cslot_used[c] = true;
        }
        return COSMA_GPU_SUCCESS;
    };

    int status = COSMA_GPU_SUCCESS;
    for (int64_t i = 0; i < std::min<int64_t>(R - 1, nsteps) && status == COSMA_GPU_SUCCESS; ++i)
        status = issue_copies(i);
    for (int64_t i = 0; i < nsteps && status == COSMA_GPU_SUCCESS; ++i) {
        if (i + R - 1 < nsteps) status = issue_copies(i + R - 1);
        if (status == COSMA_GPU_SUCCESS) status = compute(i);
    }
    for (cudaStream_t s : {cs, hs, ds}) {
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess && status == COSMA_GPU_SUCCESS) status = cuda_status(e, "cudaStreamSynchronize");
    }
    h->last_device_c = dC ? C : (keep_on_device ? h->full_c.ptr : nullptr);
    return status;
}

}  // namespace cgb

// ------------------------------------------------------------------ C ABI
namespace {

bool parse_scalar(char c, cgb::Scalar* s) {
    switch (c) {
        case 's': case 'S': *s = cgb::Scalar::S; return true;
        case 'd': case 'D': *s = cgb::Scalar::D; return true;
        case 'c': case 'C': *s = cgb::Scalar::C; return true;
        case 'z': case 'Z': *s = cgb::Scalar::Z; return true;
    }
    return false;
}

std::mutex g_singleton_mu;
cosma_gpu_mm_handle* g_singletons[4] = {nullptr, nullptr, nullptr, nullptr};
bool g_pin_default = true;

}  // namespace

extern "C" {

cosma_gpu_mm_handle* cosma_gpu_tmm_make_context(char scalar, int streams, int tile_m, int tile_n, int tile_k) {
    cgb::clear_error();
    cgb::Scalar s;
    if (!parse_scalar(scalar, &s)) {
        cgb::set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "make_context: scalar must be s, d, c or z");
        return nullptr;
    }
    auto* h = new cosma_gpu_mm_handle();
    h->scalar = s;
    h->n_streams = streams > 0 ? streams : cgb::default_streams();
    if (h->n_streams < 1) h->n_streams = 1;
    h->tile_m = tile_m > 0 ? tile_m : cgb::default_tile_m();
    h->tile_n = tile_n > 0 ? tile_n : cgb::default_tile_n();
    h->tile_k = tile_k > 0 ? tile_k : cgb::default_tile_k();
    h->method = cgb::default_method();
    if (cgb::handle_init(h) != COSMA_GPU_SUCCESS) {
        delete h;
        return nullptr;
    }
    return h;
}

void cosma_gpu_tmm_destroy_context(cosma_gpu_mm_handle* h) {
    if (!h) return;
    {
        std::lock_guard<std::mutex> lock(h->mu);
        cudaSetDevice(h->device);
        for (auto s : h->streams) cudaStreamSynchronize(s);
        for (auto& b : h->bufA) b.release();
        for (auto& b : h->bufB) b.release();
        for (auto& b : h->bufC) b.release();
        h->full_c.release();
        for (auto& kv : h->pinned) cudaHostUnregister((void*)kv.first);
        h->pinned.clear();
        for (auto s : h->streams) {
            cgb::ozaki_release_stream(s);
            cgb::ozaki2_release_stream(s);
            cgb::bf16x3_release_stream(s);
            cudaStreamDestroy(s);
        }
        for (int i = 0; i < 2; ++i)
            for (cudaEvent_t e : {h->ev_ready[i], h->ev_free[i], h->ev_cin[i], h->ev_cdone[i], h->ev_cout[i]})
                if (e) cudaEventDestroy(e);
        cudaGetLastError();
    }
    delete h;
}

int cosma_gpu_tmm_set_method(cosma_gpu_mm_handle* h, int method, int slices) {
    cgb::clear_error();
    if (!h) return cgb::set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "set_method: null handle");
    if (method < COSMA_GPU_METHOD_AUTO || method > COSMA_GPU_METHOD_OZAKI2)
        return cgb::set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "set_method: unknown method");
    std::lock_guard<std::mutex> lock(h->mu);
    h->method = method;
    h->slices = slices;
    return COSMA_GPU_SUCCESS;
}

// Device bytes a handle needs at square tiles of edge t: the double-buffered
// A, B and C tile slots, plus the method's scratch at its worst case (16
// digit slices per operand and the per-CTA partial sums for the Ozaki form,
// three BF16 slices for 3xBF16).
static double tmm_footprint(cgb::Scalar s, int method, double t) {
    const double es = (double)cgb::scalar_bytes(s);
    double bytes = 2.0 * 3.0 * t * t * es;
    if (method == COSMA_GPU_METHOD_AUTO) method = s == cgb::Scalar::S ? COSMA_GPU_METHOD_BF16X3 : COSMA_GPU_METHOD_NATIVE;
    if ((method == COSMA_GPU_METHOD_OZAKI || method == COSMA_GPU_METHOD_OZAKI2) && s == cgb::Scalar::S)
        method = COSMA_GPU_METHOD_BF16X3;
    // residue matrices (BF16) of both operands and residue bytes of C, at the largest modulus count
    if (method == COSMA_GPU_METHOD_OZAKI2 && s == cgb::Scalar::D) bytes += 28.0 * (2.0 * 2.0 + 1.0) * t * t;
    if (method == COSMA_GPU_METHOD_OZAKI2 && s == cgb::Scalar::Z) bytes += 28.0 * 14.0 * t * t + 16.0 * t * t;
    if (method == COSMA_GPU_METHOD_OZAKI && s == cgb::Scalar::D)
        bytes += 16.0 * 2.0 * t * t + 152.0 * 128 * 256 * 16;
    if (method == COSMA_GPU_METHOD_OZAKI && s == cgb::Scalar::Z)
        bytes += 16.0 * 6.0 * t * t + 152.0 * 128 * 256 * 16 + 16.0 * t * t;
    if (method == COSMA_GPU_METHOD_BF16X3 && s == cgb::Scalar::S) bytes += 3.0 * 2.0 * 2.0 * t * t;
    return bytes;
}

// The largest square tile edge (a multiple of 256) whose handle footprint
// fits in `bytes`: the one-GPU counterpart of COSMA's sequential splits
// under a memory limit (src/cosma/strategy.cpp:404-440), which cut a problem
// into steps that fit the memory; here the tile streamer runs the steps.
int cosma_gpu_tmm_tiles_for_memory(char scalar, int method, int64_t bytes, int* tile_m, int* tile_n, int* tile_k) {
    cgb::clear_error();
    cgb::Scalar s;
    if (!parse_scalar(scalar, &s) || !tile_m || !tile_n || !tile_k)
        return cgb::set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "tiles_for_memory: bad argument");
    if (method < COSMA_GPU_METHOD_AUTO || method > COSMA_GPU_METHOD_OZAKI2)
        return cgb::set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "tiles_for_memory: unknown method");
    int64_t best = 0;
    for (int64_t t = 256; t <= (1 << 20); t += 256) {
        if (tmm_footprint(s, method, (double)t) > (double)bytes) break;
        best = t;
    }
    if (!best)
        return cgb::set_error(COSMA_GPU_ERROR_OUT_OF_MEMORY,
                              "tiles_for_memory: not even 256 x 256 tiles fit in " + std::to_string(bytes) + " bytes");
    *tile_m = *tile_n = *tile_k = (int)std::min<int64_t>(best, 1 << 30);
    return COSMA_GPU_SUCCESS;
}

int cosma_gpu_tmm_set_memory_limit(cosma_gpu_mm_handle* h, int64_t bytes) {
    cgb::clear_error();
    if (!h) return cgb::set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "set_memory_limit: null handle");
    std::lock_guard<std::mutex> lock(h->mu);
    const char sc = h->scalar == cgb::Scalar::S ? 's' : h->scalar == cgb::Scalar::D ? 'd'
                  : h->scalar == cgb::Scalar::C ? 'c' : 'z';
    int tm = 0, tn = 0, tk = 0;
    CGB_CHECK(cosma_gpu_tmm_tiles_for_memory(sc, h->method, bytes, &tm, &tn, &tk));
    h->tile_m = tm;
    h->tile_n = tn;
    h->tile_k = tk;
    return COSMA_GPU_SUCCESS;
}

int cosma_gpu_tmm_tiles(cosma_gpu_mm_handle* h, int* tile_m, int* tile_n, int* tile_k) {
    if (!h || !tile_m || !tile_n || !tile_k) return cgb::set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "tiles: null");
    std::lock_guard<std::mutex> lock(h->mu);
    *tile_m = h->tile_m;
    *tile_n = h->tile_n;
    *tile_k = h->tile_k;
    return COSMA_GPU_SUCCESS;
}

void* cosma_gpu_tmm_device_buffer_c(cosma_gpu_mm_handle* h) { return h ? h->last_device_c : nullptr; }

int cosma_gpu_tmm_last_overlapped(cosma_gpu_mm_handle* h) { return h ? h->last_overlapped : 0; }

int cosma_gpu_tmm_last_transfer_bytes(cosma_gpu_mm_handle* h, int64_t* h2d_bytes, int64_t* d2h_bytes) {
    if (!h || !h2d_bytes || !d2h_bytes)
        return cgb::set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "last_transfer_bytes: null argument");
    *h2d_bytes = h->last_h2d_bytes;
    *d2h_bytes = h->last_d2h_bytes;
    return COSMA_GPU_SUCCESS;
}

int cosma_gpu_tmm_last_ozaki_info(cosma_gpu_mm_handle* h, cosma_gpu_ozaki_info* info) {
    if (!h || !info) return cgb::set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "last_ozaki_info: null argument");
    *info = h->last_info;
    return COSMA_GPU_SUCCESS;
}

int cosma_gpu_tmm_gemm_d(cosma_gpu_mm_handle* h, char ta, char tb, int m, int n, int k, double alpha, const double* A,
                         int lda, const double* B, int ldb, double beta, double* C, int ldc, int pin, int copy_c_back) {
    cgb::clear_error();
    double a[2] = {alpha, 0}, b[2] = {beta, 0};
    return cgb::tmm_gemm(h, cgb::Scalar::D, ta, tb, m, n, k, a, A, lda, B, ldb, b, C, ldc, pin != 0, copy_c_back != 0);
}
int cosma_gpu_tmm_gemm_s(cosma_gpu_mm_handle* h, char ta, char tb, int m, int n, int k, float alpha, const float* A,
                         int lda, const float* B, int ldb, float beta, float* C, int ldc, int pin, int copy_c_back) {
    cgb::clear_error();
    double a[2] = {alpha, 0}, b[2] = {beta, 0};
    return cgb::tmm_gemm(h, cgb::Scalar::S, ta, tb, m, n, k, a, A, lda, B, ldb, b, C, ldc, pin != 0, copy_c_back != 0);
}
int cosma_gpu_tmm_gemm_z(cosma_gpu_mm_handle* h, char ta, char tb, int m, int n, int k, const double* alpha,
                         const double* A, int lda, const double* B, int ldb, const double* beta, double* C, int ldc,
                         int pin, int copy_c_back) {
    cgb::clear_error();
    double a[2] = {alpha[0], alpha[1]}, b[2] = {beta[0], beta[1]};
    return cgb::tmm_gemm(h, cgb::Scalar::Z, ta, tb, m, n, k, a, A, lda, B, ldb, b, C, ldc, pin != 0, copy_c_back != 0);
}
int cosma_gpu_tmm_gemm_c(cosma_gpu_mm_handle* h, char ta, char tb, int m, int n, int k, const float* alpha,
                         const float* A, int lda, const float* B, int ldb, const float* beta, float* C, int ldc,
                         int pin, int copy_c_back) {
    cgb::clear_error();
    double a[2] = {alpha[0], alpha[1]}, b[2] = {beta[0], beta[1]};
    return cgb::tmm_gemm(h, cgb::Scalar::C, ta, tb, m, n, k, a, A, lda, B, ldb, b, C, ldc, pin != 0, copy_c_back != 0);
}

cosma_gpu_mm_handle* cosma_gpu_context_instance(char scalar) {
    cgb::Scalar s;
    if (!parse_scalar(scalar, &s)) {
        cgb::set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "context_instance: scalar must be s, d, c or z");
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(g_singleton_mu);
    int idx = (int)s;
    if (!g_singletons[idx]) {
        // Lives until process exit, like the reference's singleton
        // (src/cosma/context.cpp:155-158).
        g_singletons[idx] = cosma_gpu_tmm_make_context(scalar, 0, 0, 0, 0);
        g_pin_default = cgb::default_pinning();
    }
    return g_singletons[idx];
}

}  // extern "C"

// local_multiply: 'N','N', ld = m, k, m; pins host buffers when
// COSMA_GPU_MEMORY_PINNING is ON (default), as local_multiply.cpp:342-347.
template <class T>
static int local_multiply_impl(cosma_gpu_mm_handle* h, char scalar, cgb::Scalar sc, T* a, T* b, T* c, int m, int n,
                               int k, const double* alpha, const double* beta, int copy_c_back) {
    cgb::clear_error();
    if (!h) h = cosma_gpu_context_instance(scalar);
    if (!h) return cosma_gpu_last_error();
    return cgb::tmm_gemm(h, sc, 'N', 'N', m, n, k, alpha, a, std::max(1, m), b, std::max(1, k), beta, c,
                         std::max(1, m), g_pin_default, copy_c_back != 0);
}

extern "C" {

int cosma_gpu_local_multiply_d(cosma_gpu_mm_handle* h, double* a, double* b, double* c, int m, int n, int k,
                               double alpha, double beta, int copy_c_back) {
    double al[2] = {alpha, 0}, be[2] = {beta, 0};
    return local_multiply_impl(h, 'd', cgb::Scalar::D, a, b, c, m, n, k, al, be, copy_c_back);
}
int cosma_gpu_local_multiply_s(cosma_gpu_mm_handle* h, float* a, float* b, float* c, int m, int n, int k, float alpha,
                               float beta, int copy_c_back) {
    double al[2] = {alpha, 0}, be[2] = {beta, 0};
    return local_multiply_impl(h, 's', cgb::Scalar::S, a, b, c, m, n, k, al, be, copy_c_back);
}
int cosma_gpu_local_multiply_z(cosma_gpu_mm_handle* h, double* a, double* b, double* c, int m, int n, int k,
                               const double* alpha, const double* beta, int copy_c_back) {
    double al[2] = {alpha[0], alpha[1]}, be[2] = {beta[0], beta[1]};
    return local_multiply_impl(h, 'z', cgb::Scalar::Z, a, b, c, m, n, k, al, be, copy_c_back);
}
int cosma_gpu_local_multiply_c(cosma_gpu_mm_handle* h, float* a, float* b, float* c, int m, int n, int k,
                               const float* alpha, const float* beta, int copy_c_back) {
    double al[2] = {alpha[0], alpha[1]}, be[2] = {beta[0], beta[1]};
    return local_multiply_impl(h, 'c', cgb::Scalar::C, a, b, c, m, n, k, al, be, copy_c_back);
}

}  // extern "C"
