// Host <-> HBM copies of column-major sub-matrices from pageable memory.
//
// A pageable cudaMemcpy goes through the driver's own small staging buffer
// and one CPU thread; its speed varies widely between hosts (6.5 to 27 GB/s
// measured on the same GB300 pool).  These copies take one of two faster
// routes for pageable memory:
//  * where the GPU reaches pageable memory through the host's page tables
//    (a Grace host's coherent NVLink-C2C link with address translation
//    services), a device copy kernel reads or writes the host array in
//    place, at the link's rate and without host threads;
//  * elsewhere they stage through two pinned buffers: host threads copy
//    column blocks into one buffer while the DMA engine moves the other.
// COSMA_GPU_HOST_DIRECT=OFF keeps the staged route on a capable host.
// Pinned (or registered) and device memory take cudaMemcpy2DAsync.
#include "common.cuh"
#include "runtime.hpp"

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>
#include <unistd.h>
#include <vector>

namespace cgb {
namespace {

constexpr size_t kStageBytes = 128ull << 20;  // per staging buffer

struct Stager {
    void* buf[2] = {nullptr, nullptr};
    cudaEvent_t done[2] = {nullptr, nullptr};
    bool ok = false;
};

std::mutex g_stage_mu;
Stager g_stager;  // one per process: the copies below hold g_stage_mu

// Allocates what is still missing; a failure leaves the copies on the
// driver's own pageable path and is retried by the next copy.
bool stager_ready() {
    if (g_stager.ok) return true;
    for (int i = 0; i < 2; ++i) {
        if (!g_stager.buf[i] && pinned_alloc(&g_stager.buf[i], kStageBytes) != cudaSuccess) {
            g_stager.buf[i] = nullptr;
            break;
        }
        if (!g_stager.done[i] && cudaEventCreateWithFlags(&g_stager.done[i], cudaEventDisableTiming) != cudaSuccess) {
            g_stager.done[i] = nullptr;
            break;
        }
    }
    cudaGetLastError();
    g_stager.ok = g_stager.buf[0] && g_stager.buf[1] && g_stager.done[0] && g_stager.done[1];
    return g_stager.ok;
}

int copy_threads() {
    static const int n = [] {
        unsigned h = std::thread::hardware_concurrency();
        return (int)std::max(1u, std::min(h ? h : 1u, 16u));
    }();
    return n;
}

// Host threads kept for the parallel copies below: run(nt, f) calls f(t)
// for t = 0 .. nt-1, f(0) on the calling thread, and returns when all are
// done.  One job at a time; starting threads per job cost ~0.3 ms per
// 128 MB staging chunk.  A pool that cannot start its threads runs the job
// on the calling thread alone.
class HostPool {
   public:
    void run(int nt, const std::function<void(int)>& f) {
        std::lock_guard<std::mutex> job(job_mu_);
        if (nt > 1 && !start(nt - 1)) nt = 1;
        if (nt == 1) {
            f(0);
            return;
        }
        {
            std::lock_guard<std::mutex> lock(mu_);
            fn_ = &f;
            parts_ = nt;
            left_ = nt - 1;
            ++gen_;
        }
        cv_.notify_all();
        f(0);
        std::unique_lock<std::mutex> lock(mu_);
        done_cv_.wait(lock, [&] { return left_ == 0; });
        fn_ = nullptr;
    }
    ~HostPool() {
        {
            std::lock_guard<std::mutex> lock(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto& t : th_) t.join();
    }

   private:
    bool start(int want) {
        try {
            while ((int)th_.size() < want) {
                const int id = (int)th_.size() + 1;
                unsigned long long now;
                {
                    std::lock_guard<std::mutex> lock(mu_);
                    now = gen_;  // a new thread waits for the next job, not the last one
                }
                th_.emplace_back([this, id, now] { loop(id, now); });
            }
        } catch (...) {
            return false;  // the threads started so far stay; this job runs alone
        }
        return true;
    }
    void loop(int id, unsigned long long seen) {
        for (;;) {
            const std::function<void(int)>* f;
            {
                std::unique_lock<std::mutex> lock(mu_);
                cv_.wait(lock, [&] { return stop_ || gen_ != seen; });
                if (stop_) return;
                seen = gen_;
                if (id >= parts_) continue;  // not part of this job
                f = fn_;
            }
            (*f)(id);
            {
                std::lock_guard<std::mutex> lock(mu_);
                if (--left_ == 0) done_cv_.notify_all();
            }
        }
    }
    std::mutex job_mu_, mu_;
    std::condition_variable cv_, done_cv_;
    std::vector<std::thread> th_;
    const std::function<void(int)>* fn_ = nullptr;
    int parts_ = 0, left_ = 0;
    unsigned long long gen_ = 0;
    bool stop_ = false;
};

HostPool& host_pool() {
    static HostPool* pool = new HostPool();  // never destroyed: threads may outlive static destruction order
    return *pool;
}

// Runs body(c0, c1) over [0, cols) in pieces of about `bytes_per_piece`
// bytes (`width` bytes a column) on nt threads that take pieces as they
// finish the last: a thread that the OS puts aside (another thread of the
// process spinning on a CUDA event, say) holds up one piece, not 1/nt of
// the job.
void parallel_columns(int nt, size_t width, size_t cols, const std::function<void(size_t, size_t)>& body) {
    const size_t per = std::max<size_t>(1, (size_t)(2u << 20) / std::max<size_t>(width, 1));
    const size_t pieces = (cols + per - 1) / per;
    std::atomic<size_t> next{0};
    host_pool().run(std::min<int>(nt, (int)std::max<size_t>(pieces, 1)), [&](int) {
        for (size_t q = next++; q < pieces; q = next++) body(q * per, std::min(cols, (q + 1) * per));
    });
}

// Copies `cols` columns of `width` bytes between pitched layouts on `nt` threads.
void parallel_copy(char* dst, size_t dpitch, const char* src, size_t spitch, size_t width, size_t cols) {
    const size_t bytes = width * cols;
    const int nt = bytes < (8u << 20) ? 1 : copy_threads();
    parallel_columns(nt, width, cols, [&](size_t c0, size_t c1) {
        if (dpitch == width && spitch == width) {
            std::memcpy(dst + c0 * width, src + c0 * width, (c1 - c0) * width);
        } else {
            for (size_t c = c0; c < c1; ++c) std::memcpy(dst + c * dpitch, src + c * spitch, width);
        }
    });
}

enum class HostMem { Device, PinnedMapped, PinnedOther, Pageable };

// What kind of memory p is.  PinnedMapped: page-locked host memory that
// kernels reach under its own address (unified addressing).
HostMem host_mem(const void* p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return HostMem::Pageable;
    }
    if (at.type == cudaMemoryTypeUnregistered) return HostMem::Pageable;
    if (at.type == cudaMemoryTypeHost) return at.devicePointer == p ? HostMem::PinnedMapped : HostMem::PinnedOther;
    return HostMem::Device;
}

bool pageable(const void* p) { return host_mem(p) == HostMem::Pageable; }

// Whether kernels may dereference pageable host pointers (the device
// accesses pageable memory, and does so through the host's page tables).
bool host_direct() {
    static PerDevice<bool> cache;  // a property of the current device
    bool capable = false;
    if (cache.get(
            [](bool& v) {
                int dev = 0, pma = 0, hpt = 0;
                v = false;
                if (cudaGetDevice(&dev) != cudaSuccess ||
                    cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess ||
                    cudaDeviceGetAttribute(&hpt, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) !=
                        cudaSuccess) {
                    cudaGetLastError();
                    return 0;
                }
                v = pma == 1 && hpt == 1;
                return 0;
            },
            &capable) != 0)
        capable = false;
    return capable && env_bool("COSMA_GPU_HOST_DIRECT", true);
}

// The widest element (8 or 4 bytes) dividing both addresses, both pitches
// and the width of a copy; 0 when none does.
int copy_elem(const void* a, const void* b, size_t pa, size_t pb, size_t width) {
    const uintptr_t x = (uintptr_t)a | (uintptr_t)b | (uintptr_t)pa | (uintptr_t)pb | (uintptr_t)width;
    return x % 8 == 0 ? 8 : x % 4 == 0 ? 4 : 0;
}

// Faults in, on host threads, every page the copy will touch on the host
// side (one access per page of each column's `width` bytes; writes store the
// value they read).  A GPU access to a page the host has never touched (an
// np.zeros / malloc'd output) takes a GPU page fault, which served one page
// at a time made a 2 GB direct copy 300 ms slower; the host faults pages in
// in parallel, and an access to a resident page costs one cache miss.
// Bytes between the columns are left alone: they may be another thread's.
void prefault(const void* base, size_t pitch, size_t width, size_t cols, bool write) {
    static const size_t page = [] {
        const long p = sysconf(_SC_PAGESIZE);
        return p > 0 ? (size_t)p : (size_t)4096;
    }();
    auto work = [&](size_t c0, size_t c1) {
        unsigned sink = 0;
        for (size_t c = c0; c < c1; ++c) {
            volatile unsigned char* col = (volatile unsigned char*)base + c * pitch;
            const uintptr_t start = (uintptr_t)col;
            for (uintptr_t a = start; a < start + width; a = (a / page + 1) * page) {
                volatile unsigned char* q = (volatile unsigned char*)a;
                if (write) *q = *q;
                else sink += *q;
            }
        }
        (void)sink;
    };
    const int nt = width * cols < (8u << 20) ? 1 : copy_threads();
    parallel_columns(nt, width, cols, work);
}

// The copy as a device kernel (op N pack, 16-byte vectors where aligned)
// when the host side is pageable or mapped pinned memory and the device
// reaches host memory through the host's page tables.  On such a host (a
// Grace CPU on NVLink-C2C) the kernel also beats the copy engines on pinned
// memory: a 16384^3 Ozaki DGEMM from torch-pinned buffers took 305 to 313 ms
// with kernel copies against 329 to 342 ms with cudaMemcpy.  Pageable pages
// are faulted in first.  False, having done nothing, when the route does not
// apply.
bool direct_copy(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t cols, bool host_is_dst,
                 cudaStream_t s, int* status) {
    const void* host = host_is_dst ? (const void*)dst : src;
    const HostMem hm = host_mem(host);
    if (hm != HostMem::Pageable && hm != HostMem::PinnedMapped) return false;
    if (!host_direct()) return false;
    const int eb = copy_elem(dst, src, dpitch, spitch, width);
    if (!eb) return false;
    if (hm == HostMem::Pageable) {
        if (host_is_dst) prefault(dst, dpitch, width, cols, true);
        else prefault(src, spitch, width, cols, false);
    }
    *status = pack_device(0, false, eb, (int64_t)(width / eb), (int64_t)cols, src, (int64_t)(spitch / eb), dst,
                          (int64_t)(dpitch / eb), s);
    return true;
}

}  // namespace

int staged_h2d(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t cols,
               cudaStream_t s);
int staged_d2h(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t cols,
               cudaStream_t s);

bool prepare_direct_host(void* p, size_t pitch, size_t width, size_t cols, bool write) {
    const HostMem hm = host_mem(p);
    if (hm != HostMem::Pageable && hm != HostMem::PinnedMapped) return false;
    if (!host_direct()) return false;
    if (hm == HostMem::Pageable) prefault(p, pitch, width, cols, write);
    return true;
}

int copy_h2d_2d(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t cols,
                cudaStream_t s) {
    if (width == 0 || cols == 0) return COSMA_GPU_SUCCESS;
    int st = COSMA_GPU_SUCCESS;
    if (direct_copy(dst, dpitch, src, spitch, width, cols, false, s, &st)) return st;
    return staged_h2d(dst, dpitch, src, spitch, width, cols, s);
}

int copy_d2h_2d(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t cols,
                cudaStream_t s) {
    if (width == 0 || cols == 0) return COSMA_GPU_SUCCESS;
    int st = COSMA_GPU_SUCCESS;
    if (direct_copy(dst, dpitch, src, spitch, width, cols, true, s, &st)) {
        CGB_CHECK(st);
        CGB_CUDA(cudaStreamSynchronize(s));
        return COSMA_GPU_SUCCESS;
    }
    return staged_d2h(dst, dpitch, src, spitch, width, cols, s);
}

// Pageable host memory through the pinned staging buffers: host threads
// copy column blocks into one buffer while the DMA engine moves the other.
// The H2D form returns once every block is handed to the DMA engine, the
// D2H form once the data is in host memory.  Page-locked memory, columns
// wider than a staging buffer or staging buffers that cannot be had take
// cudaMemcpy2DAsync.
int staged_h2d(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t cols,
               cudaStream_t s) {
    const bool pg = pageable(src);
    std::lock_guard<std::mutex> lock(g_stage_mu);
    if (!pg || width > kStageBytes || !stager_ready()) {
        CGB_CUDA(cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, cols, cudaMemcpyHostToDevice, s));
        return COSMA_GPU_SUCCESS;
    }
    const size_t per = kStageBytes / width;  // columns per staging buffer
    int b = 0;
    for (size_t c0 = 0; c0 < cols; c0 += per, b ^= 1) {
        const size_t nc = std::min(per, cols - c0);
        CGB_CUDA(cudaEventSynchronize(g_stager.done[b]));  // the DMA out of this buffer has finished
        parallel_copy((char*)g_stager.buf[b], width, (const char*)src + c0 * spitch, spitch, width, nc);
        CGB_CUDA(cudaMemcpy2DAsync((char*)dst + c0 * dpitch, dpitch, g_stager.buf[b], width, width, nc,
                                   cudaMemcpyHostToDevice, s));
        CGB_CUDA(cudaEventRecord(g_stager.done[b], s));
    }
    return COSMA_GPU_SUCCESS;
}

int staged_d2h(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t cols,
               cudaStream_t s) {
    const bool pg = pageable(dst);
    std::lock_guard<std::mutex> lock(g_stage_mu);
    if (!pg || width > kStageBytes || !stager_ready()) {
        CGB_CUDA(cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, cols, cudaMemcpyDeviceToHost, s));
        CGB_CUDA(cudaStreamSynchronize(s));
        return COSMA_GPU_SUCCESS;
    }
    const size_t per = kStageBytes / width;
    const size_t nchunks = (cols + per - 1) / per;
    // DMA of chunk i+1 overlaps the host copy of chunk i out of the other buffer
    auto issue = [&](size_t i) -> int {
        const size_t c0 = i * per, nc = std::min(per, cols - c0);
        CGB_CUDA(cudaMemcpy2DAsync(g_stager.buf[i & 1], width, (const char*)src + c0 * spitch, spitch, width, nc,
                                   cudaMemcpyDeviceToHost, s));
        CGB_CUDA(cudaEventRecord(g_stager.done[i & 1], s));
        return COSMA_GPU_SUCCESS;
    };
    CGB_CHECK(issue(0));
    for (size_t i = 0; i < nchunks; ++i) {
        if (i + 1 < nchunks) CGB_CHECK(issue(i + 1));
        CGB_CUDA(cudaEventSynchronize(g_stager.done[i & 1]));
        const size_t c0 = i * per, nc = std::min(per, cols - c0);
        parallel_copy((char*)dst + c0 * dpitch, dpitch, (const char*)g_stager.buf[i & 1], width, width, nc);
    }
    return COSMA_GPU_SUCCESS;
}

}  // namespace cgb

namespace cgb {

int copy_2d_async(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t cols,
                  cudaMemcpyKind kind, cudaStream_t s) {
    if (width == 0 || cols == 0) return COSMA_GPU_SUCCESS;
    const void* host = kind == cudaMemcpyHostToDevice ? src : kind == cudaMemcpyDeviceToHost ? dst : nullptr;
    int st = COSMA_GPU_SUCCESS;
    if (host && direct_copy(dst, dpitch, src, spitch, width, cols, host == dst, s, &st)) return st;
    CGB_CUDA(cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, cols, kind, s));
    return COSMA_GPU_SUCCESS;
}

int copy_2d_overlapped(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t cols,
                       cudaMemcpyKind kind, cudaStream_t s) {
    if (width == 0 || cols == 0) return COSMA_GPU_SUCCESS;
    const void* host = kind == cudaMemcpyHostToDevice ? src : dst;
    const HostMem hm = host_mem(host);
    if (hm == HostMem::PinnedMapped || hm == HostMem::PinnedOther) {
        CGB_CUDA(cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, cols, kind, s));
        return COSMA_GPU_SUCCESS;
    }
    return copy_2d_async(dst, dpitch, src, spitch, width, cols, kind, s);
}

int copy_2d_from_thread(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t cols,
                        cudaMemcpyKind kind, cudaStream_t s) {
    if (width == 0 || cols == 0) return COSMA_GPU_SUCCESS;
    if (inject_fault(kFaultHostCopy)) return set_error(COSMA_GPU_ERROR_CUDA, "host copy refused (injected fault)");
    if (kind == cudaMemcpyHostToDevice && pageable(src)) return staged_h2d(dst, dpitch, src, spitch, width, cols, s);
    if (kind == cudaMemcpyDeviceToHost && pageable(dst)) return staged_d2h(dst, dpitch, src, spitch, width, cols, s);
    CGB_CUDA(cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, cols, kind, s));
    return COSMA_GPU_SUCCESS;
}

bool host_direct_available() { return host_direct(); }

bool host_page_locked(const void* p) {
    const HostMem hm = host_mem(p);
    return hm == HostMem::PinnedMapped || hm == HostMem::PinnedOther;
}

}  // namespace cgb

extern "C" int cosma_gpu_host_copy_route(const void* ptr) {
    const cgb::HostMem hm = cgb::host_mem(ptr);
    const bool direct = cgb::host_direct();
    if (hm == cgb::HostMem::Pageable) return direct ? 2 : 1;
    if (hm == cgb::HostMem::PinnedMapped && direct) return 2;
    return 0;
}
