// Host-side runtime declarations shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include <mutex>

struct cosma_gpu_oz_grouped_plan;   // grouped Ozaki plan (ozaki_grouped.cu)
struct cosma_gpu_oz2_grouped_plan;  // grouped Chinese-remainder plan (ozaki2_grouped.cu)

namespace cgb {

bool env_bool(const char* name, bool dflt);
long long env_ll(const char* name, long long dflt);
bool env_verbose();
int default_streams();
int default_tile_m();
int default_tile_n();
int default_tile_k();
bool default_pinning();
int default_method();

// A value computed once per device (an occupancy figure, an SM count, a
// kernel attribute having been set) and cached for the process lifetime.
// Threads that ask for the same device at the same time compute it once; a
// computation that fails is retried by the next caller.
template <class T>
class PerDevice {
   public:
    static constexpr int kMaxDevices = 64;
    // compute(T&) returns a status; on success the value is cached for the
    // current device and copied to *out.
    template <class F>
    int get(F&& compute, T* out) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) dev = kMaxDevices;
        std::lock_guard<std::mutex> lock(mu_);
        if (dev == kMaxDevices) {  // beyond the table: no caching
            T v{};
            const int s = compute(v);
            if (s == 0) *out = v;
            return s;
        }
        if (!have_[dev]) {
            T v{};
            const int s = compute(v);
            if (s != 0) return s;
            val_[dev] = v;
            have_[dev] = true;
        }
        *out = val_[dev];
        return 0;
    }

   private:
    std::mutex mu_;
    bool have_[kMaxDevices] = {};
    T val_[kMaxDevices] = {};
};

// Host-side fault injection for tests (cosma_gpu_test_fail_next): each call
// at an armed site consumes one pending fault and reports it, so the caller
// takes its error path as if the CUDA call had failed.  No GPU is involved.
enum FaultSite {
    kFaultDeviceAlloc = 1,
    kFaultHostRegister = 2,
    kFaultPinnedAlloc = 3,
    kFaultHostCopy = 4,  // a copy issued by the overlapped form's copy thread
    kFaultSites = 5
};
bool inject_fault(int site);
// cudaMallocHost behind the kFaultPinnedAlloc site.
cudaError_t pinned_alloc(void** p, size_t bytes);

// SM count of the current device (cached per device; 152 if the query fails).
int device_sm_count();

// Scalar kinds of the four GEMM flavours.
enum class Scalar { S, D, C, Z };

inline size_t scalar_bytes(Scalar s) {
    switch (s) {
        case Scalar::S: return 4;
        case Scalar::D: return 8;
        case Scalar::C: return 8;
        case Scalar::Z: return 16;
    }
    return 8;
}
inline bool scalar_complex(Scalar s) { return s == Scalar::C || s == Scalar::Z; }

// op(X) codes: 0 = 'N', 1 = 'T', 2 = 'C'; -1 for an invalid flag.
inline int parse_op(char c) {
    switch (c) {
        case 'N': case 'n': return 0;
        case 'T': case 't': return 1;
        case 'C': case 'c': return 2;
    }
    return -1;
}

// Reusable grow-only device buffer (stream-ordered allocation).
struct DeviceBuffer {
    void* ptr = nullptr;
    size_t bytes = 0;
    int reserve(size_t need, cudaStream_t stream);
    void release();
    ~DeviceBuffer() { release(); }
};

// Generic GEMM description on device pointers.  Complex scalars use
// alpha[0..1] / beta[0..1]; real scalars use alpha[0] / beta[0].
struct GemmDesc {
    Scalar scalar;
    int opa, opb;           // 0 N, 1 T, 2 C
    int64_t m, n, k;
    double alpha[2], beta[2];
    const void* A; int64_t lda;
    const void* B; int64_t ldb;
    void* C; int64_t ldc;
};

// Device-level entry points implemented in the .cu files.
int native_gemm(const GemmDesc& g, cudaStream_t stream);          // dmma_gemm.cu
int scale_matrix_device(Scalar s, int64_t rows, int64_t cols, const double* beta, void* C,
                        int64_t ldc, cudaStream_t stream);        // layout.cu
int ozaki_dgemm(const GemmDesc& g, int slices, cudaStream_t stream,
                cosma_gpu_ozaki_info* info);                     // ozaki.cu
int ozaki_zgemm(const GemmDesc& g, int slices, cudaStream_t stream,
                cosma_gpu_ozaki_info* info);                     // ozaki.cu
int unpack_device(Scalar sc, int64_t rows, int64_t cols, const double* alpha, const void* src, int64_t lds,
                  const double* beta, void* dst, int64_t ldd, cudaStream_t s);  // layout.cu
// dst = op(src) (op 0 N, 1 T, 2 C, 3 conjugate), column-major; any pointer the
// device can dereference (layout.cu)
int pack_device(int op, bool is_complex, int elem_bytes, int64_t rows, int64_t cols, const void* src, int64_t lds,
                void* dst, int64_t ldd, cudaStream_t s);
int bf16x3_sgemm(const GemmDesc& g, cudaStream_t stream);         // bf16x3.cu
int ozaki2_dgemm(const GemmDesc& g, int moduli, cudaStream_t stream,
                 cosma_gpu_ozaki_info* info);                    // ozaki2.cu
int ozaki2_zgemm(const GemmDesc& g, int moduli, cudaStream_t stream,
                 cosma_gpu_ozaki_info* info);                    // ozaki2.cu
// Free the per-stream workspaces of the precision forms before the stream is
// destroyed (ozaki.cu, ozaki2.cu).
void ozaki_release_stream(cudaStream_t s);
void ozaki2_release_stream(cudaStream_t s);
// One-step DGEMM, or ZGEMM with real alpha and beta, on host A, B, C with the
// host copies overlapped with the Chinese-remainder work (ozaki2.cu): cs
// computes, hs carries host-to-device copies, ds device-to-host copies.
// *taken = false (C untouched, nothing in flight) when the shape or the
// scalars do not pipeline, or when the first panels' modulus count differs
// from the whole data's or the data holds Inf/NaN: the caller then runs the
// regular path.
// One-step 3xBF16 SGEMM on host A, B, C with the host copies overlapped with
// the slice splits and block GEMMs (bf16x3.cu); *taken = false (nothing done)
// when the shape does not pipeline.
int bf16x3_sgemm_host(const GemmDesc& g, cudaStream_t cs, cudaStream_t hs, cudaStream_t ds, int64_t* h2d_bytes,
                      int64_t* d2h_bytes, bool* taken);
void bf16x3_release_stream(cudaStream_t s);
int ozaki2_gemm_host(const GemmDesc& g, int moduli, cudaStream_t cs, cudaStream_t hs, cudaStream_t ds,
                      cosma_gpu_ozaki_info* info, int64_t* h2d_bytes, int64_t* d2h_bytes, bool* taken);

// The method of the process-wide entry points (p?gemm, multiply_using_layout):
// cosma_gpu_pxgemm_set_method, else COSMA_GPU_GEMM_METHOD (pxgemm.cpp).
int process_gemm_method();

// Column-major sub-matrix copies between host and HBM (host_copy.cpp).
// Pageable host memory is copied by a device kernel where the GPU reads the
// host's page tables, else through pinned staging buffers filled by several
// host threads; pinned / device memory is copied directly.  The D2H form
// returns once the data is in host memory.
int copy_h2d_2d(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t cols,
                cudaStream_t s);
int copy_d2h_2d(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t cols,
                cudaStream_t s);
// Asynchronous 2-D copy on stream s: a pageable host side goes through the
// device copy kernel where the GPU reads the host's page tables, everything
// else through cudaMemcpy2DAsync (pageable memory then takes the driver's
// own staging).  Nothing is waited for.
int copy_2d_async(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t cols,
                  cudaMemcpyKind kind, cudaStream_t s);
// The same, for copies that overlap a running persistent kernel: page-locked
// host memory goes through the copy engines (at the link's rate, without
// taking SMs from the kernel: copy kernels beside the modular GEMM, whether
// a full grid or 64 CTAs, held a 16384^3 call at ~120 ms against ~100 ms),
// pageable memory as in copy_2d_async.
int copy_2d_overlapped(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t cols,
                       cudaMemcpyKind kind, cudaStream_t s);
// A copy issued from a thread that may wait for it (the overlapped form's
// copy thread): pageable host memory goes through the pinned staging buffers
// (host threads and the copy engines: no SM is taken from running kernels,
// and the driver's own pageable copies are avoided, whose speed swung
// between 190 and 4 GB/s from one call to the next on the virtual machines
// measured); page-locked memory through cudaMemcpy2DAsync.  For pageable
// memory the H2D form returns once its data is handed to the copy engine,
// the D2H form once it is in host memory; page-locked copies return at once.
int copy_2d_from_thread(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t cols,
                        cudaMemcpyKind kind, cudaStream_t s);
// Whether the device copy kernel route is on (capable device, and
// COSMA_GPU_HOST_DIRECT not OFF).
bool host_direct_available();
// Whether kernels may read and write the column-major host array at p in
// place (pageable or mapped pinned memory on a host whose page tables the
// device uses); pageable pages are faulted in on the host first.
bool prepare_direct_host(void* p, size_t pitch, size_t width, size_t cols, bool write);
// Whether p is page-locked host memory (host_copy.cpp).
bool host_page_locked(const void* p);

// Grouped Ozaki-split FP64 GEMM (ozaki_grouped.cu), driven by the grouped
// plan of grouped.cu when it is created with the Ozaki method.
cosma_gpu_oz_grouped_plan* oz_grouped_create(int count, const cosma_gpu_gemm_problem* problems, int autotune,
                                             cudaStream_t st, int* status);
int oz_grouped_run(cosma_gpu_oz_grouped_plan* pl, cudaStream_t st);
void oz_grouped_destroy(cosma_gpu_oz_grouped_plan* pl);
void oz_grouped_info(const cosma_gpu_oz_grouped_plan* pl, cosma_gpu_grouped_info* info);
int oz_grouped_slices(const cosma_gpu_oz_grouped_plan* pl, int* out);
cosma_gpu_oz2_grouped_plan* oz2_grouped_create(int count, const cosma_gpu_gemm_problem* problems, int autotune,
                                               cudaStream_t st, int* status);
int oz2_grouped_run(cosma_gpu_oz2_grouped_plan* pl, cudaStream_t st);
void oz2_grouped_destroy(cosma_gpu_oz2_grouped_plan* pl);
void oz2_grouped_info(const cosma_gpu_oz2_grouped_plan* pl, cosma_gpu_grouped_info* info);
int oz2_grouped_slices(const cosma_gpu_oz2_grouped_plan* pl, int* out);
int oz2_grouped_fraction_bits(const cosma_gpu_oz2_grouped_plan* pl, int* out);

// Dispatches one device-pointer GEMM by method (handles the k == 0 /
// alpha == 0 corner cases).  Defined in gemm_dispatch.cpp.
GemmDesc make_gemm_desc(Scalar s, char ta, char tb, int64_t m, int64_t n, int64_t k, const double* alpha,
                        const void* A, int64_t lda, const void* B, int64_t ldb, const double* beta, void* C,
                        int64_t ldc);  // gemm_dispatch.cpp
int gemm_device(const GemmDesc& g, int method, int ozaki_slices, cudaStream_t stream,
                cosma_gpu_ozaki_info* info);

}  // namespace cgb
