// Status reporting and COSMA_* environment knobs.
//
// Environment variables and defaults follow src/cosma/environment_variables.hpp:10-97;
// booleans are "ON" (case-insensitive) exactly as get_bool_env_var parses them
// (src/cosma/environment_variables.cpp:9-21).
#include "common.cuh"
#include "runtime.hpp"

#include <algorithm>
#include <atomic>
#include <cctype>
#include <cstdlib>
#include <string>

namespace cgb {

namespace {
thread_local int t_last_code = COSMA_GPU_SUCCESS;
thread_local std::string t_last_msg;
}  // namespace

int set_error(int code, const std::string& msg) {
    t_last_code = code;
    t_last_msg = msg;
    if (env_verbose()) std::fprintf(stderr, "[cosma_gb300] error %d: %s\n", code, msg.c_str());
    return code;
}

void clear_error() {
    t_last_code = COSMA_GPU_SUCCESS;
    t_last_msg.clear();
}

int cuda_status(cudaError_t e, const char* what) {
    int code = (e == cudaErrorMemoryAllocation) ? COSMA_GPU_ERROR_OUT_OF_MEMORY : COSMA_GPU_ERROR_CUDA;
    return set_error(code, std::string(what) + ": " + cudaGetErrorString(e));
}

static const char* env_raw(const char* name) { return std::getenv(name); }

bool env_bool(const char* name, bool dflt) {
    const char* v = env_raw(name);
    if (!v) return dflt;
    std::string s(v);
    std::transform(s.begin(), s.end(), s.begin(), [](unsigned char c) { return (char)std::toupper(c); });
    return s == "ON";
}

long long env_ll(const char* name, long long dflt) {
    const char* v = env_raw(name);
    if (!v || !*v) return dflt;
    return std::atoll(v);
}

bool env_verbose() {
    static const bool v = env_bool("COSMA_GPU_VERBOSE", false);
    return v;
}

// Built-in defaults.  The reference defaults to 2 streams and 5000^3 tiles
// (environment_variables.hpp:57-62), sized for 16 GB P100s; one GB300 holds
// 280 GB, so the default tile here covers every in-core problem up to 32768
// in one piece and streams only when the matrices do not fit.
int default_streams() { return (int)env_ll("COSMA_GPU_STREAMS", 3); }
int default_tile_m() { return (int)env_ll("COSMA_GPU_MAX_TILE_M", 32768); }
int default_tile_n() { return (int)env_ll("COSMA_GPU_MAX_TILE_N", 32768); }
int default_tile_k() { return (int)env_ll("COSMA_GPU_MAX_TILE_K", 32768); }
bool default_pinning() { return env_bool("COSMA_GPU_MEMORY_PINNING", true); }

namespace {
std::atomic<int> g_faults[kFaultSites];
}  // namespace

bool inject_fault(int site) {
    if (site <= 0 || site >= kFaultSites) return false;
    int v = g_faults[site].load();
    while (v > 0)
        if (g_faults[site].compare_exchange_weak(v, v - 1)) return true;
    return false;
}

cudaError_t pinned_alloc(void** p, size_t bytes) {
    if (inject_fault(kFaultPinnedAlloc)) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMallocHost(p, bytes);
}

int device_sm_count() {
    static PerDevice<int> cache;
    int n = kNumSMs;
    if (cache.get(
            [](int& v) {
                int dev = 0;
                if (cudaGetDevice(&dev) != cudaSuccess ||
                    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
                    v = kNumSMs;
                cudaGetLastError();
                return 0;
            },
            &n) != 0)
        n = kNumSMs;
    return n;
}

int default_method() {
    const char* v = env_raw("COSMA_GPU_GEMM_METHOD");
    if (!v) return COSMA_GPU_METHOD_AUTO;
    std::string s(v);
    std::transform(s.begin(), s.end(), s.begin(), [](unsigned char c) { return (char)std::tolower(c); });
    if (s == "native") return COSMA_GPU_METHOD_NATIVE;
    if (s == "ozaki") return COSMA_GPU_METHOD_OZAKI;
    if (s == "ozaki2") return COSMA_GPU_METHOD_OZAKI2;
    if (s == "bf16x3") return COSMA_GPU_METHOD_BF16X3;
    return COSMA_GPU_METHOD_AUTO;
}

}  // namespace cgb

extern "C" {

int cosma_gpu_last_error(void) { return cgb::t_last_code; }

int cosma_gpu_test_fail_next(int site, int count) {
    cgb::clear_error();
    if (site <= 0 || site >= cgb::kFaultSites || count < 0)
        return cgb::set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "test_fail_next: site 1..4 and count >= 0");
    cgb::g_faults[site].store(count);
    return COSMA_GPU_SUCCESS;
}

int cosma_gpu_test_faults_pending(int site) {
    if (site <= 0 || site >= cgb::kFaultSites) return -1;
    return cgb::g_faults[site].load();
}

const char* cosma_gpu_last_error_string(void) { return cgb::t_last_msg.c_str(); }

const char* cosma_gpu_version(void) { return "cosma_gb300 0.1.0 (sm_103a)"; }

}  // extern "C"
