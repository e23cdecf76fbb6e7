// Shared host/device helpers for the cosma_gb300 library (sm_103a only).
//
// Status convention: every C-ABI entry point returns an int status
// (COSMA_GPU_SUCCESS == 0) and records a thread-local message readable through
// cosma_gpu_last_error_string().  The reference reports GPU errors by throwing
// std::runtime_error("GPU ERROR") from check_runtime_status
// (src/cosma/gpu/utils.hpp:7-13); exceptions must not cross a C ABI, so the
// same condition becomes a status code here.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/cosma_gb300.h"

namespace cgb {

// Records `msg` as the calling thread's last error and returns `code`.
int set_error(int code, const std::string& msg);
// Clears the calling thread's last error.
void clear_error();

// Maps a CUDA runtime error to a status, recording the call site.
int cuda_status(cudaError_t e, const char* what);

}  // namespace cgb

#define CGB_CUDA(call)                                               \
    do {                                                             \
        cudaError_t _e = (call);                                     \
        if (_e != cudaSuccess) return ::cgb::cuda_status(_e, #call); \
    } while (0)

#define CGB_CHECK(expr)                 \
    do {                                \
        int _s = (expr);                \
        if (_s != COSMA_GPU_SUCCESS) return _s; \
    } while (0)

namespace cgb {

constexpr int kNumSMs = 152;  // GB300: 2 dies x 76 SMs

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// ---------------------------------------------------------------------------
// Device-side error word: kernels that wait on mbarriers give up after a
// bounded number of polls, set a code here and return; the host reads it after
// the launch (see read_device_error()).
// ---------------------------------------------------------------------------
enum DeviceErr : unsigned {
    kDevOk = 0,
    kDevTimeoutFull = 1,      // consumer gave up waiting for a filled stage
    kDevTimeoutEmpty = 2,     // producer gave up waiting for a free stage
    kDevTimeoutAcc = 3,       // epilogue gave up waiting for an accumulator
    kDevTimeoutAccEmpty = 4,  // MMA issuer gave up waiting for the epilogue
    kDevBadConfig = 5,
};

}  // namespace cgb
