// Host-side pieces of the overlapped one-step forms (ozaki2.cu: the
// Chinese-remainder DGEMM / ZGEMM; bf16x3.cu: the 3xBF16 SGEMM): the copy
// thread that issues their host copies and the panel split of a dimension.
#pragma once

#include "common.cuh"
#include "runtime.hpp"

#include <algorithm>
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <functional>
#include <mutex>
#include <string>
#include <thread>

namespace cgb {

// Host copies issued from a worker thread, in order.  A copy of pageable
// host memory returns only once it is done (even cudaMemcpy2DAsync), so the
// thread that feeds the GPU must not issue it; page-locked copies return at
// once either way.  post() queues a task and returns its ticket; wait(t)
// returns once task t has run (its copy issued, or for pageable memory done,
// and its event recorded), with the first error of the tasks so far.
class CopyWorker {
public:
    explicit CopyWorker(int device) : device_(device), th_([this] { loop(); }) {}
    ~CopyWorker() {
        {
            std::lock_guard<std::mutex> lock(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        th_.join();
    }
    uint64_t post(std::function<int()> task) {
        std::lock_guard<std::mutex> lock(mu_);
        q_.push_back(std::move(task));
        cv_.notify_all();
        return ++posted_;
    }
    // An error of the worker's thread is reported again on the caller's (the
    // library's last-error record is per thread).
    int wait(uint64_t ticket) {
        std::unique_lock<std::mutex> lock(mu_);
        cv_.wait(lock, [&] { return done_ >= ticket; });
        if (err_ != COSMA_GPU_SUCCESS) set_error(err_, msg_);
        return err_;
    }
    int drain() {
        uint64_t t;
        {
            std::lock_guard<std::mutex> lock(mu_);
            t = posted_;
        }
        const int e = wait(t);
        std::lock_guard<std::mutex> lock(mu_);
        err_ = COSMA_GPU_SUCCESS;  // reported once
        msg_.clear();
        return e;
    }

private:
    void loop() {
        cudaSetDevice(device_);
        for (;;) {
            std::function<int()> task;
            {
                std::unique_lock<std::mutex> lock(mu_);
                cv_.wait(lock, [&] { return stop_ || !q_.empty(); });
                if (q_.empty()) return;  // stopping
                task = std::move(q_.front());
                q_.pop_front();
            }
            const int e = task();
            {
                std::lock_guard<std::mutex> lock(mu_);
                if (e != COSMA_GPU_SUCCESS && err_ == COSMA_GPU_SUCCESS) {
                    err_ = e;
                    msg_ = std::string("overlapped host copy: ") + cosma_gpu_last_error_string();
                }
                ++done_;
            }
            cv_.notify_all();
        }
    }
    int device_;
    std::mutex mu_;
    std::condition_variable cv_;
    std::deque<std::function<int()>> q_;
    uint64_t posted_ = 0, done_ = 0;
    int err_ = COSMA_GPU_SUCCESS;
    std::string msg_;
    bool stop_ = false;
    std::thread th_;  // last: started once everything it uses exists
};

// Panel split of one dimension: `parts` pieces, each a multiple of 256 rows
// (the GEMMs' tile) but the last, where the first (the lead panel) may be
// shorter than the others: the first block can start once less data has
// crossed the link.
struct Panels {
    int count = 1;
    int64_t lead = 0, size = 0;
    int64_t first(int i) const { return i == 0 ? 0 : lead + (int64_t)(i - 1) * size; }
    int64_t rows(int i, int64_t total) const { return std::min(i == 0 ? lead : size, total - first(i)); }
    int64_t largest() const { return std::max(lead, size); }
};

inline Panels make_panels(int64_t total, int parts, int64_t lead_max) {
    Panels p;
    p.size = ceil_div(ceil_div(total, parts), 256) * 256;
    p.lead = std::min(p.size, lead_max);
    p.count = 1 + (int)ceil_div(std::max<int64_t>(total - p.lead, 0), p.size);
    return p;
}

}  // namespace cgb
