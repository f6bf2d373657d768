// Launch counting and optional per-group kernel timing with CUDA events.
//
// The reference has no tracing; this gives the engine its own: every kernel
// launch increments a process-wide counter, and when profiling is enabled the
// launches of each group (term enumeration, key sorting, selection, other)
// are bracketed by CUDA events on the launching stream.  qmbx_profile_read
// waits for the recorded events and returns the per-group totals.
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>
#include <vector>

#include "../../include/qmbx.h"
#include "common.h"
#include "profile.h"

namespace qmbx {
namespace {

std::atomic<int64_t> g_launches{0};
std::atomic<bool> g_enabled{false};
std::mutex g_mu;
struct Pending {
    int group;
    cudaEvent_t start, stop;
};
std::vector<Pending> g_pending;
std::vector<cudaEvent_t> g_pool;
int64_t g_count[kProfileGroups] = {};
double g_ms[kProfileGroups] = {};

cudaEvent_t take_event() {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_pool.empty()) {
        cudaEvent_t e = g_pool.back();
        g_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    return e;
}

}  // namespace

void note_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

Timing::Timing(int group, cudaStream_t stream) : group_(group), stream_(stream) {
    if (!g_enabled.load(std::memory_order_relaxed)) return;
    start_ = take_event();
    stop_ = take_event();
    if (start_ && stop_) cudaEventRecord(start_, stream_);
}

Timing::~Timing() {
    if (!start_ || !stop_) return;
    cudaEventRecord(stop_, stream_);
    std::lock_guard<std::mutex> lock(g_mu);
    g_pending.push_back({group_, start_, stop_});
}

}  // namespace qmbx

using namespace qmbx;

extern "C" int qmbx_profile_enable(int32_t on) {
    clear_error();
    std::lock_guard<std::mutex> lock(g_mu);
    for (const Pending& p : g_pending) {
        cudaEventSynchronize(p.stop);
        g_pool.push_back(p.start);
        g_pool.push_back(p.stop);
    }
    g_pending.clear();
    for (int k = 0; k < kProfileGroups; ++k) {
        g_count[k] = 0;
        g_ms[k] = 0.0;
    }
    g_enabled.store(on != 0);
    return QMBX_OK;
}

extern "C" int qmbx_profile_read(int64_t* launches, int64_t* counts, double* ms) {
    clear_error();
    std::lock_guard<std::mutex> lock(g_mu);
    for (const Pending& p : g_pending) {
        float t = 0.f;
        if (cudaEventSynchronize(p.stop) == cudaSuccess && cudaEventElapsedTime(&t, p.start, p.stop) == cudaSuccess) {
            g_count[p.group] += 1;
            g_ms[p.group] += t;
        }
        g_pool.push_back(p.start);
        g_pool.push_back(p.stop);
    }
    g_pending.clear();
    if (launches) *launches = g_launches.load();
    for (int k = 0; k < kProfileGroups; ++k) {
        if (counts) counts[k] = g_count[k];
        if (ms) ms[k] = g_ms[k];
    }
    return QMBX_OK;
}
