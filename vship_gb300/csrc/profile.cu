// profile.cu -- per-kernel event timing registry (see profile.h).
#include "profile.h"
#include "common.cuh"

#include <nvtx3/nvToolsExt.h>

#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>
#include <vector>

namespace vship {

namespace {
struct Rec {
    std::string name;
    cudaEvent_t a = nullptr, b = nullptr;
};
std::atomic<bool> g_on{false};
std::mutex g_mu;
std::vector<Rec> g_recs;
std::vector<cudaEvent_t> g_pool;

cudaEvent_t get_event() {
    if (!g_pool.empty()) {
        cudaEvent_t e = g_pool.back();
        g_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}
}  // namespace

bool prof_enabled() { return g_on.load(std::memory_order_relaxed); }

namespace {
std::atomic<long> g_dev_allocs{0}, g_pinned_allocs{0};

// true when this allocation must fail: the variable is set and n allocations already passed
bool injected(const char* var, std::atomic<long>& count) {
    const char* e = getenv(var);
    if (!e) {
        count.store(0);
        return false;
    }
    return count.fetch_add(1) >= atol(e);
}
}  // namespace

cudaError_t vship_malloc(void** p, size_t bytes) {
    if (injected("VSHIP_FAIL_DEVICE_ALLOC_AFTER", g_dev_allocs)) return cudaErrorMemoryAllocation;
    return cudaMalloc(p, bytes);
}

cudaError_t vship_malloc_host(void** p, size_t bytes) {
    if (injected("VSHIP_FAIL_PINNED_ALLOC_AFTER", g_pinned_allocs)) return cudaErrorMemoryAllocation;
    return cudaMallocHost(p, bytes);
}

bool vship_alloc_injected_failure() { return injected("VSHIP_FAIL_DEVICE_ALLOC_AFTER", g_dev_allocs); }

void prof_range_push(const char* name) { nvtxRangePushA(name); }
void prof_range_pop() { nvtxRangePop(); }

int prof_begin(const char* name, cudaStream_t st) {
    if (!prof_enabled()) return -1;
    std::lock_guard<std::mutex> g(g_mu);
    Rec r;
    r.name = name;
    r.a = get_event();
    r.b = get_event();
    cudaEventRecord(r.a, st);
    g_recs.push_back(r);
    return (int)g_recs.size() - 1;
}

void prof_end(int token, cudaStream_t st) {
    if (token < 0) return;
    std::lock_guard<std::mutex> g(g_mu);
    if (token < (int)g_recs.size()) cudaEventRecord(g_recs[token].b, st);
}

// JSON object {"kernel": [launches, total_ms], ...}. A call with a buffer (len > 0) also clears
// the records; a size query (len == 0) leaves them in place.
int prof_report(char* buf, int len) {
    std::map<std::string, std::pair<long, double>> agg;
    const bool consume = buf && len > 0;
    {
        std::lock_guard<std::mutex> g(g_mu);
        for (Rec& r : g_recs) {
            float ms = 0.f;
            cudaEventSynchronize(r.b);
            if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
                auto& e = agg[r.name];
                e.first += 1;
                e.second += ms;
            }
        }
        if (consume) {
            for (Rec& r : g_recs) {
                g_pool.push_back(r.a);
                g_pool.push_back(r.b);
            }
            g_recs.clear();
        }
    }
    std::string s = "{";
    bool first = true;
    for (auto& kv : agg) {
        char tmp[256];
        snprintf(tmp, sizeof(tmp), "%s\"%s\": [%ld, %.6f]", first ? "" : ", ", kv.first.c_str(), kv.second.first,
                 kv.second.second);
        s += tmp;
        first = false;
    }
    s += "}";
    if (consume) {
        int n = (int)s.size() < len - 1 ? (int)s.size() : len - 1;
        for (int i = 0; i < n; i++) buf[i] = s[i];
        buf[n] = 0;
    }
    return (int)s.size() + 1;
}

void prof_set(bool on) { g_on.store(on); }

}  // namespace vship
