// Per-launch timing of this library's kernels with CUDA events.
//
// When enabled, every kernel launch is bracketed by two events recorded on the
// launch's own stream; collect() waits for them and sums the durations per
// kernel name.  Used by the benchmark to time the dominant kernel inside the
// timed region (the events cost a few microseconds of host time per launch
// and nothing measurable on the GPU).
#include <cuda_runtime.h>

#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "dtfft_gb300.h"

namespace gb {

struct Pending { std::string name; cudaEvent_t a, b; };
struct Total { int64_t launches = 0; double ms = 0; };

static std::mutex g_pmu;
static bool g_prof_on = false;
static std::vector<Pending> g_pending;
static std::vector<cudaEvent_t> g_pool;
static std::map<std::string, Total> g_totals;

static cudaEvent_t take_event() {
    if (!g_pool.empty()) { cudaEvent_t e = g_pool.back(); g_pool.pop_back(); return e; }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

bool profiling() { return g_prof_on; }

void* prof_begin(cudaStream_t s) {
    if (!g_prof_on) return nullptr;
    // launches captured into a graph are not timed (their events never complete as recorded here)
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
        cudaGetLastError();
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(g_pmu);
    Pending* p = new Pending();
    p->a = take_event();
    p->b = take_event();
    cudaEventRecord(p->a, s);
    return p;
}

void prof_end(void* tok, const std::string& name, cudaStream_t s) {
    if (!tok) return;
    Pending* p = static_cast<Pending*>(tok);
    cudaEventRecord(p->b, s);
    std::lock_guard<std::mutex> lk(g_pmu);
    p->name = name;
    g_pending.push_back(*p);
    delete p;
}

static void collect_locked() {
    for (Pending& p : g_pending) {
        cudaEventSynchronize(p.b);
        float ms = 0;
        cudaEventElapsedTime(&ms, p.a, p.b);
        Total& t = g_totals[p.name];
        t.launches += 1;
        t.ms += ms;
        g_pool.push_back(p.a);
        g_pool.push_back(p.b);
    }
    g_pending.clear();
}

}  // namespace gb

using namespace gb;

extern "C" {

void dtfft_gb_profile_start(void) {
    std::lock_guard<std::mutex> lk(g_pmu);
    collect_locked();
    g_totals.clear();
    g_prof_on = true;
}

void dtfft_gb_profile_stop(void) {
    std::lock_guard<std::mutex> lk(g_pmu);
    g_prof_on = false;
    collect_locked();
}

int32_t dtfft_gb_profile_count(void) {
    std::lock_guard<std::mutex> lk(g_pmu);
    collect_locked();
    return (int32_t)g_totals.size();
}

int32_t dtfft_gb_profile_get(int32_t index, char* name, int32_t name_len, int64_t* launches, double* total_ms) {
    std::lock_guard<std::mutex> lk(g_pmu);
    collect_locked();
    int i = 0;
    for (auto& kv : g_totals) {
        if (i++ != index) continue;
        if (name && name_len > 0) {
            strncpy(name, kv.first.c_str(), (size_t)name_len - 1);
            name[name_len - 1] = 0;
        }
        if (launches) *launches = kv.second.launches;
        if (total_ms) *total_ms = kv.second.ms;
        return DTFFT_SUCCESS;
    }
    return DTFFT_ERROR_INVALID_USAGE;
}

}  // extern "C"
