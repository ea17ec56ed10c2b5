// Measured autotuner for the box-list move kernels.
//
// Replaces the analytic scoring of the reference's NVRTC block optimizer
// (src/dtfft_nvrtc_block_optimizer.F90:502-751) and its optional candidate
// timing (src/dtfft_kernel_device.F90:338-397): every compiled tile shape is
// timed with CUDA events on scratch buffers of the plan's size and the fastest
// is kept.  Choices are cached per (element size, box geometry) for the life
// of the process and, when DTFFT_GB_TUNE_CACHE names a file, across processes.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>

#include "plan.h"

namespace gb {

static std::mutex g_tune_mu;
static std::map<std::string, TransposeConfig> g_tune_cache;
static bool g_cache_loaded = false;

static std::string gpu_name() {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return "unknown";
    std::string s = prop.name;
    for (char& c : s) if (c == ' ' || c == '|') c = '_';
    return s;
}

static std::string key_of(const BoxList& bl) {
    std::ostringstream o;
    o << gpu_name() << "|" << bl.elem << "|" << (bl.copy ? "c" : "t");
    for (const Box& b : bl.host) o << "|" << b.na << "," << b.nb << "," << b.nc << "," << b.sb << "," << b.da_or_db;
    return o.str();
}

static void load_cache() {
    if (g_cache_loaded) return;
    g_cache_loaded = true;
    const char* path = getenv("DTFFT_GB_TUNE_CACHE");
    if (!path) return;
    std::ifstream f(path);
    std::string line;
    while (std::getline(f, line)) {
        // version 1 line: v1 <key> <tile_a> <tile_b> <rows>
        std::istringstream is(line);
        std::string v, key;
        TransposeConfig c;
        if (is >> v >> key >> c.tile_a >> c.tile_b >> c.rows && v == "v1") g_tune_cache[key] = c;
    }
}

static void store_cache(const std::string& key, const TransposeConfig& c) {
    const char* path = getenv("DTFFT_GB_TUNE_CACHE");
    if (!path) return;
    std::ofstream f(path, std::ios::app);
    f << "v1 " << key << " " << c.tile_a << " " << c.tile_b << " " << c.rows << "\n";
}

dtfft_error_t autotune_boxes(BoxList& bl, i64 max_elems, cudaStream_t s, int warmup, int iters, bool log) {
    if (bl.host.empty()) return DTFFT_SUCCESS;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    load_cache();
    const std::string key = key_of(bl);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
        bl.cfg = it->second;
        return boxes_upload(bl);
    }
    void *a = nullptr, *b = nullptr;
    const size_t bytes = (size_t)max_elems * bl.elem;
    if (cudaMalloc(&a, bytes) != cudaSuccess || cudaMalloc(&b, bytes) != cudaSuccess) {
        cudaGetLastError();
        if (a) cudaFree(a);
        return DTFFT_SUCCESS;  // keep the default tile when scratch is not available
    }
    cudaMemsetAsync(a, 0, bytes, s);
    static const TransposeConfig cands[] = {
        {32, 32, 8}, {32, 32, 4}, {64, 32, 8}, {32, 64, 8}, {64, 64, 8}, {64, 64, 16}, {128, 32, 8}};
    TransposeConfig best = bl.cfg;
    float best_ms = 1e30f;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (const TransposeConfig& c : cands) {
        if (bl.elem == 16 && c.tile_a * c.tile_b > 32 * 64) continue;  // static smem limit
        // 128 x 32 exists only as the TMA kernel of 4-byte elements
        if (c.tile_a == 128 && !(bl.elem == 4 && tma_eligible(bl))) continue;
        bl.cfg = c;
        if (boxes_upload(bl) != DTFFT_SUCCESS) continue;
        bool ok = true;
        for (int i = 0; i < warmup && ok; ++i) ok = boxes_launch(bl, a, b, s) == DTFFT_SUCCESS;
        cudaEventRecord(e0, s);
        for (int i = 0; i < iters && ok; ++i) ok = boxes_launch(bl, a, b, s) == DTFFT_SUCCESS;
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        if (!ok) { cudaGetLastError(); continue; }
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        ms /= (float)iters;
        if (log) printf("dtFFT-gb300: tile %dx%d rows %d: %.4f ms\n", c.tile_a, c.tile_b, c.rows, ms);
        if (ms < best_ms) { best_ms = ms; best = c; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(a);
    cudaFree(b);
    cudaGetLastError();
    bl.cfg = best;
    g_tune_cache[key] = best;
    store_cache(key, best);
    return boxes_upload(bl);
}

}  // namespace gb
