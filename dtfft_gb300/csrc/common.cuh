// Shared definitions of the GB300 execute path: element types, launch
// bookkeeping and the CUDA error check used by every translation unit.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstdio>
#include <stdint.h>

#include <atomic>
#include <string>
#include <vector>

#include "dtfft.h"

namespace gb {

typedef int64_t i64;

// 16-byte element (complex<double>); the move kernels only copy it.
struct __align__(16) e16 { uint64_t lo, hi; };

// Number of this library's kernel launches since load (benchmark accounting).
extern std::atomic<int64_t> g_launches;
inline void count_launch(int n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

// Host-side trace range (NVTX) around the public entry points, in the places
// the reference marks with REGION_BEGIN/END (execute, transpose, reshape, plan
// creation): shown by Nsight tools when one is attached, a few nanoseconds
// otherwise.
struct TraceRange {
    explicit TraceRange(const char* name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange&) = delete;
    TraceRange& operator=(const TraceRange&) = delete;
};

// Optional per-launch event timing (profile.cpp); prof_begin returns nullptr when off.
void* prof_begin(cudaStream_t s);
void prof_end(void* token, const std::string& name, cudaStream_t s);
bool profiling();

// A failed CUDA call is reported on stderr (which call, where, CUDA's error
// name) and turns into DTFFT_ERROR_GPU_CALL_FAILED.
inline void report_cuda_error(cudaError_t e, const char* what, const char* file, int line) {
    fprintf(stderr, "dtFFT-gb300: %s failed: %s (%s) at %s:%d\n", what, cudaGetErrorName(e), cudaGetErrorString(e),
            file, line);
}

#define GB_CUDA_TRY(expr)                                             \
    do {                                                              \
        cudaError_t e_ = (expr);                                      \
        if (e_ != cudaSuccess) {                                      \
            ::gb::report_cuda_error(e_, #expr, __FILE__, __LINE__);   \
            return DTFFT_ERROR_GPU_CALL_FAILED;                       \
        }                                                             \
    } while (0)

#define GB_TRY(expr)                                                  \
    do {                                                              \
        dtfft_error_t r_ = (expr);                                    \
        if (r_ != DTFFT_SUCCESS) return r_;                           \
    } while (0)

// ---------------------------------------------------------------------------
// Transposition boxes.
//
// A transpose of the virtual grid is a list of boxes, one per (source rank,
// destination rank) pair whose global blocks intersect.  Inside a box, `a` is
// the source's contiguous axis, `b` the destination's contiguous axis and `c`
// the third axis:
//     src[src_off + a + b*sb + c*sc]  ->  dst[dst_off + b + a*da + c*dc]
// Boxes with a == b (plain copies) use the same struct with `copy` set:
//     src[src_off + a + b*sb + c*sc]  ->  dst[dst_off + a + b*db + c*dc]
// Offsets and strides are in elements, 64-bit: the whole grid lives in one
// allocation that may exceed 2^31 elements.
// ---------------------------------------------------------------------------
struct Box {
    i64 src_off, dst_off;
    int32_t na, nb, nc;
    int32_t tiles_a, tiles_b;   // tiles per c-plane (set by the launcher)
    int32_t a0;                 // start of the box along the source block's contiguous axis
    i64 sb, sc;                 // source strides of b and c
    i64 da_or_db, dc;           // destination stride of a (transpose) or b (copy), and of c
    i64 tile_begin;             // first global tile index of this box
};

// Kernel launch choice for a box list (autotuned or default).
struct TransposeConfig {
    int tile_a = 32;   // tile extent along the source-contiguous axis
    int tile_b = 32;   // tile extent along the destination-contiguous axis
    int rows = 8;      // thread rows per CTA (blockDim.y)
};

// Device-resident box list of one data movement.
struct BoxList {
    std::vector<Box> host;
    Box* dev = nullptr;
    i64 total_tiles = 0;
    bool copy = false;        // all boxes are copies (a == b)
    int elem = 8;             // element size in bytes
    TransposeConfig cfg;
    // tensor maps of the TMA transpose per input pointer (transpose_tma.cu)
    mutable std::vector<std::pair<const void*, void*>> tma_cache;
};

dtfft_error_t boxes_upload(BoxList& bl);
void boxes_free(BoxList& bl);
dtfft_error_t boxes_launch(const BoxList& bl, const void* in, void* out, cudaStream_t stream);

// TMA tensor-load transpose (transpose_tma.cu): boxes it can take, its tile
// extent along a, the launch, and the release of a list's tensor maps.
bool tma_eligible(const BoxList& bl);
int tma_tile_a(int elem);
void tma_default_tile(BoxList& bl);
dtfft_error_t tma_launch(const BoxList& bl, const void* in, void* out, cudaStream_t s, int* status,
                         std::vector<std::pair<const void*, void*>>& cache);
void tma_cache_free(std::vector<std::pair<const void*, void*>>& cache);
// The driver's cuTensorMapEncodeTiled (PFN_cuTensorMapEncodeTiled_v12000), or
// nullptr when it cannot be reached.
void* tma_encode_tiled_fn();

// Status word of the bounded waits on the current device (fft_host.cu): a
// portable mapped host word per device, created by status_setup() when a
// plan, kernel or executor is created.  check_device_status() returns
// DTFFT_ERROR_GPU_WAIT_TIMEOUT (and clears the word) when a kernel on the
// current device gave up a wait since the last check.
int* gb_status_word();
dtfft_error_t status_setup();
dtfft_error_t check_device_status();

// Iteration limit of the consumer waits of the tile kernels and the TMA
// transpose (the waits for a bulk copy to land).  The default bounds a wait
// at well over a second; tests set a limit of 0 through dtfft_gb_set_wait_limit
// to make a wait run out.  Drains of copies in flight always use the default.
constexpr int kWaitLimitDefault = 1 << 22;
extern int g_wait_limit;

// A kernel that gave up a bounded wait records `code` in the status word.
__device__ __forceinline__ void report_status(int* status, int code) {
    *reinterpret_cast<volatile int*>(status) = code;
    __threadfence_system();
}

}  // namespace gb
