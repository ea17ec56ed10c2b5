// dtfft_execute_noalloc: dtfft_execute for callers that cannot allocate device
// memory.
//
// dtfft_execute needs one scratch buffer of dtfft_get_aux_bytes() bytes; when
// the caller passes aux = NULL the plan allocates it with cudaMalloc on the
// first call.  Some callers cannot let that happen: processes whose device
// memory belongs to another allocator (a framework's caching allocator or a
// fixed pool that forbids raw cudaMalloc), and latency-critical loops that
// cannot take the first-use allocation and the device synchronisation that
// cudaMalloc may bring.  This entry point takes its scratch from a fixed
// buffer compiled into the library instead, and calls no allocating routine.
//
// The buffer is a file-scope __device__ array of kNoAllocScratchBytes (16 MiB);
// every GPU on which this file's code is loaded holds it until the process
// exits.  Plans whose aux_bytes exceed it are refused with
// DTFFT_ERROR_NOALLOC_SCRATCH_TOO_SMALL.
#include <cuda_runtime.h>

#include <mutex>

#include "plan.h"

namespace gb {

dtfft_error_t execute_into_scratch(dtfft_plan_t plan, void* in, void* out, int execute_type, void* scratch,
                                   size_t scratch_bytes, size_t* needed);

static constexpr size_t kNoAllocScratchBytes = 16u << 20;

// Shared by every call on a device; holds whatever the last call left there.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

static constexpr int kMaxDevices = 64;
// Per device: the context the address was looked up in, and the address.
static void* g_scratch_ctx[kMaxDevices] = {};
static void* g_scratch_addr[kMaxDevices] = {};
static std::mutex g_scratch_mu;

typedef int (*CtxGetCurrentFn)(void**);
static CtxGetCurrentFn g_ctx_get = nullptr;
static std::once_flag g_ctx_once;

// The current context of the calling thread (the driver's cuCtxGetCurrent,
// reached through the runtime's entry-point query); nullptr if unavailable.
static void* current_context() {
    std::call_once(g_ctx_once, [] {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_ctx_get = (CtxGetCurrentFn)fn;
        cudaGetLastError();
    });
    void* ctx = nullptr;
    if (!g_ctx_get || g_ctx_get(&ctx) != 0) return nullptr;
    return ctx;
}

// Device address of the scratch array on the current device.  The host-side
// name g_noalloc_scratch is not a device address, so it is looked up with
// cudaGetSymbolAddress while that device is current: once per device, and
// again if the device's context has changed since (cudaDeviceReset destroys
// the context and the module with its array; the next context loads a new
// copy at another address).
static dtfft_error_t scratch_address(void** ptr) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return DTFFT_ERROR_GPU_CALL_FAILED; }
    if (dev < 0 || dev >= kMaxDevices) return DTFFT_ERROR_GPU_CALL_FAILED;
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    void* ctx = current_context();
    if (!g_scratch_addr[dev] || ctx != g_scratch_ctx[dev]) {
        void* p = nullptr;
        const cudaError_t rc = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (rc != cudaSuccess || !p) { cudaGetLastError(); return DTFFT_ERROR_GPU_CALL_FAILED; }
        g_scratch_addr[dev] = p;
        // the lookup may have made the device's primary context current
        g_scratch_ctx[dev] = current_context();
    }
    *ptr = g_scratch_addr[dev];
    return DTFFT_SUCCESS;
}

}  // namespace gb

extern "C" dtfft_error_t dtfft_execute_noalloc(dtfft_plan_t plan, void* in, void* out,
                                               dtfft_execute_t execute_type) {
    void* scratch = nullptr;
    GB_TRY(gb::scratch_address(&scratch));
    // Every execute schedule writes its scratch before reading it, so the
    // previous call's contents need no clearing.
    return gb::execute_into_scratch(plan, in, out, (int)execute_type, scratch, gb::kNoAllocScratchBytes, nullptr);
}

extern "C" size_t dtfft_execute_noalloc_max_bytes(void) { return gb::kNoAllocScratchBytes; }
