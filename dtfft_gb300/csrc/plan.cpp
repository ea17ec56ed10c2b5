// Plan layer of the GB300 execute path: the dtfft_* C ABI of the reference
// (include/dtfft.h), re-implemented for one GPU that holds every rank of a
// pencil decomposition.
//
// Reference semantics kept here, each with the place it comes from:
//   grid choice / slab selection ........ src/dtfft_transpose_plan.F90:58-209
//   pencil start/count rule ............. src/dtfft_pencil.F90:237-279
//   pencil dims and comm permutations ... src/dtfft_transpose_plan.F90:1045-1131
//   FFT plans per axis and their sizes .. src/dtfft_plan.F90:2221-2284, 2381-2653,
//                                         src/dtfft_abstract_executor.F90:115-216
//   execute schedules ................... src/dtfft_plan.F90:839-1101
//   local sizes / alloc / aux sizes ..... src/dtfft_plan.F90:1338-1420, 1797-1877
//   argument checks and error codes ..... src/dtfft_plan.F90:771-837, 645-695, 2107-2219
//
// What is GB300-specific: a virtual rank's local block is a slice of one
// device buffer (blocks packed in cartesian rank order), and each transpose of
// the whole grid is one box-list kernel (transpose.cu) instead of
// pack -> NCCL/MPI exchange -> unpack.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "dtfft_gb300.h"
#include "fft.cuh"
#include "plan.h"

namespace gb {

// ---------------------------------------------------------------------------
// Configuration (src/dtfft_config.F90; defaults include/dtfft_config.h.in:177-178)
// ---------------------------------------------------------------------------
static dtfft_config_t g_cfg;
static bool g_cfg_init = false;
static std::mutex g_mu;

static bool env_bool(const char* name, bool def) {
    const char* v = getenv(name);
    if (!v) return def;
    return !(strcmp(v, "0") == 0 || strcasecmp(v, "false") == 0 || strcasecmp(v, "no") == 0);
}
static int env_int(const char* name, int def) {
    const char* v = getenv(name);
    return v ? atoi(v) : def;
}

void default_config(dtfft_config_t* c) {
    memset(c, 0, sizeof(*c));
    c->enable_log = false;
    c->enable_z_slab = true;
    c->enable_y_slab = false;
    c->n_measure_warmup_iters = 2;
    c->n_measure_iters = 5;
    c->platform = DTFFT_PLATFORM_CUDA;
    c->stream = nullptr;
    c->backend = DTFFT_BACKEND_NCCL;
    c->reshape_backend = DTFFT_BACKEND_NCCL;
    c->enable_datatype_backend = true;
    c->enable_mpi_backends = false;
    c->enable_pipelined_backends = true;
    c->enable_rma_backends = true;
    c->enable_fused_backends = true;
    c->enable_nccl_backends = true;
    c->enable_nvshmem_backends = true;
    c->enable_kernel_autotune = false;
    c->enable_fourier_reshape = false;
    c->transpose_mode = DTFFT_TRANSPOSE_MODE_PACK;
    c->access_mode = DTFFT_ACCESS_MODE_WRITE;
}

// Environment overrides, read once (names from src/dtfft_config.F90:390-510).
static void apply_env(dtfft_config_t* c) {
    c->enable_log = env_bool("DTFFT_ENABLE_LOG", c->enable_log);
    c->enable_z_slab = env_bool("DTFFT_ENABLE_Z_SLAB", c->enable_z_slab);
    c->enable_y_slab = env_bool("DTFFT_ENABLE_Y_SLAB", c->enable_y_slab);
    c->n_measure_warmup_iters = env_int("DTFFT_MEASURE_WARMUP_ITERS", c->n_measure_warmup_iters);
    c->n_measure_iters = env_int("DTFFT_MEASURE_ITERS", c->n_measure_iters);
    c->enable_kernel_autotune = env_bool("DTFFT_ENABLE_KERNEL_AUTOTUNE", c->enable_kernel_autotune);
}

const dtfft_config_t& config() {
    if (!g_cfg_init) {
        default_config(&g_cfg);
        apply_env(&g_cfg);
        g_cfg_init = true;
    }
    return g_cfg;
}

// ---------------------------------------------------------------------------
// Virtual communicators
// ---------------------------------------------------------------------------
struct VComm {
    bool cart = false;
    int nprocs = 1;
    int ndims = 0;
    int dims[3] = {1, 1, 1};
    int block_ndims = 0;                   // > 0: every rank's own block is registered
    std::vector<int32_t> starts, counts;   // nprocs x block_ndims, Fortran order
};
static std::map<int, VComm> g_vcomms;
static int g_next_comm = 0x4c000010;

static bool lookup_comm(MPI_Comm comm, VComm& out) {
    if (comm == MPI_COMM_WORLD || comm == MPI_COMM_SELF) { out = VComm(); return true; }
    auto it = g_vcomms.find((int)comm);
    if (it == g_vcomms.end()) return false;
    out = it->second;
    return true;
}

VCommInfo comm_info(MPI_Comm comm) {
    VCommInfo r;
    memset(&r, 0, sizeof(r));
    VComm v;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!lookup_comm(comm, v)) return r;
    r.known = true;
    r.cart = v.cart;
    r.nprocs = v.nprocs;
    r.ndims = v.ndims;
    for (int i = 0; i < 3; ++i) r.dims[i] = v.dims[i];
    return r;
}

bool comm_blocks(MPI_Comm comm, int* ndims, std::vector<int32_t>* starts, std::vector<int32_t>* counts) {
    VComm v;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!lookup_comm(comm, v) || v.block_ndims == 0) return false;
    *ndims = v.block_ndims;
    *starts = v.starts;
    *counts = v.counts;
    return true;
}

// ---------------------------------------------------------------------------
// Pencils
// ---------------------------------------------------------------------------
void split(int n, int P, int r, int& start, int& count) {
    // remainder to the last ranks (src/dtfft_pencil.F90:258-262)
    const int base = n / P, rem = n % P, first_big = P - rem;
    count = base + (r >= first_big ? 1 : 0);
    start = r * base + std::max(0, r - first_big);
}

// Global axis and grid-comm index of pencil dim d (get_permutations,
// src/dtfft_transpose_plan.F90:1045-1082).
void perms(int ndims, int aligned, int* axes, int* comms) {
    if (ndims == 2) {
        axes[0] = aligned == 1 ? 0 : 1; axes[1] = aligned == 1 ? 1 : 0;
        comms[0] = 0; comms[1] = 1;
        return;
    }
    static const int A[3][3] = {{0, 1, 2}, {1, 2, 0}, {2, 0, 1}};
    static const int Cm[3][3] = {{0, 1, 2}, {0, 2, 1}, {0, 1, 2}};
    for (int d = 0; d < 3; ++d) { axes[d] = A[aligned - 1][d]; comms[d] = Cm[aligned - 1][d]; }
}

Layout make_pencil_layout(int ndims, const int* gdims, const int* grid, int aligned) {
    Layout L;
    L.id = aligned;
    L.nd = ndims;
    int comms[3];
    perms(ndims, aligned, L.axes, comms);
    const int P = ndims == 3 ? grid[1] * grid[2] : grid[1];
    L.r.resize(P);
    L.off.resize(P + 1);
    i64 off = 0;
    for (int r = 0; r < P; ++r) {
        int c[3] = {0, 0, 0};
        if (ndims == 3) { c[1] = r / grid[2]; c[2] = r % grid[2]; } else c[1] = r;
        i64 n = 1;
        for (int d = 0; d < ndims; ++d) {
            const int cm = comms[d];
            split(gdims[L.axes[d]], grid[cm], c[cm], L.r[r].start[d], L.r[r].count[d]);
            n *= L.r[r].count[d];
        }
        for (int d = ndims; d < 3; ++d) { L.r[r].start[d] = 0; L.r[r].count[d] = 1; }
        L.off[r] = off;
        off += n;
        L.max_local = std::max(L.max_local, n);
    }
    L.off[P] = off;
    L.total = off;
    for (int d = 0; d < ndims; ++d) L.gsize[d] = gdims[L.axes[d]];
    return L;
}

Layout layout_from_boxes(int ndims, int aligned, const int* gdims, const std::vector<RankBox>& boxes) {
    Layout L;
    L.id = aligned;
    L.nd = ndims;
    int comms[3];
    perms(ndims, aligned, L.axes, comms);
    const int P = (int)boxes.size();
    L.r = boxes;
    L.off.resize(P + 1);
    i64 off = 0;
    for (int r = 0; r < P; ++r) {
        i64 n = 1;
        for (int d = 0; d < ndims; ++d) n *= L.r[r].count[d];
        for (int d = ndims; d < 3; ++d) { L.r[r].start[d] = 0; L.r[r].count[d] = 1; }
        L.off[r] = off;
        off += n;
        L.max_local = std::max(L.max_local, n);
    }
    L.off[P] = off;
    L.total = off;
    for (int d = 0; d < ndims; ++d) L.gsize[d] = gdims[L.axes[d]];
    return L;
}

// Box list moving layout S into layout R (same global dims): one box per
// intersecting (source rank, destination rank) pair.
BoxList make_boxes(const Layout& S, const Layout& R, int elem) {
    BoxList bl;
    bl.elem = elem;
    const int nd = S.nd;
    const int a_ax = S.axes[0], b_ax = R.axes[0];
    bl.copy = (a_ax == b_ax);
    int c_ax = -1, b2_ax = -1;
    if (bl.copy) { b2_ax = S.axes[1]; if (nd == 3) c_ax = S.axes[2]; }
    else if (nd == 3) c_ax = 3 - a_ax - b_ax;
    auto pos = [&](const Layout& L, int ax) { for (int d = 0; d < L.nd; ++d) if (L.axes[d] == ax) return d; return -1; };
    const int P = (int)S.r.size();
    for (int i = 0; i < P; ++i) {
        const RankBox& si = S.r[i];
        i64 sstr[3] = {1, si.count[0], (i64)si.count[0] * si.count[1]};
        for (int j = 0; j < P; ++j) {
            const RankBox& rj = R.r[j];
            int lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
            bool empty = false;
            for (int d = 0; d < nd; ++d) {
                const int ax = S.axes[d];
                lo[ax] = si.start[d];
                hi[ax] = si.start[d] + si.count[d];
            }
            for (int d = 0; d < nd; ++d) {
                const int ax = R.axes[d];
                lo[ax] = std::max(lo[ax], rj.start[d]);
                hi[ax] = std::min(hi[ax], rj.start[d] + rj.count[d]);
                if (hi[ax] <= lo[ax]) empty = true;
            }
            for (int ax = 0; ax < nd; ++ax) if (hi[ax] <= lo[ax]) empty = true;
            if (empty) continue;
            i64 rstr[3] = {1, rj.count[0], (i64)rj.count[0] * rj.count[1]};
            Box b;
            memset(&b, 0, sizeof(b));
            b.src_off = S.off[i];
            for (int d = 0; d < nd; ++d) b.src_off += (i64)(lo[S.axes[d]] - si.start[d]) * sstr[d];
            b.dst_off = R.off[j];
            for (int d = 0; d < nd; ++d) b.dst_off += (i64)(lo[R.axes[d]] - rj.start[d]) * rstr[d];
            b.na = hi[a_ax] - lo[a_ax];
            b.a0 = lo[a_ax] - si.start[0];
            if (bl.copy) {
                b.nb = hi[b2_ax] - lo[b2_ax];
                b.sb = sstr[pos(S, b2_ax)];
                b.da_or_db = rstr[pos(R, b2_ax)];
            } else {
                b.nb = hi[b_ax] - lo[b_ax];
                b.sb = sstr[pos(S, b_ax)];
                b.da_or_db = rstr[pos(R, a_ax)];
            }
            if (c_ax >= 0) {
                b.nc = hi[c_ax] - lo[c_ax];
                b.sc = sstr[pos(S, c_ax)];
                b.dc = rstr[pos(R, c_ax)];
            } else {
                b.nc = 1; b.sc = 0; b.dc = 0;
            }
            bl.host.push_back(b);
        }
    }
    return bl;
}

// Default tile per element size: 64-element runs for 4-byte data, 32 otherwise.
TransposeConfig default_tile(int elem) {
    TransposeConfig c;
    // measured on GB300 (c64 512^3 2x4 grid): 8-byte 64x32 at 0.350 ms per 2 GiB
    // transpose vs 0.414 ms for 32x32
    if (elem == 4) { c.tile_a = 64; c.tile_b = 64; c.rows = 8; }
    else if (elem == 8) { c.tile_a = 64; c.tile_b = 32; c.rows = 8; }
    else { c.tile_a = 32; c.tile_b = 32; c.rows = 8; }
    return c;
}

}  // namespace gb

using namespace gb;

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

int32_t dtfft_get_version(void) { return DTFFT_VERSION_CODE; }

int32_t dtfft_vgrid_cart_create(int32_t ndims, const int32_t* dims, MPI_Comm* comm) {
    if (!dims || !comm) return DTFFT_ERROR_INVALID_USAGE;
    if (ndims < 1 || ndims > 3) return DTFFT_ERROR_INVALID_COMM_DIMS;
    VComm v;
    v.cart = true;
    v.ndims = ndims;
    v.nprocs = 1;
    for (int i = 0; i < ndims; ++i) {
        if (dims[i] < 1) return DTFFT_ERROR_INVALID_COMM_DIMS;
        v.dims[i] = dims[i];
        v.nprocs *= dims[i];
    }
    std::lock_guard<std::mutex> lk(g_mu);
    const int h = g_next_comm++;
    g_vcomms[h] = v;
    *comm = (MPI_Comm)h;
    return DTFFT_SUCCESS;
}

int32_t dtfft_vgrid_pencils_create(int32_t nprocs, int32_t ndims, const int32_t* starts, const int32_t* counts,
                                   MPI_Comm* comm) {
    if (!comm || !starts || !counts || nprocs < 1) return DTFFT_ERROR_INVALID_USAGE;
    if (ndims != 2 && ndims != 3) return DTFFT_ERROR_PENCIL_NOT_INITIALIZED;
    VComm v;
    v.cart = false;
    v.nprocs = nprocs;
    v.block_ndims = ndims;
    v.starts.assign(starts, starts + (size_t)nprocs * ndims);
    v.counts.assign(counts, counts + (size_t)nprocs * ndims);
    std::lock_guard<std::mutex> lk(g_mu);
    const int h = g_next_comm++;
    g_vcomms[h] = v;
    *comm = (MPI_Comm)h;
    return DTFFT_SUCCESS;
}

int32_t dtfft_vgrid_world_create(int32_t nprocs, MPI_Comm* comm) {
    if (!comm || nprocs < 1) return DTFFT_ERROR_INVALID_USAGE;
    VComm v;
    v.cart = false;
    v.nprocs = nprocs;
    std::lock_guard<std::mutex> lk(g_mu);
    const int h = g_next_comm++;
    g_vcomms[h] = v;
    *comm = (MPI_Comm)h;
    return DTFFT_SUCCESS;
}

int32_t dtfft_vgrid_comm_size(MPI_Comm comm, int32_t* size) {
    if (!size) return DTFFT_ERROR_INVALID_USAGE;
    if (comm == MPI_COMM_WORLD || comm == MPI_COMM_SELF) { *size = 1; return DTFFT_SUCCESS; }
    VComm v;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!lookup_comm(comm, v)) return DTFFT_ERROR_INVALID_COMM_TYPE;
    *size = v.nprocs;
    return DTFFT_SUCCESS;
}

int32_t dtfft_vgrid_free(MPI_Comm* comm) {
    if (!comm) return DTFFT_ERROR_INVALID_USAGE;
    std::lock_guard<std::mutex> lk(g_mu);
    g_vcomms.erase((int)*comm);
    *comm = MPI_COMM_WORLD;
    return DTFFT_SUCCESS;
}

dtfft_error_t dtfft_create_config(dtfft_config_t* config) {
    if (!config) return DTFFT_ERROR_INVALID_USAGE;
    default_config(config);
    return DTFFT_SUCCESS;
}

dtfft_error_t dtfft_set_config(const dtfft_config_t* c) {
    if (!c) return DTFFT_ERROR_INVALID_USAGE;
    if (c->n_measure_warmup_iters < 0) return DTFFT_ERROR_INVALID_MEASURE_WARMUP_ITERS;
    if (c->n_measure_iters < 1) return DTFFT_ERROR_INVALID_MEASURE_ITERS;
    if (c->platform != DTFFT_PLATFORM_HOST && c->platform != DTFFT_PLATFORM_CUDA) return DTFFT_ERROR_INVALID_PLATFORM;
    if (c->transpose_mode != DTFFT_TRANSPOSE_MODE_PACK && c->transpose_mode != DTFFT_TRANSPOSE_MODE_UNPACK)
        return DTFFT_ERROR_INVALID_TRANSPOSE_MODE;
    if (c->access_mode != DTFFT_ACCESS_MODE_WRITE && c->access_mode != DTFFT_ACCESS_MODE_READ)
        return DTFFT_ERROR_INVALID_ACCESS_MODE;
    config();
    g_cfg = *c;
    return DTFFT_SUCCESS;
}

const char* dtfft_get_error_string(dtfft_error_t e) {
    switch (e) {
    case DTFFT_SUCCESS: return "DTFFT_SUCCESS";
    case DTFFT_ERROR_MPI_FINALIZED: return "MPI_Init is not called or MPI_Finalize has already been called";
    case DTFFT_ERROR_PLAN_NOT_CREATED: return "Plan not created";
    case DTFFT_ERROR_INVALID_TRANSPOSE_TYPE: return "Invalid `transpose_type` provided";
    case DTFFT_ERROR_INVALID_N_DIMENSIONS: return "Invalid Number of dimensions provided. Valid options are 2 and 3";
    case DTFFT_ERROR_INVALID_DIMENSION_SIZE: return "One or more provided dimension sizes <= 0";
    case DTFFT_ERROR_INVALID_COMM_TYPE: return "Invalid communicator type provided";
    case DTFFT_ERROR_INVALID_PRECISION: return "Invalid `precision` parameter provided";
    case DTFFT_ERROR_INVALID_EFFORT: return "Invalid `effort` parameter provided";
    case DTFFT_ERROR_INVALID_EXECUTOR: return "Invalid `executor` parameter provided";
    case DTFFT_ERROR_INVALID_COMM_DIMS: return "Number of dimensions in provided Cartesian communicator > Number of dimension passed to `create` subroutine";
    case DTFFT_ERROR_INVALID_COMM_FAST_DIM: return "Passed Cartesian communicator with number of processes in 1st (fastest varying) dimension > 1";
    case DTFFT_ERROR_MISSING_R2R_KINDS: return "For R2R plan, `kinds` parameter must be passed if `executor` != `DTFFT_EXECUTOR_NONE`";
    case DTFFT_ERROR_INVALID_R2R_KINDS: return "Invalid values detected in `kinds` parameter";
    case DTFFT_ERROR_R2C_TRANSPOSE_PLAN: return "Transpose plan is not supported in R2C, use R2R or C2C plan instead";
    case DTFFT_ERROR_INPLACE_TRANSPOSE: return "Inplace transpose is not supported";
    case DTFFT_ERROR_INVALID_AUX: return "Invalid `aux` buffer provided";
    case DTFFT_ERROR_INVALID_LAYOUT: return "Invalid `layout` passed to `dtfft_get_pencil`";
    case DTFFT_ERROR_INVALID_USAGE: return "Invalid API Usage";
    case DTFFT_ERROR_PLAN_IS_CREATED: return "Trying to create already created plan";
    case DTFFT_ERROR_ALLOC_FAILED: return "Internal call of dtfft_mem_alloc failed";
    case DTFFT_ERROR_FREE_FAILED: return "Internal call of dtfft_mem_free failed";
    case DTFFT_ERROR_INVALID_ALLOC_BYTES: return "Invalid `alloc_bytes` provided";
    case DTFFT_ERROR_DLOPEN_FAILED: return "Failed to dynamically load library";
    case DTFFT_ERROR_DLSYM_FAILED: return "Failed to dynamically load symbol";
    case DTFFT_ERROR_PENCIL_ARRAYS_SIZE_MISMATCH: return "Sizes of `starts` and `counts` arrays passed to `dtfft_pencil_t` constructor do not match";
    case DTFFT_ERROR_PENCIL_ARRAYS_INVALID_SIZES: return "Sizes of `starts` and `counts` < 2 or > 3 provided to `dtfft_pencil_t` constructor";
    case DTFFT_ERROR_PENCIL_INVALID_COUNTS: return "Invalid `counts` provided to `dtfft_pencil_t` constructor";
    case DTFFT_ERROR_PENCIL_INVALID_STARTS: return "Invalid `starts` provided to `dtfft_pencil_t` constructor";
    case DTFFT_ERROR_PENCIL_SHAPE_MISMATCH: return "Processes have same lower bounds but different sizes in some dimensions";
    case DTFFT_ERROR_PENCIL_OVERLAP: return "Pencil overlap detected, i.e. two processes share same part of global space";
    case DTFFT_ERROR_PENCIL_NOT_CONTINUOUS: return "Local pencils do not cover the global space without gaps";
    case DTFFT_ERROR_PENCIL_NOT_INITIALIZED: return "Pencil is not initialized, i.e. `constructor` subroutine was not called";
    case DTFFT_ERROR_INVALID_MEASURE_WARMUP_ITERS: return "Invalid `n_measure_warmup_iters` provided";
    case DTFFT_ERROR_INVALID_MEASURE_ITERS: return "Invalid `n_measure_iters` provided";
    case DTFFT_ERROR_INVALID_REQUEST: return "Invalid `dtfft_request_t` provided";
    case DTFFT_ERROR_TRANSPOSE_ACTIVE: return "Attempting to execute already active transposition";
    case DTFFT_ERROR_TRANSPOSE_NOT_ACTIVE: return "Attempting to finalize non-active transposition";
    case DTFFT_ERROR_INVALID_RESHAPE_TYPE: return "Invalid `reshape_type` provided";
    case DTFFT_ERROR_RESHAPE_ACTIVE: return "Attempting to execute already active reshape";
    case DTFFT_ERROR_RESHAPE_NOT_ACTIVE: return "Attempting to finalize non-active reshape";
    case DTFFT_ERROR_INPLACE_RESHAPE: return "Inplace reshape is not supported";
    case DTFFT_ERROR_INVALID_EXECUTE_TYPE: return "Invalid `execute_type` provided";
    case DTFFT_ERROR_RESHAPE_NOT_SUPPORTED: return "Reshape is not supported for this plan";
    case DTFFT_ERROR_R2C_EXECUTE_CALLED: return "Execute called for transpose-only R2C Plan";
    case DTFFT_ERROR_INVALID_CART_COMM: return "Invalid cartesian communicator provided";
    case DTFFT_ERROR_INVALID_TRANSPOSE_MODE: return "Invalid transpose mode provided";
    case DTFFT_ERROR_INVALID_ACCESS_MODE: return "Invalid access mode provided";
    case DTFFT_ERROR_R2R_FFT_NOT_SUPPORTED: return "Selected `executor` do not support R2R FFTs";
    case DTFFT_ERROR_GPU_INVALID_STREAM: return "Invalid stream provided";
    case DTFFT_ERROR_INVALID_BACKEND: return "Invalid backend provided";
    case DTFFT_ERROR_GPU_NOT_SET: return "Multiple MPI Processes located on same host share same GPU which is not supported";
    case DTFFT_ERROR_VKFFT_R2R_2D_PLAN: return "When using R2R FFT and executor type is vkFFT and plan uses Z-slab optimization, it is required that types of R2R transform are same in X and Y directions";
    case DTFFT_ERROR_BACKENDS_DISABLED: return "Passed `effort` == `DTFFT_PATIENT` but all Backends has been disabled by `dtfft_config_t`";
    case DTFFT_ERROR_NOT_DEVICE_PTR: return "One of pointers passed to `dtfft_execute` or `dtfft_transpose` cannot be accessed from device";
    case DTFFT_ERROR_NOT_NVSHMEM_PTR: return "One of pointers passed to `dtfft_execute` or `dtfft_transpose` is not an `NVSHMEM` pointer";
    case DTFFT_ERROR_INVALID_PLATFORM: return "Invalid platform provided";
    case DTFFT_ERROR_INVALID_PLATFORM_EXECUTOR: return "Invalid executor provided for selected platform";
    case DTFFT_ERROR_INVALID_PLATFORM_BACKEND: return "Invalid backend provided for selected platform";
    case DTFFT_ERROR_GPU_CALL_FAILED: return "A CUDA call made by the library failed";
    case DTFFT_ERROR_FFT_SIZE_NOT_SUPPORTED: return "Transform size is not supported by this library's FFT kernels";
    case DTFFT_ERROR_NOALLOC_SCRATCH_TOO_SMALL:
        return "Plan needs more scratch than the 16 MiB static buffer of dtfft_execute_noalloc; use dtfft_execute";
    case DTFFT_ERROR_GPU_WAIT_TIMEOUT:
        return "A kernel of an earlier call on this device gave up a bounded wait; its output is incomplete";
    default: return "Unknown error";
    }
}

const char* dtfft_get_precision_string(dtfft_precision_t p) {
    return p == DTFFT_SINGLE ? "Single" : (p == DTFFT_DOUBLE ? "Double" : "Unknown precision");
}

const char* dtfft_get_executor_string(dtfft_executor_t e) {
    switch (e) {
    case DTFFT_EXECUTOR_NONE: return "None";
    case DTFFT_EXECUTOR_FFTW3: return "FFTW3";
    case DTFFT_EXECUTOR_MKL: return "MKL";
    case DTFFT_EXECUTOR_CUFFT: return "CUFFT";
    case DTFFT_EXECUTOR_VKFFT: return "VkFFT";
    }
    return "Unknown executor";
}

const char* dtfft_get_backend_string(dtfft_backend_t b) {
    switch (b) {
    case DTFFT_BACKEND_MPI_DATATYPE: return "MPI_DATATYPE";
    case DTFFT_BACKEND_MPI_P2P: return "MPI_P2P";
    case DTFFT_BACKEND_MPI_P2P_PIPELINED: return "MPI_P2P_PIPELINED";
    case DTFFT_BACKEND_MPI_A2A: return "MPI_A2A";
    case DTFFT_BACKEND_MPI_RMA: return "MPI_RMA";
    case DTFFT_BACKEND_MPI_RMA_PIPELINED: return "MPI_RMA_PIPELINED";
    case DTFFT_BACKEND_MPI_P2P_SCHEDULED: return "MPI_P2P_SCHEDULED";
    case DTFFT_BACKEND_MPI_P2P_FUSED: return "MPI_P2P_FUSED";
    case DTFFT_BACKEND_MPI_RMA_FUSED: return "MPI_RMA_FUSED";
    case DTFFT_BACKEND_MPI_P2P_COMPRESSED: return "MPI_P2P_COMPRESSED";
    case DTFFT_BACKEND_MPI_RMA_COMPRESSED: return "MPI_RMA_COMPRESSED";
    case DTFFT_BACKEND_NCCL: return "NCCL";
    case DTFFT_BACKEND_NCCL_PIPELINED: return "NCCL_PIPELINED";
    case DTFFT_BACKEND_NCCL_COMPRESSED: return "NCCL_COMPRESSED";
    case DTFFT_BACKEND_CUFFTMP: return "CUFFTMP";
    case DTFFT_BACKEND_CUFFTMP_PIPELINED: return "CUFFTMP_PIPELINED";
    case DTFFT_BACKEND_ADAPTIVE: return "ADAPTIVE";
    case DTFFT_BACKEND_NONE: return "NONE";
    }
    return "Unknown backend";
}

dtfft_error_t dtfft_get_backend_pipelined(const dtfft_backend_t b, bool* is_pipe) {
    if (!is_pipe) return DTFFT_ERROR_INVALID_USAGE;
    *is_pipe = (b == DTFFT_BACKEND_MPI_P2P_PIPELINED || b == DTFFT_BACKEND_NCCL_PIPELINED ||
                b == DTFFT_BACKEND_CUFFTMP_PIPELINED || b == DTFFT_BACKEND_MPI_RMA_PIPELINED ||
                b == DTFFT_BACKEND_MPI_P2P_FUSED || b == DTFFT_BACKEND_MPI_RMA_FUSED ||
                b == DTFFT_BACKEND_MPI_P2P_COMPRESSED || b == DTFFT_BACKEND_MPI_RMA_COMPRESSED ||
                b == DTFFT_BACKEND_NCCL_COMPRESSED);
    return DTFFT_SUCCESS;
}

int64_t dtfft_gb_kernel_launch_count(void) { return g_launches.load(); }

}  // extern "C"
