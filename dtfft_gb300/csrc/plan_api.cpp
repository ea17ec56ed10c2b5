// dtfft_plan_t of the GB300 execute path: creation, execute / transpose
// schedules and the query functions of the reference's C ABI.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>

#include "plan.h"

namespace gb {

static const uint32_t kPlanMagic = 0x47423330u;  // "GB30"

enum { K_C2C = 0, K_R2C = 1, K_R2R = 2 };

struct Plan {
    uint32_t magic = kPlanMagic;
    int kind = K_C2C;
    int ndims = 3;
    int dims[3] = {1, 1, 1};    // user dims (real dims for R2C), fastest first
    int tdims[3] = {1, 1, 1};   // dims of the transposed type (R2C: dims[0]/2+1)
    dtfft_precision_t precision = DTFFT_DOUBLE;
    dtfft_effort_t effort = DTFFT_ESTIMATE;
    dtfft_executor_t executor = DTFFT_EXECUTOR_NONE;
    int kinds[3] = {0, 0, 0};
    bool transpose_only = true;
    int grid[3] = {1, 1, 1};
    int P = 1;
    bool z_slab = false, y_slab = false;
    bool zs_generic = false;    // Z-slab C2C plan executed through the fused generic schedule
    Layout pen[3];
    Layout real_x;              // R2C: real X pencils
    bool user = false;          // built from every virtual rank's own block
    bool reshape = false;       // the blocks split X: brick <-> pencil reshapes
    bool final_reshape = false; // execute ends in / starts from Fourier-space bricks
    Layout brick_x, brick_z;    // user bricks (real space), Fourier-space bricks
    BoxList rs[4];              // reshape_type - DTFFT_RESHAPE_X_BRICKS_TO_PENCILS
    int elem = 8;               // bytes of a transposed element
    int real_elem = 4;          // bytes of a real element
    BoxList tr[7];              // index transpose_type + 3
    FftPlan* fft[3] = {nullptr, nullptr, nullptr};
    FusedFT* ft[7] = {};        // FFT on the send layout fused with transpose t (index t + 3)
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    void* aux = nullptr;
    int32_t out_dims[3] = {0, 0, 0};
    int32_t out_grid[3] = {0, 0, 0};
    bool log = false;

    ~Plan() {
        for (auto& b : tr) boxes_free(b);
        for (auto& b : rs) boxes_free(b);
        for (auto*& f : fft) { delete f; f = nullptr; }
        for (auto*& f : ft) { delete f; f = nullptr; }
        if (aux) cudaFree(aux);
        if (own_stream && stream) cudaStreamDestroy(stream);
        magic = 0;
    }
    i64 alloc_size() const {
        // src/dtfft_plan.F90:1863-1877: R2C counts real elements
        i64 m = 0;
        for (int d = 0; d < ndims; ++d) m = std::max(m, pen[d].total);
        if (kind == K_R2C) return std::max(real_x.total, 2 * m);
        return m;
    }
    size_t element_size() const { return kind == K_R2C ? (size_t)real_elem : (size_t)elem; }
    size_t alloc_bytes() const { return (size_t)alloc_size() * element_size(); }
    int final_layout() const { return (ndims == 2 || y_slab) ? 2 : 3; }
};

static Plan* as_plan(dtfft_plan_t p) {
    Plan* q = reinterpret_cast<Plan*>(p);
    if (!q || q->magic != kPlanMagic) return nullptr;
    return q;
}


static bool valid_kind(int k) { return k >= DTFFT_DCT_1 && k <= DTFFT_DST_4; }

// Grid choice of src/dtfft_transpose_plan.F90:98-209 for the CUDA platform.
static dtfft_error_t choose_grid(Plan& p, const VCommInfo& vc, bool zs_conf, bool ys_conf) {
    const int nd = p.ndims;
    const int* d = p.tdims;
    int cd[3] = {1, 1, 1};
    p.z_slab = p.y_slab = false;
    if (vc.cart) {
        if (vc.ndims > nd) return DTFFT_ERROR_INVALID_COMM_DIMS;
        if (vc.ndims == nd) {
            if (vc.dims[0] != 1) return DTFFT_ERROR_INVALID_COMM_FAST_DIM;
            for (int i = 0; i < nd; ++i) cd[i] = vc.dims[i];
        } else if (vc.ndims == nd - 1) {
            for (int i = 0; i < vc.ndims; ++i) cd[i + 1] = vc.dims[i];
        } else {
            cd[2] = vc.dims[0];
        }
        if (nd == 3) {
            if (cd[1] == 1 && zs_conf) p.z_slab = true;
            else if (cd[2] == 1 && ys_conf) p.y_slab = true;
        }
    } else {
        const int P = vc.nprocs;
        const int tile = 32;  // DEF_TILE_SIZE, src/dtfft_parameters.F90:555
        if (nd == 2) {
            cd[1] = P;
        } else {
            const bool c1 = tile <= d[2] / P;
            const bool c2 = tile <= d[0] / P && tile <= d[1] / P;
            if (c1 && zs_conf) { cd[2] = P; p.z_slab = true; }
            else if (c2 && ys_conf) { cd[1] = P; p.y_slab = true; }
            else if (c1) cd[2] = P;
            else if (c2) cd[1] = P;
            else {
                // MPI_Dims_create over the two free dims: balanced, non-increasing
                int best_a = P, best_b = 1;
                for (int a = 1; a <= P; ++a)
                    if (P % a == 0 && a >= P / a && a - P / a < best_a - best_b) { best_a = a; best_b = P / a; }
                cd[1] = best_a; cd[2] = best_b;
            }
        }
    }
    for (int i = 0; i < 3; ++i) p.grid[i] = cd[i];
    p.P = nd == 3 ? cd[1] * cd[2] : cd[1];
    return DTFFT_SUCCESS;
}

static int send_layout(int t) { return (t == 1 || t == 3) ? 1 : ((t == -1 || t == 2) ? 2 : 3); }
static int recv_layout(int t) { return (t == -1 || t == -3) ? 1 : ((t == 1 || t == -2) ? 2 : 3); }

static dtfft_error_t build_transposes(Plan& p) {
    std::vector<int> types;
    if (p.ndims == 2) types = {1, -1};
    else {
        types = {1, -1, 2, -2};
        if (p.z_slab) { types.push_back(3); types.push_back(-3); }
    }
    for (int t : types) {
        BoxList& bl = p.tr[t + 3];
        bl = make_boxes(p.pen[send_layout(t) - 1], p.pen[recv_layout(t) - 1], p.elem);
        bl.cfg = default_tile(p.elem);
        tma_default_tile(bl);
        GB_TRY(boxes_upload(bl));
    }
    return DTFFT_SUCCESS;
}

// Brick <-> pencil moves (src/dtfft_reshape_plan.F90:338-367): X reshapes in
// the real element for R2C, Z reshapes in the transformed element.
static dtfft_error_t build_reshapes(Plan& p) {
    if (!p.reshape) return DTFFT_SUCCESS;
    const Layout& xp = p.kind == K_R2C ? p.real_x : p.pen[0];
    const Layout& zp = p.pen[p.ndims - 1];
    const int xe = p.kind == K_R2C ? p.real_elem : p.elem;
    const Layout* from[4] = {&p.brick_x, &xp, &zp, &p.brick_z};
    const Layout* to[4] = {&xp, &p.brick_x, &p.brick_z, &zp};
    const int es[4] = {xe, xe, p.elem, p.elem};
    for (int i = 0; i < 4; ++i) {
        BoxList& bl = p.rs[i];
        bl = make_boxes(*from[i], *to[i], es[i]);
        bl.cfg = default_tile(es[i]);
        GB_TRY(boxes_upload(bl));
    }
    return DTFFT_SUCCESS;
}

// FFT plan along aligned dim d (2D over the slab's two dims with two_d)
// (src/dtfft_plan.F90:2381-2653)
static dtfft_error_t build_fft(Plan& p, int d, bool two_d) {
    const int dbl = p.precision == DTFFT_DOUBLE ? 1 : 0;
    {
        FftDesc fd;
        fd.dbl = dbl;
        fd.rank = two_d ? 2 : 1;
        const Layout& L = (p.kind == K_R2C && d == 1) ? p.real_x : p.pen[d - 1];
        fd.n_fast = L.gsize[0];
        fd.n_slow = two_d ? L.gsize[1] : 1;
        const i64 per = (i64)fd.n_fast * fd.n_slow;
        fd.batch = per > 0 ? L.total / per : 0;
        if (p.kind == K_C2C) {
            fd.type = FFT_C2C;
            fd.idist = fd.odist = fd.n_fast;
        } else if (p.kind == K_R2C) {
            if (d == 1) {
                fd.type = FFT_R2C;
                fd.idist = fd.n_fast;
                fd.odist = fd.n_fast / 2 + 1;
            } else {
                fd.type = FFT_C2C;
                fd.idist = fd.odist = fd.n_fast;
            }
        } else {
            fd.type = FFT_R2R;
            fd.idist = fd.odist = fd.n_fast;
            if (two_d) {
                // 2D kinds of the slab plan (src/dtfft_plan.F90:2419-2434)
                if (p.z_slab) { fd.kind_fast = p.kinds[0]; fd.kind_slow = p.kinds[1]; }
                else { fd.kind_fast = p.kinds[1]; fd.kind_slow = p.kinds[2]; }
            } else {
                fd.kind_fast = p.kinds[d - 1];
            }
        }
        delete p.fft[d - 1];
        p.fft[d - 1] = nullptr;
        GB_TRY(FftPlan::create(fd, &p.fft[d - 1]));
    }
    return DTFFT_SUCCESS;
}

static dtfft_error_t build_ffts(Plan& p) {
    if (p.transpose_only) return DTFFT_SUCCESS;
    for (int d = 1; d <= p.ndims; ++d) {
        if ((p.z_slab && d == 2) || (p.y_slab && d == 3)) continue;
        GB_TRY(build_fft(p, d, (p.z_slab && d == 1) || (p.y_slab && d == 2)));
    }
    return DTFFT_SUCCESS;
}

// Fused FFT + transpose steps of the generic and 2D schedules (C2C axes only).
// A step that does not fit the fused kernel keeps the two-kernel form.
static dtfft_error_t build_fused(Plan& p) {
    if (p.transpose_only || p.kind == K_R2R || p.y_slab) return DTFFT_SUCCESS;
    if (p.z_slab && (p.kind == K_R2R || p.reshape || p.ndims != 3)) return DTFFT_SUCCESS;
    // Default: fuse where the warp-per-row tile kernel or (float) the
    // two-factor kernel takes the rows (they beat FFT + transpose there).
    // DTFFT_GB_FUSE=1 also fuses the other lengths with the register kernels;
    // DTFFT_GB_FUSE=0 keeps every step unfused.
    // Under the tensor-core form (fft_form() == 1) the fused passes stay on
    // the FP32 tile / two-factor kernels and the plain row passes left over
    // (a Z-slab plan's forward Z rows and backward X rows) run on tensor
    // cores where their length has a tensor-core kernel.
    const char* fz = getenv("DTFFT_GB_FUSE");
    if (fz && strcmp(fz, "0") == 0) return DTFFT_SUCCESS;
    const bool tile_only = !(fz && strcmp(fz, "1") == 0);
    const int dbl = p.precision == DTFFT_DOUBLE ? 1 : 0;
    std::vector<std::pair<int, int>> steps;   // (transpose type, FFT dim on its send layout)
    if (p.ndims == 2) steps = {{1, 1}, {-1, 2}};
    else steps = {{1, 1}, {2, 2}, {-2, 3}, {-1, 2}};
    for (auto st : steps) {
        const int t = st.first, d = st.second;
        if (p.kind == K_R2C && d == 1) continue;   // the X axis is R2C
        const BoxList& bl = p.tr[t + 3];
        if (bl.host.empty() || (!p.fft[d - 1] && !p.z_slab)) continue;
        FusedFT* f = nullptr;
        if (FusedFT::create(bl, p.pen[d - 1].gsize[0], dbl, p.z_slab || tile_only, &f) == DTFFT_SUCCESS)
            p.ft[t + 3] = f;
    }
    if (!p.z_slab) return DTFFT_SUCCESS;
    // A Z-slab plan on one GPU: when every FFT + transpose pass fuses (C2C: all
    // four; R2C: the three after the real X axis), the generic X -> Y -> Z
    // schedule moves the data fewer times than the slab's 2D FFT (rows +
    // strided columns) + X -> Z + Z rows, with the same result in the same
    // Z-pencil layout.
    bool all = true;   // (an R2C plan's X axis is R2C: its step never fuses)
    for (auto st : steps) all = all && (p.ft[st.first + 3] != nullptr || (p.kind == K_R2C && st.second == 1));
    if (all && build_fft(p, 1, false) == DTFFT_SUCCESS && build_fft(p, 2, false) == DTFFT_SUCCESS) {
        p.zs_generic = true;
        return DTFFT_SUCCESS;
    }
    for (auto st : steps) { delete p.ft[st.first + 3]; p.ft[st.first + 3] = nullptr; }
    if (!all) return DTFFT_SUCCESS;
    // the rank-1 plans could not be built: back to the slab's 2D plan
    delete p.fft[1];
    p.fft[1] = nullptr;
    return build_fft(p, 1, true);
}

static dtfft_error_t create_plan(int kind, int8_t ndims, const int32_t* dims, const int32_t* kinds,
                                 MPI_Comm comm, dtfft_precision_t precision, dtfft_effort_t effort,
                                 dtfft_executor_t executor, dtfft_plan_t* out, const UserGeometry* ug = nullptr) {
    TraceRange tr("dtfft_create_plan");
    if (!out) return DTFFT_ERROR_INVALID_USAGE;
    *out = nullptr;
    // check_create_args order (src/dtfft_plan.F90:2107-2219)
    if (ndims != 2 && ndims != 3) return DTFFT_ERROR_INVALID_N_DIMENSIONS;
    if (!dims) return DTFFT_ERROR_INVALID_USAGE;
    for (int i = 0; i < ndims; ++i) if (dims[i] <= 0) return DTFFT_ERROR_INVALID_DIMENSION_SIZE;
    VCommInfo vc = comm_info(comm);
    if (!vc.known) return DTFFT_ERROR_INVALID_COMM_TYPE;
    if (precision != DTFFT_SINGLE && precision != DTFFT_DOUBLE) return DTFFT_ERROR_INVALID_PRECISION;
    if (effort < DTFFT_ESTIMATE || effort > DTFFT_EXHAUSTIVE) return DTFFT_ERROR_INVALID_EFFORT;
    if (executor < DTFFT_EXECUTOR_NONE || executor > DTFFT_EXECUTOR_VKFFT) return DTFFT_ERROR_INVALID_EXECUTOR;
    const dtfft_config_t& cfg = config();
    if (cfg.platform != DTFFT_PLATFORM_CUDA) return DTFFT_ERROR_INVALID_PLATFORM;
    if (executor == DTFFT_EXECUTOR_FFTW3 || executor == DTFFT_EXECUTOR_MKL) return DTFFT_ERROR_INVALID_PLATFORM_EXECUTOR;
    const bool tonly = executor == DTFFT_EXECUTOR_NONE;
    if (kind == K_R2R && !tonly && kinds)
        for (int i = 0; i < ndims; ++i) if (!valid_kind(kinds[i])) return DTFFT_ERROR_INVALID_R2R_KINDS;

    Plan* p = new Plan();
    p->kind = kind;
    p->ndims = ndims;
    for (int i = 0; i < ndims; ++i) p->dims[i] = p->tdims[i] = dims[i];
    if (kind == K_R2C) p->tdims[0] = dims[0] / 2 + 1;
    p->precision = precision;
    p->effort = effort;
    p->executor = executor;
    p->transpose_only = tonly;
    p->log = cfg.enable_log;
    const int real = precision == DTFFT_DOUBLE ? 8 : 4;
    p->real_elem = real;
    p->elem = kind == K_R2R ? real : 2 * real;

    dtfft_error_t e = DTFFT_SUCCESS;
    if (ug) {
        // every rank's own block (src/dtfft_plan.F90:2014-2089)
        p->user = true;
        for (int i = 0; i < 3; ++i) p->grid[i] = ug->grid[i];
        p->P = (int)ug->pen[0].r.size();
        p->z_slab = ug->z_slab;
        p->y_slab = ug->y_slab;
        for (int d = 0; d < ndims; ++d) p->pen[d] = ug->pen[d];
        if (kind == K_R2C) p->real_x = ug->real_x;
        p->reshape = ug->reshape;
        if (p->reshape) {
            p->brick_x = ug->brick_x;
            p->brick_z = ug->brick_z;
            p->final_reshape = ug->final_grid > 1 && cfg.enable_fourier_reshape && !p->z_slab;
        }
    } else {
        e = choose_grid(*p, vc, cfg.enable_z_slab, cfg.enable_y_slab);
        if (e == DTFFT_SUCCESS) {
            for (int d = 0; d < ndims; ++d) p->pen[d] = make_pencil_layout(ndims, p->tdims, p->grid, d + 1);
            if (kind == K_R2C) p->real_x = make_pencil_layout(ndims, p->dims, p->grid, 1);
        }
    }
    if (e == DTFFT_SUCCESS) {
        if (kind == K_R2R && !tonly && !kinds) e = DTFFT_ERROR_MISSING_R2R_KINDS;
        if (kind == K_R2R && !tonly && executor == DTFFT_EXECUTOR_CUFFT) e = DTFFT_ERROR_R2R_FFT_NOT_SUPPORTED;
    }
    if (e == DTFFT_SUCCESS && kind == K_R2R && kinds)
        for (int i = 0; i < ndims; ++i) p->kinds[i] = kinds[i];
    if (e == DTFFT_SUCCESS) {
        if (cfg.stream) { p->stream = (cudaStream_t)cfg.stream; p->own_stream = false; }
        else if (cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) == cudaSuccess) p->own_stream = true;
        else e = DTFFT_ERROR_GPU_CALL_FAILED;
    }
    if (e == DTFFT_SUCCESS) e = status_setup();
    if (e == DTFFT_SUCCESS) e = build_transposes(*p);
    if (e == DTFFT_SUCCESS) e = build_reshapes(*p);
    if (e == DTFFT_SUCCESS) e = build_ffts(*p);
    if (e == DTFFT_SUCCESS) e = build_fused(*p);
    if (e == DTFFT_SUCCESS && (effort == DTFFT_EXHAUSTIVE || cfg.enable_kernel_autotune)) {
        for (auto& bl : p->tr) {
            if (bl.host.empty()) continue;
            e = autotune_boxes(bl, p->alloc_size(), p->stream, cfg.n_measure_warmup_iters, cfg.n_measure_iters, p->log);
            if (e != DTFFT_SUCCESS) break;
        }
        for (FusedFT* f : p->ft) {
            if (!f || e != DTFFT_SUCCESS) continue;
            const i64 elems = p->kind == K_R2C ? p->alloc_size() / 2 : p->alloc_size();   // transformed elements
            e = f->autotune(elems, p->stream, cfg.n_measure_warmup_iters, cfg.n_measure_iters, p->log);
        }
        for (FftPlan* f : p->fft) {
            if (!f || e != DTFFT_SUCCESS) continue;
            e = f->autotune(p->stream, cfg.n_measure_warmup_iters, cfg.n_measure_iters, p->log);
        }
    }
    if (e != DTFFT_SUCCESS) { delete p; return e; }
    for (int i = 0; i < ndims; ++i) { p->out_dims[i] = p->dims[i]; p->out_grid[i] = p->grid[i]; }
    *out = p;
    return DTFFT_SUCCESS;
}

static bool is_device_ptr(const void* ptr) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) { cudaGetLastError(); return false; }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

static dtfft_error_t check_ptrs(const void* in, const void* out, const void* aux) {
    if (!is_device_ptr(in) || !is_device_ptr(out)) return DTFFT_ERROR_NOT_DEVICE_PTR;
    if (aux && !is_device_ptr(aux)) return DTFFT_ERROR_NOT_DEVICE_PTR;
    return DTFFT_SUCCESS;
}

// aux buffer: user's or allocated once (src/dtfft_plan.F90:2286-2331)
static dtfft_error_t get_aux(Plan& p, void* aux, void** out) {
    if (aux) { *out = aux; return DTFFT_SUCCESS; }
    if (!p.aux) {
        size_t bytes = p.alloc_bytes();
        if (cudaMalloc(&p.aux, std::max<size_t>(bytes, 16)) != cudaSuccess) {
            cudaGetLastError();
            p.aux = nullptr;
            return DTFFT_ERROR_ALLOC_FAILED;
        }
    }
    *out = p.aux;
    return DTFFT_SUCCESS;
}

static dtfft_error_t T(Plan& p, int t, const void* in, void* out) {
    return boxes_launch(p.tr[t + 3], in, out, p.stream);
}

static dtfft_error_t F(Plan& p, int d, const void* in, void* out, int sign) {
    FftPlan* f = p.fft[d - 1];
    if (!f) return DTFFT_SUCCESS;
    return f->execute(in, out, sign, p.stream);
}

static dtfft_error_t RS(Plan& p, int type, const void* in, void* out) {
    return boxes_launch(p.rs[type - DTFFT_RESHAPE_X_BRICKS_TO_PENCILS], in, out, p.stream);
}

// execute_2d_reshape / execute_z_slab_reshape / execute_generic_reshape
// (src/dtfft_plan.F90:915-966,1018-1048,1103-1162), with their buffer roles.
static dtfft_error_t run_execute_reshape(Plan& p, void* in, void* out, bool fwd, void* aux) {
    const int S = fwd ? FFT_FWD : FFT_BWD;
    const int XB2P = DTFFT_RESHAPE_X_BRICKS_TO_PENCILS, XP2B = DTFFT_RESHAPE_X_PENCILS_TO_BRICKS;
    const int ZP2B = DTFFT_RESHAPE_Z_PENCILS_TO_BRICKS, ZB2P = DTFFT_RESHAPE_Z_BRICKS_TO_PENCILS;
    const bool fin = p.final_reshape;
    if (p.ndims == 2 || p.y_slab) {
        if (p.transpose_only) {
            if (fwd) {
                GB_TRY(RS(p, XB2P, in, aux));
                if (fin) { GB_TRY(T(p, 1, aux, in)); return RS(p, ZP2B, in, out); }
                return T(p, 1, aux, out);
            }
            if (fin) { GB_TRY(RS(p, ZB2P, in, out)); GB_TRY(T(p, -1, out, aux)); }
            else GB_TRY(T(p, -1, in, aux));
            return RS(p, XP2B, aux, out);
        }
        if (fwd) {
            GB_TRY(RS(p, XB2P, in, aux));
            GB_TRY(F(p, 1, aux, out, S));
            GB_TRY(T(p, 1, out, aux));
            if (fin) { GB_TRY(F(p, 2, aux, aux, S)); return RS(p, ZP2B, aux, out); }
            return F(p, 2, aux, out, S);
        }
        if (fin) { GB_TRY(RS(p, ZB2P, in, aux)); GB_TRY(F(p, 2, aux, aux, S)); }
        else GB_TRY(F(p, 2, in, aux, S));
        GB_TRY(T(p, -1, aux, in));
        GB_TRY(F(p, 1, in, aux, S));
        return RS(p, XP2B, aux, out);
    }
    if (p.z_slab) {
        if (p.transpose_only) {
            if (fwd) { GB_TRY(RS(p, XB2P, in, aux)); return T(p, 3, aux, out); }
            GB_TRY(T(p, -3, in, aux));
            return RS(p, XP2B, aux, out);
        }
        if (fwd) {
            GB_TRY(RS(p, XB2P, in, aux));
            GB_TRY(F(p, 1, aux, in, S));
            GB_TRY(T(p, 3, in, aux));
            return F(p, 3, aux, out, S);
        }
        GB_TRY(F(p, 3, in, aux, S));
        GB_TRY(T(p, -3, aux, in));
        GB_TRY(F(p, 1, in, aux, S));
        return RS(p, XP2B, aux, out);
    }
    if (p.transpose_only) {
        if (fwd) {
            GB_TRY(RS(p, XB2P, in, aux));
            GB_TRY(T(p, 1, aux, in));
            if (fin) { GB_TRY(T(p, 2, in, aux)); return RS(p, ZP2B, aux, out); }
            return T(p, 2, in, out);
        }
        if (fin) { GB_TRY(RS(p, ZB2P, in, aux)); GB_TRY(T(p, -2, aux, out)); }
        else GB_TRY(T(p, -2, in, out));
        GB_TRY(T(p, -1, out, aux));
        return RS(p, XP2B, aux, out);
    }
    if (fwd) {
        GB_TRY(RS(p, XB2P, in, aux));
        GB_TRY(F(p, 1, aux, out, S));
        GB_TRY(T(p, 1, out, aux));
        GB_TRY(F(p, 2, aux, aux, S));
        GB_TRY(T(p, 2, aux, out));
        if (fin) { GB_TRY(F(p, 3, out, aux, S)); return RS(p, ZP2B, aux, out); }
        return F(p, 3, out, out, S);
    }
    if (fin) { GB_TRY(RS(p, ZB2P, in, aux)); GB_TRY(F(p, 3, aux, in, S)); }
    else GB_TRY(F(p, 3, in, in, S));
    GB_TRY(T(p, -2, in, aux));
    GB_TRY(F(p, 2, aux, aux, S));
    GB_TRY(T(p, -1, aux, in));
    GB_TRY(F(p, 1, in, aux, S));
    return RS(p, XP2B, aux, out);
}

// FFT along the send layout of transpose t followed by transpose t, from
// `src` to `dst`: one fused pass when the plan built one and it can run on
// these buffers, else FFT in place on `src` then the transpose.  `src` is
// clobbered either way.
static dtfft_error_t FT(Plan& p, int t, void* src, void* dst, int S) {
    FusedFT* f = p.ft[t + 3];
    if (f && f->usable(src, dst)) return f->execute(src, dst, S, p.stream);
    const int d = t == 1 ? 1 : (t == 2 || t == -1) ? 2 : 3;
    GB_TRY(F(p, d, src, src, S));
    return T(p, t, src, dst);
}
static bool fused(const Plan& p, int t) { return p.ft[t + 3] != nullptr; }

// execute_2d / execute_z_slab / execute_generic (src/dtfft_plan.F90:877-1101).
// Buffer roles follow the reference's: `in` may be clobbered by the backward
// direction, `aux` holds intermediate layouts, and in == out is allowed.
static dtfft_error_t run_execute(Plan& p, void* in, void* out, bool fwd, void* aux, bool inplace) {
    if (p.reshape) return run_execute_reshape(p, in, out, fwd, aux);
    const int S = fwd ? FFT_FWD : FFT_BWD;
    if (p.ndims == 2 || p.y_slab) {
        if (p.transpose_only) return T(p, fwd ? 1 : -1, in, out);
        if (fwd) {
            // fft(1) + X->Y, then fft(2) in place
            if (fused(p, 1)) {
                void* y = inplace ? aux : out;
                GB_TRY(FT(p, 1, in, y, S));
                return F(p, 2, y, out, S);
            }
            GB_TRY(F(p, 1, in, aux, S));
            GB_TRY(T(p, 1, aux, out));
            return F(p, 2, out, out, S);
        }
        GB_TRY(FT(p, -1, in, aux, S));   // fft(2) + Y->X
        return F(p, 1, aux, out, S);
    }
    if (p.z_slab && !p.zs_generic && !(p.transpose_only && inplace)) {
        if (p.transpose_only) return T(p, fwd ? 3 : -3, in, out);
        if (fwd) {
            GB_TRY(F(p, 1, in, aux, S));
            GB_TRY(T(p, 3, aux, out));
            return F(p, 3, out, out, S);
        }
        GB_TRY(F(p, 3, in, in, S));
        GB_TRY(T(p, -3, in, aux));
        return F(p, 1, aux, out, S);
    }
    if (p.transpose_only) {
        if (fwd) { GB_TRY(T(p, 1, in, aux)); return T(p, 2, aux, out); }
        GB_TRY(T(p, -2, in, aux));
        return T(p, -1, aux, out);
    }
    // generic schedule (also the single-GPU route of Z-slab C2C plans whose
    // passes all fuse: three HBM passes instead of the slab's four)
    if (fwd) {
        void* y;                                   // Y-pencil data after fft(1) + X->Y
        if (fused(p, 1)) { y = inplace ? aux : out; GB_TRY(FT(p, 1, in, y, S)); }
        else { GB_TRY(F(p, 1, in, aux, S)); GB_TRY(T(p, 1, aux, out)); y = out; }
        void* z = y == aux ? out : aux;            // Z-pencil data after fft(2) + Y->Z
        GB_TRY(FT(p, 2, y, z, S));
        return F(p, 3, z, out, S);
    }
    void* y;                                       // Y-pencil data after fft(3) + Z->Y
    if (fused(p, -2)) { y = aux; GB_TRY(FT(p, -2, in, aux, S)); }
    else { GB_TRY(F(p, 3, in, aux, S)); GB_TRY(T(p, -2, aux, in)); y = in; }
    void* x = y == aux ? in : aux;                 // X-pencil data after fft(2) + Y->X
    GB_TRY(FT(p, -1, y, x, S));
    return F(p, 1, x, out, S);
}

struct Request { uint32_t magic; int type; };
static const uint32_t kReqMagic = 0x52455131u;

}  // namespace gb

using namespace gb;


extern "C" {

dtfft_error_t dtfft_create_plan_c2c(int8_t ndims, const int32_t* dims, MPI_Comm comm, dtfft_precision_t precision,
                                    dtfft_effort_t effort, dtfft_executor_t executor, dtfft_plan_t* plan) {
    return create_plan(K_C2C, ndims, dims, nullptr, comm, precision, effort, executor, plan);
}

dtfft_error_t dtfft_create_plan_r2c(int8_t ndims, const int32_t* dims, MPI_Comm comm, dtfft_precision_t precision,
                                    dtfft_effort_t effort, dtfft_executor_t executor, dtfft_plan_t* plan) {
    if (executor == DTFFT_EXECUTOR_NONE) {
        // a transpose-only R2C plan can be created; execute then reports R2C_EXECUTE_CALLED
    }
    return create_plan(K_R2C, ndims, dims, nullptr, comm, precision, effort, executor, plan);
}

dtfft_error_t dtfft_create_plan_r2r(int8_t ndims, const int32_t* dims, const dtfft_r2r_kind_t* kinds, MPI_Comm comm,
                                    dtfft_precision_t precision, dtfft_effort_t effort, dtfft_executor_t executor,
                                    dtfft_plan_t* plan) {
    return create_plan(K_R2R, ndims, dims, (const int32_t*)kinds, comm, precision, effort, executor, plan);
}

// Pencil constructors: one process owns the whole domain, so the pencil must
// start at zero in every dim (src/dtfft_pencil.F90:777-1081 would report a gap
// otherwise); its counts are the global dims.
static dtfft_error_t pencil_dims(const dtfft_pencil_t* pencil, MPI_Comm comm, int32_t* dims) {
    if (!pencil) return DTFFT_ERROR_INVALID_USAGE;
    if (pencil->ndims != 2 && pencil->ndims != 3) return DTFFT_ERROR_PENCIL_NOT_INITIALIZED;
    VCommInfo vc = comm_info(comm);
    if (!vc.known) return DTFFT_ERROR_INVALID_COMM_TYPE;
    if (vc.nprocs != 1) return DTFFT_ERROR_INVALID_USAGE;
    for (int i = 0; i < pencil->ndims; ++i) {
        if (pencil->counts[i] <= 0) return DTFFT_ERROR_PENCIL_INVALID_COUNTS;
        if (pencil->starts[i] < 0) return DTFFT_ERROR_PENCIL_INVALID_STARTS;
        if (pencil->starts[i] != 0) return DTFFT_ERROR_PENCIL_NOT_CONTINUOUS;
        dims[i] = pencil->counts[i];
    }
    return DTFFT_SUCCESS;
}

// Virtual ranks with their own blocks (dtfft_vgrid_pencils_create): the
// calling process plays virtual rank 0, so `pencil` is rank 0's block; the
// plan covers every rank (src/dtfft_plan.F90:2014-2089).
static dtfft_error_t create_user_plan(int kind, const dtfft_pencil_t* pencil, const int32_t* kinds, MPI_Comm comm,
                                      dtfft_precision_t precision, dtfft_effort_t effort, dtfft_executor_t executor,
                                      dtfft_plan_t* plan) {
    if (!plan) return DTFFT_ERROR_INVALID_USAGE;
    if (!pencil) return DTFFT_ERROR_INVALID_USAGE;
    if (pencil->ndims != 2 && pencil->ndims != 3) return DTFFT_ERROR_PENCIL_NOT_INITIALIZED;
    int bnd = 0;
    std::vector<int32_t> st, ct;
    if (comm_blocks(comm, &bnd, &st, &ct)) {
        if (bnd != pencil->ndims) return DTFFT_ERROR_PENCIL_ARRAYS_SIZE_MISMATCH;
        for (int d = 0; d < bnd; ++d)
            if (pencil->starts[d] != st[d] || pencil->counts[d] != ct[d]) return DTFFT_ERROR_PENCIL_SHAPE_MISMATCH;
        const int P = (int)(st.size() / bnd);
        UserGeometry g;
        const dtfft_config_t& cfg = config();
        GB_TRY(user_geometry(bnd, P, st.data(), ct.data(), kind == K_R2C, cfg.enable_z_slab, cfg.enable_y_slab, g));
        return create_plan(kind, (int8_t)bnd, g.dims, kinds, comm, precision, effort, executor, plan, &g);
    }
    int32_t dims[3];
    GB_TRY(pencil_dims(pencil, comm, dims));
    return create_plan(kind, pencil->ndims, dims, kinds, comm, precision, effort, executor, plan);
}

dtfft_error_t dtfft_create_plan_c2c_pencil(const dtfft_pencil_t* pencil, MPI_Comm comm, dtfft_precision_t precision,
                                           dtfft_effort_t effort, dtfft_executor_t executor, dtfft_plan_t* plan) {
    return create_user_plan(K_C2C, pencil, nullptr, comm, precision, effort, executor, plan);
}

dtfft_error_t dtfft_create_plan_r2c_pencil(const dtfft_pencil_t* pencil, MPI_Comm comm, dtfft_precision_t precision,
                                           dtfft_effort_t effort, dtfft_executor_t executor, dtfft_plan_t* plan) {
    return create_user_plan(K_R2C, pencil, nullptr, comm, precision, effort, executor, plan);
}

dtfft_error_t dtfft_create_plan_r2r_pencil(const dtfft_pencil_t* pencil, const dtfft_r2r_kind_t* kinds, MPI_Comm comm,
                                           dtfft_precision_t precision, dtfft_effort_t effort,
                                           dtfft_executor_t executor, dtfft_plan_t* plan) {
    return create_user_plan(K_R2R, pencil, (const int32_t*)kinds, comm, precision, effort, executor, plan);
}

dtfft_error_t dtfft_destroy(dtfft_plan_t* plan) {
    if (!plan) return DTFFT_ERROR_INVALID_USAGE;
    Plan* p = as_plan(*plan);
    if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    if (p->stream) cudaStreamSynchronize(p->stream);
    delete p;
    *plan = nullptr;
    return DTFFT_SUCCESS;
}

// execute_private checks (src/dtfft_plan.F90:780-835)
static dtfft_error_t execute_checks(Plan* p, void* in, void* out, int execute_type, void* aux) {
    if (!in || !out) return DTFFT_ERROR_INVALID_USAGE;
    if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    if (execute_type != DTFFT_EXECUTE_FORWARD && execute_type != DTFFT_EXECUTE_BACKWARD)
        return DTFFT_ERROR_INVALID_EXECUTE_TYPE;
    const bool inplace = in == out;
    if (p->transpose_only && inplace && (p->ndims == 2 || p->y_slab || (p->reshape && !p->final_reshape)))
        return DTFFT_ERROR_INPLACE_TRANSPOSE;
    if (aux && (aux == in || aux == out)) return DTFFT_ERROR_INVALID_AUX;
    if (p->transpose_only && p->kind == K_R2C) return DTFFT_ERROR_R2C_EXECUTE_CALLED;
    return check_ptrs(in, out, aux);
}

dtfft_error_t dtfft_execute(dtfft_plan_t plan, void* in, void* out, dtfft_execute_t execute_type, void* aux) {
    TraceRange tr("dtfft_execute");
    Plan* p = as_plan(plan);
    GB_TRY(execute_checks(p, in, out, (int)execute_type, aux));
    GB_TRY(check_device_status());
    void* a = nullptr;
    GB_TRY(get_aux(*p, aux, &a));
    return run_execute(*p, in, out, execute_type == DTFFT_EXECUTE_FORWARD, a, in == out);
}

}  // extern "C"

namespace gb {
// Execute with caller-provided scratch of `scratch_bytes` (used by the
// no-allocation entry point in noalloc.cu): the checks of dtfft_execute, then
// the same schedule with `scratch` as aux.  Never allocates.
dtfft_error_t execute_into_scratch(dtfft_plan_t plan, void* in, void* out, int execute_type, void* scratch,
                                   size_t scratch_bytes, size_t* needed) {
    TraceRange tr("dtfft_execute_noalloc");
    if (!in || !out) return DTFFT_ERROR_INVALID_USAGE;
    Plan* p = as_plan(plan);
    if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    if (execute_type != DTFFT_EXECUTE_FORWARD && execute_type != DTFFT_EXECUTE_BACKWARD)
        return DTFFT_ERROR_INVALID_EXECUTE_TYPE;
    const bool inplace = in == out;
    if (p->transpose_only && inplace && (p->ndims == 2 || p->y_slab || (p->reshape && !p->final_reshape)))
        return DTFFT_ERROR_INPLACE_TRANSPOSE;
    if (p->transpose_only && p->kind == K_R2C) return DTFFT_ERROR_R2C_EXECUTE_CALLED;
    if (needed) *needed = p->alloc_bytes();
    if (p->alloc_bytes() > scratch_bytes) return DTFFT_ERROR_NOALLOC_SCRATCH_TOO_SMALL;
    GB_TRY(check_ptrs(in, out, nullptr));
    GB_TRY(check_device_status());
    return run_execute(*p, in, out, execute_type == DTFFT_EXECUTE_FORWARD, scratch, inplace);
}
}  // namespace gb

extern "C" {

static dtfft_error_t transpose_checks(Plan* p, void* in, void* out, int t, void* aux) {
    const bool valid = (t >= -3 && t <= 3 && t != 0);
    if (!valid || (p->ndims == 2 && std::abs(t) > 1) || (std::abs(t) == 3 && !p->z_slab))
        return DTFFT_ERROR_INVALID_TRANSPOSE_TYPE;
    if (in == out) return DTFFT_ERROR_INPLACE_TRANSPOSE;
    if (aux && (aux == in || aux == out)) return DTFFT_ERROR_INVALID_AUX;
    return check_ptrs(in, out, aux);
}

dtfft_error_t dtfft_transpose(dtfft_plan_t plan, void* in, void* out, dtfft_transpose_t t, void* aux) {
    TraceRange tr("dtfft_transpose");
    if (!in || !out) return DTFFT_ERROR_INVALID_USAGE;
    Plan* p = as_plan(plan);
    if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    GB_TRY(transpose_checks(p, in, out, (int)t, aux));
    GB_TRY(check_device_status());
    return T(*p, (int)t, in, out);
}

dtfft_error_t dtfft_transpose_start(dtfft_plan_t plan, void* in, void* out, dtfft_transpose_t t, void* aux,
                                    dtfft_request_t* request) {
    TraceRange tr("dtfft_transpose_start");
    if (!in || !out || !request) return DTFFT_ERROR_INVALID_USAGE;
    Plan* p = as_plan(plan);
    if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    GB_TRY(transpose_checks(p, in, out, (int)t, aux));
    GB_TRY(check_device_status());
    // the move is one kernel on the plan stream; the request only records it
    GB_TRY(T(*p, (int)t, in, out));
    Request* r = new Request{kReqMagic, (int)t};
    *request = r;
    return DTFFT_SUCCESS;
}

dtfft_error_t dtfft_transpose_end(dtfft_plan_t plan, dtfft_request_t request) {
    Plan* p = as_plan(plan);
    if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    Request* r = reinterpret_cast<Request*>(request);
    if (!r || r->magic != kReqMagic) return DTFFT_ERROR_INVALID_REQUEST;
    if (r->type >= DTFFT_RESHAPE_X_BRICKS_TO_PENCILS) return DTFFT_ERROR_INVALID_REQUEST;
    r->magic = 0;
    delete r;
    return DTFFT_SUCCESS;
}

// reshape_private checks (src/dtfft_plan.F90:508-537)
static dtfft_error_t reshape_checks(Plan* p, void* in, void* out, int t, void* aux) {
    if (t < DTFFT_RESHAPE_X_BRICKS_TO_PENCILS || t > DTFFT_RESHAPE_Z_BRICKS_TO_PENCILS)
        return DTFFT_ERROR_INVALID_RESHAPE_TYPE;
    if (in == out) return DTFFT_ERROR_INPLACE_RESHAPE;
    if (!p->reshape) return DTFFT_ERROR_RESHAPE_NOT_SUPPORTED;
    if (aux && (aux == in || aux == out)) return DTFFT_ERROR_INVALID_AUX;
    return check_ptrs(in, out, aux);
}

dtfft_error_t dtfft_reshape(dtfft_plan_t plan, void* in, void* out, dtfft_reshape_t reshape_type, void* aux) {
    TraceRange tr("dtfft_reshape");
    if (!in || !out) return DTFFT_ERROR_INVALID_USAGE;
    Plan* p = as_plan(plan);
    if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    GB_TRY(reshape_checks(p, in, out, (int)reshape_type, aux));
    GB_TRY(check_device_status());
    return RS(*p, (int)reshape_type, in, out);
}

dtfft_error_t dtfft_reshape_start(dtfft_plan_t plan, void* in, void* out, dtfft_reshape_t reshape_type, void* aux,
                                  dtfft_request_t* request) {
    TraceRange tr("dtfft_reshape_start");
    if (!in || !out || !request) return DTFFT_ERROR_INVALID_USAGE;
    Plan* p = as_plan(plan);
    if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    GB_TRY(reshape_checks(p, in, out, (int)reshape_type, aux));
    GB_TRY(check_device_status());
    // one copy kernel on the plan stream; the request only records it
    GB_TRY(RS(*p, (int)reshape_type, in, out));
    Request* r = new Request{kReqMagic, (int)reshape_type};
    *request = r;
    return DTFFT_SUCCESS;
}

dtfft_error_t dtfft_reshape_end(dtfft_plan_t plan, dtfft_request_t request) {
    Plan* p = as_plan(plan);
    if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    Request* r = reinterpret_cast<Request*>(request);
    if (!r || r->magic != kReqMagic) return DTFFT_ERROR_INVALID_REQUEST;
    if (r->type < DTFFT_RESHAPE_X_BRICKS_TO_PENCILS) return DTFFT_ERROR_INVALID_REQUEST;
    r->magic = 0;
    delete r;
    return DTFFT_SUCCESS;
}

dtfft_error_t dtfft_get_z_slab_enabled(dtfft_plan_t plan, bool* v) {
    if (!v) return DTFFT_ERROR_INVALID_USAGE;
    Plan* p = as_plan(plan); if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    *v = p->z_slab; return DTFFT_SUCCESS;
}

dtfft_error_t dtfft_get_y_slab_enabled(dtfft_plan_t plan, bool* v) {
    if (!v) return DTFFT_ERROR_INVALID_USAGE;
    Plan* p = as_plan(plan); if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    *v = p->y_slab; return DTFFT_SUCCESS;
}

// Local sizes.  One process: the reference's values.  Several virtual ranks:
// the process owns every rank, so starts are 0, counts are the global extents
// of the layout and alloc_size covers the packed buffer of all ranks.
static void box_of(const Plan& p, const Layout& L, int32_t* starts, int32_t* counts) {
    for (int d = 0; d < p.ndims; ++d) {
        // report in natural (X, Y, Z) order like get_local_sizes does for the
        // X pencil; for the output layout the reference reports the pencil's own order
        if (p.P == 1) { if (starts) starts[d] = L.r[0].start[d]; if (counts) counts[d] = L.r[0].count[d]; }
        else { if (starts) starts[d] = 0; if (counts) counts[d] = L.gsize[d]; }
    }
}

dtfft_error_t dtfft_get_local_sizes(dtfft_plan_t plan, int32_t* in_starts, int32_t* in_counts, int32_t* out_starts,
                                    int32_t* out_counts, size_t* alloc_size) {
    Plan* p = as_plan(plan);
    if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    if (!in_starts && !in_counts && !out_starts && !out_counts && !alloc_size) return DTFFT_ERROR_INVALID_USAGE;
    const Layout& in_l = p->kind == K_R2C ? p->real_x : p->pen[0];
    const Layout& out_l = p->pen[p->final_layout() - 1];
    box_of(*p, in_l, in_starts, in_counts);
    box_of(*p, out_l, out_starts, out_counts);
    if (alloc_size) *alloc_size = (size_t)p->alloc_size();
    return DTFFT_SUCCESS;
}

dtfft_error_t dtfft_get_alloc_size(dtfft_plan_t plan, size_t* alloc_size) {
    if (!alloc_size) return DTFFT_ERROR_INVALID_USAGE;
    return dtfft_get_local_sizes(plan, nullptr, nullptr, nullptr, nullptr, alloc_size);
}

dtfft_error_t dtfft_get_element_size(dtfft_plan_t plan, size_t* es) {
    if (!es) return DTFFT_ERROR_INVALID_USAGE;
    Plan* p = as_plan(plan); if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    *es = p->element_size(); return DTFFT_SUCCESS;
}

dtfft_error_t dtfft_get_alloc_bytes(dtfft_plan_t plan, size_t* b) {
    if (!b) return DTFFT_ERROR_INVALID_USAGE;
    Plan* p = as_plan(plan); if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    *b = p->alloc_bytes(); return DTFFT_SUCCESS;
}

// aux = transposes' workspace (none: the fused move needs no staging) + one buffer
// (src/dtfft_plan.F90:1398-1420)
dtfft_error_t dtfft_get_aux_bytes(dtfft_plan_t plan, size_t* b) {
    if (!b) return DTFFT_ERROR_INVALID_USAGE;
    Plan* p = as_plan(plan); if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    *b = p->alloc_bytes(); return DTFFT_SUCCESS;
}

dtfft_error_t dtfft_get_aux_size(dtfft_plan_t plan, size_t* s) {
    if (!s) return DTFFT_ERROR_INVALID_USAGE;
    Plan* p = as_plan(plan); if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    *s = p->alloc_bytes() / p->element_size(); return DTFFT_SUCCESS;
}

dtfft_error_t dtfft_get_aux_bytes_transpose(dtfft_plan_t plan, size_t* b) {
    if (!b) return DTFFT_ERROR_INVALID_USAGE;
    Plan* p = as_plan(plan); if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    *b = 0; return DTFFT_SUCCESS;
}

dtfft_error_t dtfft_get_aux_size_transpose(dtfft_plan_t plan, size_t* s) {
    if (!s) return DTFFT_ERROR_INVALID_USAGE;
    Plan* p = as_plan(plan); if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    *s = 0; return DTFFT_SUCCESS;
}

// A reshape is one copy kernel from `in` to `out`: no workspace
// (src/dtfft_plan.F90:1436-1451 reports the exchange backend's).
dtfft_error_t dtfft_get_aux_bytes_reshape(dtfft_plan_t plan, size_t* b) {
    if (!b) return DTFFT_ERROR_INVALID_USAGE;
    Plan* p = as_plan(plan); if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    if (!p->reshape) return DTFFT_ERROR_RESHAPE_NOT_SUPPORTED;
    *b = 0; return DTFFT_SUCCESS;
}

dtfft_error_t dtfft_get_aux_size_reshape(dtfft_plan_t plan, size_t* s) {
    if (!s) return DTFFT_ERROR_INVALID_USAGE;
    Plan* p = as_plan(plan); if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    if (!p->reshape) return DTFFT_ERROR_RESHAPE_NOT_SUPPORTED;
    *s = 0; return DTFFT_SUCCESS;
}

dtfft_error_t dtfft_get_pencil(dtfft_plan_t plan, dtfft_layout_t layout, dtfft_pencil_t* pencil) {
    if (!pencil) return DTFFT_ERROR_INVALID_USAGE;
    Plan* p = as_plan(plan); if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    if (layout < DTFFT_LAYOUT_X_BRICKS || layout > DTFFT_LAYOUT_Z_BRICKS) return DTFFT_ERROR_INVALID_LAYOUT;
    const Layout* L = nullptr;
    switch (layout) {
    case DTFFT_LAYOUT_X_BRICKS: if (p->reshape) L = &p->brick_x; break;
    case DTFFT_LAYOUT_X_PENCILS: L = p->kind == K_R2C ? &p->real_x : &p->pen[0]; break;
    case DTFFT_LAYOUT_X_PENCILS_FOURIER: if (p->kind == K_R2C) L = &p->pen[0]; break;
    case DTFFT_LAYOUT_Y_PENCILS: L = &p->pen[1]; break;
    case DTFFT_LAYOUT_Z_PENCILS: if (p->ndims == 3) L = &p->pen[2]; break;
    case DTFFT_LAYOUT_Z_BRICKS: if (p->reshape) L = &p->brick_z; break;
    default: break;
    }
    if (!L) return DTFFT_ERROR_INVALID_LAYOUT;
    memset(pencil, 0, sizeof(*pencil));
    pencil->dim = (uint8_t)L->id;
    pencil->ndims = (uint8_t)p->ndims;
    box_of(*p, *L, pencil->starts, pencil->counts);
    size_t sz = 1;
    for (int d = 0; d < p->ndims; ++d) sz *= (size_t)pencil->counts[d];
    pencil->size = sz;
    return DTFFT_SUCCESS;
}

dtfft_error_t dtfft_vgrid_get_nranks(dtfft_plan_t plan, int32_t* n) {
    if (!n) return DTFFT_ERROR_INVALID_USAGE;
    Plan* p = as_plan(plan); if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    *n = p->P; return DTFFT_SUCCESS;
}

dtfft_error_t dtfft_vgrid_get_pencil(dtfft_plan_t plan, dtfft_layout_t layout, int32_t vrank, dtfft_pencil_t* pencil,
                                     size_t* offset) {
    if (!pencil && !offset) return DTFFT_ERROR_INVALID_USAGE;
    Plan* p = as_plan(plan); if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    if (vrank < 0 || vrank >= p->P) return DTFFT_ERROR_INVALID_USAGE;
    const Layout* L = nullptr;
    switch (layout) {
    case DTFFT_LAYOUT_X_BRICKS: if (p->reshape) L = &p->brick_x; break;
    case DTFFT_LAYOUT_X_PENCILS: L = p->kind == K_R2C ? &p->real_x : &p->pen[0]; break;
    case DTFFT_LAYOUT_X_PENCILS_FOURIER: if (p->kind == K_R2C) L = &p->pen[0]; break;
    case DTFFT_LAYOUT_Y_PENCILS: L = &p->pen[1]; break;
    case DTFFT_LAYOUT_Z_PENCILS: if (p->ndims == 3) L = &p->pen[2]; break;
    case DTFFT_LAYOUT_Z_BRICKS: if (p->reshape) L = &p->brick_z; break;
    default: break;
    }
    if (!L) return DTFFT_ERROR_INVALID_LAYOUT;
    if (pencil) {
        memset(pencil, 0, sizeof(*pencil));
        pencil->dim = (uint8_t)L->id;
        pencil->ndims = (uint8_t)p->ndims;
        size_t sz = 1;
        for (int d = 0; d < p->ndims; ++d) {
            pencil->starts[d] = L->r[vrank].start[d];
            pencil->counts[d] = L->r[vrank].count[d];
            sz *= (size_t)L->r[vrank].count[d];
        }
        pencil->size = sz;
    }
    if (offset) *offset = (size_t)L->off[vrank];
    return DTFFT_SUCCESS;
}

dtfft_error_t dtfft_mem_alloc(dtfft_plan_t plan, size_t alloc_bytes, void** ptr) {
    if (!ptr) return DTFFT_ERROR_INVALID_USAGE;
    Plan* p = as_plan(plan); if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    if (alloc_bytes < 4) return DTFFT_ERROR_INVALID_ALLOC_BYTES;
    if (cudaMalloc(ptr, alloc_bytes) != cudaSuccess) { cudaGetLastError(); *ptr = nullptr; return DTFFT_ERROR_ALLOC_FAILED; }
    return DTFFT_SUCCESS;
}

dtfft_error_t dtfft_mem_free(dtfft_plan_t plan, void* ptr) {
    Plan* p = as_plan(plan); if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    if (cudaFree(ptr) != cudaSuccess) { cudaGetLastError(); return DTFFT_ERROR_FREE_FAILED; }
    return DTFFT_SUCCESS;
}

dtfft_error_t dtfft_report(dtfft_plan_t plan) {
    Plan* p = as_plan(plan); if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    static const char* kn[] = {"C2C", "R2C", "R2R"};
    printf("**Plan report**\n  %dD %s, %s precision, executor %s\n", p->ndims, kn[p->kind],
           dtfft_get_precision_string(p->precision), dtfft_get_executor_string(p->executor));
    printf("  global dims:");
    for (int d = 0; d < p->ndims; ++d) printf(" %d", p->dims[d]);
    printf("\n  grid: 1x%dx%d (%d virtual ranks)%s%s\n", p->grid[1], p->ndims == 3 ? p->grid[2] : 1, p->P,
           p->z_slab ? ", Z-slab" : "", p->y_slab ? ", Y-slab" : "");
    for (int t = -3; t <= 3; ++t) {
        const BoxList& b = p->tr[t + 3];
        if (b.host.empty()) continue;
        printf("  transpose %+d: %zu boxes, tile %dx%d rows %d\n", t, b.host.size(), b.cfg.tile_a, b.cfg.tile_b, b.cfg.rows);
    }
    for (int d = 0; d < 3; ++d)
        if (p->fft[d]) printf("  fft dim %d: rank %d, n=%d x %d, batch %lld\n", d + 1, p->fft[d]->desc().rank,
                              p->fft[d]->desc().n_fast, p->fft[d]->desc().n_slow, (long long)p->fft[d]->desc().batch);
    printf("  alloc size: %zu elements of %zu bytes\n", (size_t)p->alloc_size(), p->element_size());
    return DTFFT_SUCCESS;
}

dtfft_error_t dtfft_get_executor(dtfft_plan_t plan, dtfft_executor_t* e) {
    if (!e) return DTFFT_ERROR_INVALID_USAGE;
    Plan* p = as_plan(plan); if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    *e = p->executor; return DTFFT_SUCCESS;
}

dtfft_error_t dtfft_get_precision(dtfft_plan_t plan, dtfft_precision_t* pr) {
    if (!pr) return DTFFT_ERROR_INVALID_USAGE;
    Plan* p = as_plan(plan); if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    *pr = p->precision; return DTFFT_SUCCESS;
}

dtfft_error_t dtfft_get_dims(dtfft_plan_t plan, int8_t* ndims, const int32_t* dims[]) {
    if (!ndims && !dims) return DTFFT_ERROR_INVALID_USAGE;
    Plan* p = as_plan(plan); if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    if (ndims) *ndims = (int8_t)p->ndims;
    if (dims) *dims = p->out_dims;
    return DTFFT_SUCCESS;
}

dtfft_error_t dtfft_get_grid_dims(dtfft_plan_t plan, int8_t* ndims, const int32_t* grid_dims[]) {
    if (!ndims && !grid_dims) return DTFFT_ERROR_INVALID_USAGE;
    Plan* p = as_plan(plan); if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    if (ndims) *ndims = (int8_t)p->ndims;
    if (grid_dims) *grid_dims = p->out_grid;
    return DTFFT_SUCCESS;
}

dtfft_error_t dtfft_get_stream(dtfft_plan_t plan, dtfft_stream_t* s) {
    if (!s) return DTFFT_ERROR_INVALID_USAGE;
    Plan* p = as_plan(plan); if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    *s = (dtfft_stream_t)p->stream; return DTFFT_SUCCESS;
}

dtfft_error_t dtfft_get_platform(dtfft_plan_t plan, dtfft_platform_t* pl) {
    if (!pl) return DTFFT_ERROR_INVALID_USAGE;
    Plan* p = as_plan(plan); if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    *pl = DTFFT_PLATFORM_CUDA; return DTFFT_SUCCESS;
}

// One GPU: no exchange backend is ever used (src/dtfft_transpose_plan.F90:220).
dtfft_error_t dtfft_get_backend(dtfft_plan_t plan, dtfft_backend_t* b) {
    if (!b) return DTFFT_ERROR_INVALID_USAGE;
    Plan* p = as_plan(plan); if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    *b = DTFFT_BACKEND_NONE; return DTFFT_SUCCESS;
}

dtfft_error_t dtfft_get_reshape_backend(dtfft_plan_t plan, dtfft_backend_t* b) {
    if (!b) return DTFFT_ERROR_INVALID_USAGE;
    Plan* p = as_plan(plan); if (!p) return DTFFT_ERROR_PLAN_NOT_CREATED;
    *b = DTFFT_BACKEND_NONE; return DTFFT_SUCCESS;
}

}  // extern "C"

// ===========================================================================
// Batches: many plans executed as one CUDA graph.  The reference has no
// batching API; a caller of it runs one dtfft_execute per plan.  Here every
// plan's schedule is captured once on its own branch of a graph (plans spread
// over `lanes` streams, so the kernels of small transforms run side by side)
// and later calls replay the graph with one launch.
// ===========================================================================
namespace gb {

static const uint32_t kBatchMagic = 0x47424254u;   // "GBBT"

// One captured schedule: the graph of every plan's execute for one set of
// buffers and one direction.
struct BatchGraph {
    std::vector<const void*> key;   // type, then in/out/aux of every plan
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    size_t nodes = 0;
    uint64_t used = 0;
    void drop() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr; graph = nullptr; nodes = 0;
    }
};

struct Batch {
    static const int kMaxGraphs = 4;   // e.g. forward and backward over two buffer sets
    uint32_t magic = kBatchMagic;
    std::vector<Plan*> plans;
    std::vector<cudaStream_t> lanes;
    cudaStream_t cap = nullptr;
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> joins;
    std::vector<BatchGraph> graphs;
    uint64_t tick = 0;
    size_t last_nodes = 0;
    ~Batch() {
        for (auto& g : graphs) g.drop();
        for (auto l : lanes) cudaStreamDestroy(l);
        for (auto e : joins) cudaEventDestroy(e);
        if (fork) cudaEventDestroy(fork);
        if (cap) cudaStreamDestroy(cap);
        magic = 0;
    }
};

static Batch* as_batch(dtfft_gb_batch_t b) {
    Batch* q = reinterpret_cast<Batch*>(b);
    if (!q || q->magic != kBatchMagic) return nullptr;
    return q;
}

static dtfft_error_t capture_batch(Batch& b, BatchGraph& bg, void* const* ins, void* const* outs, void* const* auxs,
                                   bool fwd) {
    const int n = (int)b.plans.size(), K = (int)b.lanes.size();
    GB_CUDA_TRY(cudaStreamBeginCapture(b.cap, cudaStreamCaptureModeThreadLocal));
    dtfft_error_t e = DTFFT_SUCCESS;
    if (cudaEventRecord(b.fork, b.cap) != cudaSuccess) e = DTFFT_ERROR_GPU_CALL_FAILED;
    for (int l = 0; l < K && e == DTFFT_SUCCESS; ++l)
        if (cudaStreamWaitEvent(b.lanes[l], b.fork, 0) != cudaSuccess) e = DTFFT_ERROR_GPU_CALL_FAILED;
    for (int i = 0; i < n && e == DTFFT_SUCCESS; ++i) {
        Plan& p = *b.plans[i];
        cudaStream_t saved = p.stream;
        p.stream = b.lanes[i % K];
        e = run_execute(p, ins[i], outs[i], fwd, auxs[i], ins[i] == outs[i]);
        p.stream = saved;
    }
    for (int l = 0; l < K && e == DTFFT_SUCCESS; ++l) {
        if (cudaEventRecord(b.joins[l], b.lanes[l]) != cudaSuccess ||
            cudaStreamWaitEvent(b.cap, b.joins[l], 0) != cudaSuccess)
            e = DTFFT_ERROR_GPU_CALL_FAILED;
    }
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(b.cap, &g);
    if (e == DTFFT_SUCCESS && ce != cudaSuccess) e = DTFFT_ERROR_GPU_CALL_FAILED;
    if (e == DTFFT_SUCCESS && cudaGraphInstantiate(&bg.exec, g, 0) != cudaSuccess) e = DTFFT_ERROR_GPU_CALL_FAILED;
    if (e != DTFFT_SUCCESS) {
        if (g) cudaGraphDestroy(g);
        bg.exec = nullptr;
        cudaGetLastError();
        return e;
    }
    bg.graph = g;
    cudaGraphGetNodes(g, nullptr, &bg.nodes);
    return DTFFT_SUCCESS;
}

}  // namespace gb

extern "C" {

dtfft_error_t dtfft_gb_batch_create(int32_t n, const dtfft_plan_t* plans, int32_t lanes, dtfft_gb_batch_t* batch) {
    if (!plans || !batch || n < 1) return DTFFT_ERROR_INVALID_USAGE;
    *batch = nullptr;
    Batch* b = new Batch();
    for (int i = 0; i < n; ++i) {
        Plan* p = as_plan(plans[i]);
        if (!p) { delete b; return DTFFT_ERROR_PLAN_NOT_CREATED; }
        b->plans.push_back(p);
    }
    const int K = std::max(1, std::min<int>(lanes > 0 ? lanes : 8, n));
    bool ok = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) == cudaSuccess;
    for (int l = 0; l < K && ok; ++l) {
        cudaStream_t s = nullptr;
        cudaEvent_t e = nullptr;
        ok = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess &&
             cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
        if (s) b->lanes.push_back(s);
        if (e) b->joins.push_back(e);
    }
    if (!ok) { cudaGetLastError(); delete b; return DTFFT_ERROR_GPU_CALL_FAILED; }
    *batch = reinterpret_cast<dtfft_gb_batch_t>(b);
    return DTFFT_SUCCESS;
}

dtfft_error_t dtfft_gb_batch_execute(dtfft_gb_batch_t batch, void* const* ins, void* const* outs, void* const* auxs,
                                     dtfft_execute_t execute_type, void* stream) {
    TraceRange tr("dtfft_gb_batch_execute");
    Batch* b = as_batch(batch);
    if (!b) return DTFFT_ERROR_INVALID_USAGE;
    if (!ins || !outs) return DTFFT_ERROR_INVALID_USAGE;
    GB_TRY(check_device_status());
    const int n = (int)b->plans.size();
    std::vector<const void*> key;
    key.reserve(3 * n + 1);
    key.push_back((const void*)(intptr_t)execute_type);
    for (int i = 0; i < n; ++i) {
        key.push_back(ins[i]);
        key.push_back(outs[i]);
        key.push_back(auxs ? auxs[i] : nullptr);
    }
    BatchGraph* hit = nullptr;
    for (auto& g : b->graphs) if (g.exec && g.key == key) hit = &g;
    if (!hit) {
        // new buffers: check them like dtfft_execute, make the plans' aux
        // buffers now (outside the capture) and capture the schedules; the
        // least recently used graph makes room
        std::vector<void*> a(n);
        for (int i = 0; i < n; ++i) {
            void* ua = auxs ? auxs[i] : nullptr;
            GB_TRY(execute_checks(b->plans[i], ins[i], outs[i], (int)execute_type, ua));
            GB_TRY(get_aux(*b->plans[i], ua, &a[i]));
        }
        if ((int)b->graphs.size() >= Batch::kMaxGraphs) {
            auto lru = std::min_element(b->graphs.begin(), b->graphs.end(),
                                        [](const BatchGraph& x, const BatchGraph& y) { return x.used < y.used; });
            cudaStreamSynchronize((cudaStream_t)stream);
            lru->drop();
            b->graphs.erase(lru);
        }
        BatchGraph bg;
        GB_TRY(capture_batch(*b, bg, ins, outs, a.data(), execute_type == DTFFT_EXECUTE_FORWARD));
        bg.key = key;
        b->graphs.push_back(bg);
        hit = &b->graphs.back();
    }
    hit->used = ++b->tick;
    b->last_nodes = hit->nodes;
    GB_CUDA_TRY(cudaGraphLaunch(hit->exec, (cudaStream_t)stream));
    return DTFFT_SUCCESS;
}

dtfft_error_t dtfft_gb_batch_graph_nodes(dtfft_gb_batch_t batch, int64_t* nodes) {
    Batch* b = as_batch(batch);
    if (!b || !nodes) return DTFFT_ERROR_INVALID_USAGE;
    *nodes = (int64_t)b->last_nodes;
    return DTFFT_SUCCESS;
}

dtfft_error_t dtfft_gb_batch_destroy(dtfft_gb_batch_t* batch) {
    if (!batch) return DTFFT_ERROR_INVALID_USAGE;
    Batch* b = as_batch(*batch);
    if (!b) return DTFFT_ERROR_INVALID_USAGE;
    cudaDeviceSynchronize();
    delete b;
    *batch = nullptr;
    return DTFFT_SUCCESS;
}

}  // extern "C"
