// Kernel and FFT-executor plug-ins: the two seams where the reference's
// Fortran plan code calls device code (abstract_kernel, abstract_executor).
// A Fortran build binds these with iso_c_binding in place of kernel_device
// (src/dtfft_kernel_device.F90) and the cuFFT / VkFFT executors
// (src/interfaces/fft/cufft/dtfft_executor_cufft_m.F90,
//  src/interfaces/fft/vkfft/dtfft_executor_vkfft_m.F90).
//
// Every local move kernel of the reference is a set of strided boxes, so each
// kernel type maps onto the same box-list launch used by the plans:
//   PERMUTE_FORWARD        (nx,ny,nz) -> (ny,nz,nx)      one transpose box
//   PERMUTE_BACKWARD       (nx,ny,nz) -> (nz,nx,ny)      one transpose box
//   PERMUTE_BACKWARD_START (nx,ny,nz) -> (nz,ny,nx)      one transpose box
//   PERMUTE_BACKWARD_END   per-neighbour (x,z,y) -> (x,y,z) copy boxes
//   PACK / UNPACK          per-neighbour sub-box copies
//   COPY                   one contiguous copy
// (index maps: src/include/_dtfft_kernel_host_routines.inc:140-752)
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "plan.h"

namespace gb {

struct KernelObj {
    uint32_t magic = 0x4b45524eu;
    int type = 0;
    int ndims = 3;
    int dims[3] = {1, 1, 1};
    int elem = 8;
    BoxList all;                    // every neighbour / the whole permute
    std::vector<BoxList> per;       // one list per neighbour (pipelined kinds)
    std::vector<int> nbr;           // 5 x n neighbour data
    ~KernelObj() {
        boxes_free(all);
        for (auto& b : per) boxes_free(b);
    }
};

struct FftObj {
    uint32_t magic = 0x46465450u;
    FftPlan* plan = nullptr;
    cudaStream_t stream = nullptr;
    ~FftObj() { delete plan; }
};

static Box transpose_box(i64 na, i64 nb, i64 nc, i64 sb, i64 sc, i64 da, i64 dc) {
    Box b;
    memset(&b, 0, sizeof(b));
    b.na = (int32_t)na; b.nb = (int32_t)nb; b.nc = (int32_t)nc;
    b.sb = sb; b.sc = sc; b.da_or_db = da; b.dc = dc;
    return b;
}

// Neighbour box of UNPACK / PACK / PERMUTE_BACKWARD_END as a copy box.
static Box neighbour_box(int type, int ndims, const int* dims, const int* nb) {
    const i64 nx = dims[0], ny = dims[1];
    const i64 nxx = nb[0], nyy = nb[1], nzz = ndims == 2 ? 1 : nb[2], din = nb[3], dout = nb[4];
    Box b;
    memset(&b, 0, sizeof(b));
    b.src_off = din;
    b.dst_off = dout;
    b.na = (int32_t)nxx;
    if (type == GB_KERNEL_UNPACK || type == GB_KERNEL_UNPACK_PIPELINED) {
        // out[dout + z*nx*ny + y*nx + x] = in[din + z*nxx*nyy + y*nxx + x]
        b.nb = (int32_t)nyy; b.nc = (int32_t)nzz;
        b.sb = nxx; b.sc = nxx * nyy; b.da_or_db = nx; b.dc = nx * ny;
    } else if (type == GB_KERNEL_PACK || type == GB_KERNEL_PACK_PIPELINED) {
        // out[dout + z*nxx*nyy + y*nxx + x] = in[din + z*nx*ny + y*nx + x]
        b.nb = (int32_t)nyy; b.nc = (int32_t)nzz;
        b.sb = nx; b.sc = nx * ny; b.da_or_db = nxx; b.dc = nxx * nyy;
    } else {
        // PERMUTE_BACKWARD_END: out[dout + z*nx*ny + y*nx + x] = in[din + z*nxx + y*nzz*nxx + x]
        b.nb = (int32_t)nzz; b.nc = (int32_t)nyy;
        b.sb = nxx; b.sc = nzz * nxx; b.da_or_db = nx * ny; b.dc = nx;
    }
    return b;
}

}  // namespace gb

using namespace gb;

extern "C" {

dtfft_error_t gb_kernel_create(int32_t ndims, const int32_t* dims, int32_t base_storage, int32_t kernel_type,
                               const int32_t* neighbor_data, int32_t n_neighbors, int32_t effort,
                               gb_kernel_t* kernel) {
    if (!kernel || !dims) return DTFFT_ERROR_INVALID_USAGE;
    *kernel = nullptr;
    if (ndims != 2 && ndims != 3) return DTFFT_ERROR_INVALID_N_DIMENSIONS;
    if (base_storage != 4 && base_storage != 8 && base_storage != 16) return DTFFT_ERROR_INVALID_USAGE;
    GB_TRY(status_setup());
    KernelObj* k = new KernelObj();
    k->type = kernel_type;
    k->ndims = ndims;
    k->elem = base_storage;
    for (int i = 0; i < ndims; ++i) k->dims[i] = dims[i];
    // 2D backward kinds alias the forward permute (src/dtfft_abstract_kernel.F90:272-282)
    if (ndims == 2 && kernel_type == GB_KERNEL_PERMUTE_BACKWARD) k->type = GB_KERNEL_PERMUTE_FORWARD;
    const i64 nx = dims[0], ny = dims[1], nz = ndims == 3 ? dims[2] : 1;
    bool any_zero = false;
    for (int i = 0; i < ndims; ++i) if (dims[i] <= 0) any_zero = true;
    k->all.elem = base_storage;
    k->all.cfg = default_tile(base_storage);
    const bool needs_nbr = k->type == GB_KERNEL_PACK || k->type == GB_KERNEL_UNPACK ||
                           k->type == GB_KERNEL_PACK_PIPELINED || k->type == GB_KERNEL_UNPACK_PIPELINED ||
                           k->type == GB_KERNEL_PERMUTE_BACKWARD_END ||
                           k->type == GB_KERNEL_PERMUTE_BACKWARD_END_PIPELINED || k->type == GB_KERNEL_COPY_PIPELINED;
    if (needs_nbr && (!neighbor_data || n_neighbors < 1)) { delete k; return DTFFT_ERROR_INVALID_USAGE; }
    if (needs_nbr) k->nbr.assign(neighbor_data, neighbor_data + 5 * n_neighbors);
    dtfft_error_t e = DTFFT_SUCCESS;
    if (any_zero || k->type == GB_KERNEL_DUMMY) {
        k->type = GB_KERNEL_DUMMY;  // empty local data (src/dtfft_abstract_kernel.F90:241-245)
    } else {
        switch (k->type) {
        case GB_KERNEL_PERMUTE_FORWARD:
            k->all.copy = false;
            if (ndims == 2) k->all.host.push_back(transpose_box(nx, ny, 1, nx, 0, ny, 0));
            else k->all.host.push_back(transpose_box(nx, ny, nz, nx, nx * ny, ny * nz, ny));
            break;
        case GB_KERNEL_PERMUTE_BACKWARD:
            k->all.copy = false;
            k->all.host.push_back(transpose_box(nx, nz, ny, nx * ny, nx, nz, nz * nx));
            break;
        case GB_KERNEL_PERMUTE_BACKWARD_START:
            if (ndims != 3) { e = DTFFT_ERROR_INVALID_USAGE; break; }
            k->all.copy = false;
            k->all.host.push_back(transpose_box(nx, nz, ny, nx * ny, nx, nz * ny, nz));
            break;
        case GB_KERNEL_COPY:
            break;
        case GB_KERNEL_PACK: case GB_KERNEL_UNPACK: case GB_KERNEL_PERMUTE_BACKWARD_END:
        case GB_KERNEL_PACK_PIPELINED: case GB_KERNEL_UNPACK_PIPELINED:
        case GB_KERNEL_PERMUTE_BACKWARD_END_PIPELINED: {
            int base = k->type;
            if (base == GB_KERNEL_PERMUTE_BACKWARD_END_PIPELINED) base = GB_KERNEL_PERMUTE_BACKWARD_END;
            k->all.copy = true;
            for (int i = 0; i < n_neighbors; ++i) {
                Box b = neighbour_box(base, ndims, dims, &k->nbr[5 * i]);
                k->all.host.push_back(b);
                BoxList one;
                one.elem = base_storage;
                one.copy = true;
                one.cfg = k->all.cfg;
                one.host.push_back(b);
                k->per.push_back(one);
            }
        } break;
        case GB_KERNEL_COPY_PIPELINED:
            break;
        default:
            e = DTFFT_ERROR_INVALID_USAGE;
        }
    }
    if (e == DTFFT_SUCCESS && !k->all.host.empty()) {
        if (!k->all.copy) tma_default_tile(k->all);
        e = boxes_upload(k->all);
        for (auto& b : k->per) if (e == DTFFT_SUCCESS) e = boxes_upload(b);
        if (e == DTFFT_SUCCESS && effort == DTFFT_EXHAUSTIVE) {
            i64 n = nx * ny * nz;
            for (int i = 0; i < (int)k->nbr.size() / 5; ++i) n = std::max<i64>(n, (i64)k->nbr[5 * i + 3] + (i64)k->nbr[5 * i] * k->nbr[5 * i + 1] * k->nbr[5 * i + 2]);
            e = autotune_boxes(k->all, n, nullptr, 2, 5, false);
        }
    }
    if (e != DTFFT_SUCCESS) { delete k; return e; }
    *kernel = reinterpret_cast<gb_kernel_t>(k);
    return DTFFT_SUCCESS;
}

dtfft_error_t gb_kernel_execute(gb_kernel_t kernel, const void* in, void* out, void* stream, int32_t neighbor) {
    KernelObj* k = reinterpret_cast<KernelObj*>(kernel);
    if (!k || k->magic != 0x4b45524eu) return DTFFT_ERROR_INVALID_USAGE;
    if (k->type == GB_KERNEL_DUMMY) return DTFFT_SUCCESS;
    GB_TRY(check_device_status());
    cudaStream_t s = (cudaStream_t)stream;
    if (k->type == GB_KERNEL_COPY) {
        size_t n = (size_t)k->dims[0] * k->dims[1] * (k->ndims == 3 ? k->dims[2] : 1);
        GB_CUDA_TRY(cudaMemcpyAsync(out, in, n * k->elem, cudaMemcpyDeviceToDevice, s));
        return DTFFT_SUCCESS;
    }
    if (k->type == GB_KERNEL_COPY_PIPELINED) {
        if (neighbor < 1 || neighbor > (int)k->nbr.size() / 5) return DTFFT_ERROR_INVALID_USAGE;
        const int* nb = &k->nbr[5 * (neighbor - 1)];
        size_t n = (size_t)nb[0] * nb[1] * nb[2];
        GB_CUDA_TRY(cudaMemcpyAsync((char*)out + (size_t)nb[4] * k->elem, (const char*)in + (size_t)nb[3] * k->elem,
                                    n * k->elem, cudaMemcpyDeviceToDevice, s));
        return DTFFT_SUCCESS;
    }
    const bool pipelined = k->type == GB_KERNEL_PACK_PIPELINED || k->type == GB_KERNEL_UNPACK_PIPELINED ||
                           k->type == GB_KERNEL_PERMUTE_BACKWARD_END_PIPELINED;
    if (pipelined) {
        if (neighbor < 1 || neighbor > (int)k->per.size()) return DTFFT_ERROR_INVALID_USAGE;
        return boxes_launch(k->per[neighbor - 1], in, out, s);
    }
    return boxes_launch(k->all, in, out, s);
}

dtfft_error_t gb_kernel_destroy(gb_kernel_t* kernel) {
    if (!kernel) return DTFFT_ERROR_INVALID_USAGE;
    KernelObj* k = reinterpret_cast<KernelObj*>(*kernel);
    if (!k || k->magic != 0x4b45524eu) return DTFFT_ERROR_INVALID_USAGE;
    k->magic = 0;
    delete k;
    *kernel = nullptr;
    return DTFFT_SUCCESS;
}

dtfft_error_t gb_fft_create(int32_t fft_rank, int32_t fft_type, int32_t precision, int32_t idist, int32_t odist,
                            int32_t how_many, const int32_t* fft_sizes, const int32_t* inembed,
                            const int32_t* onembed, const int32_t* r2r_kinds, void* stream, gb_fft_t* fft) {
    (void)inembed; (void)onembed;
    if (!fft || !fft_sizes) return DTFFT_ERROR_INVALID_USAGE;
    *fft = nullptr;
    if (fft_rank != 1 && fft_rank != 2) return DTFFT_ERROR_INVALID_USAGE;
    if (precision != DTFFT_SINGLE && precision != DTFFT_DOUBLE) return DTFFT_ERROR_INVALID_PRECISION;
    GB_TRY(status_setup());
    FftDesc d;
    d.dbl = precision == DTFFT_DOUBLE;
    d.rank = fft_rank;
    // FFTW order: fft_sizes[0] is the slowest dim
    d.n_fast = fft_sizes[fft_rank - 1];
    d.n_slow = fft_rank == 2 ? fft_sizes[0] : 1;
    d.batch = how_many;
    d.idist = idist;
    d.odist = odist;
    switch (fft_type) {
    case GB_FFT_C2C: d.type = FFT_C2C; break;
    case GB_FFT_R2C: d.type = FFT_R2C; break;
    case GB_FFT_R2R:
        if (!r2r_kinds) return DTFFT_ERROR_MISSING_R2R_KINDS;
        d.type = FFT_R2R;
        d.kind_fast = r2r_kinds[fft_rank - 1];
        d.kind_slow = fft_rank == 2 ? r2r_kinds[0] : 0;
        break;
    default: return DTFFT_ERROR_INVALID_USAGE;
    }
    FftObj* o = new FftObj();
    o->stream = (cudaStream_t)stream;
    dtfft_error_t e = FftPlan::create(d, &o->plan);
    if (e != DTFFT_SUCCESS) { delete o; return e; }
    *fft = reinterpret_cast<gb_fft_t>(o);
    return DTFFT_SUCCESS;
}

dtfft_error_t gb_fft_execute(gb_fft_t fft, void* a, void* b, int32_t sign) {
    FftObj* o = reinterpret_cast<FftObj*>(fft);
    if (!o || o->magic != 0x46465450u) return DTFFT_ERROR_INVALID_USAGE;
    if (sign != GB_FFT_FORWARD && sign != GB_FFT_BACKWARD) return DTFFT_ERROR_INVALID_USAGE;
    GB_TRY(check_device_status());
    return o->plan->execute(a, b, sign, o->stream);
}

dtfft_error_t gb_fft_destroy(gb_fft_t* fft) {
    if (!fft) return DTFFT_ERROR_INVALID_USAGE;
    FftObj* o = reinterpret_cast<FftObj*>(*fft);
    if (!o || o->magic != 0x46465450u) return DTFFT_ERROR_INVALID_USAGE;
    o->magic = 0;
    delete o;
    *fft = nullptr;
    return DTFFT_SUCCESS;
}

}  // extern "C"
