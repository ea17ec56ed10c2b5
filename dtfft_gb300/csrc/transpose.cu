// Box-list transpose and copy kernels.
//
// One launch moves every (source rank -> destination rank) block of a virtual
// grid transpose: the reference's pack kernel, exchange and unpack kernel
// (src/dtfft_reshape_handle_generic.F90:695-759 with the NVRTC kernels of
// src/dtfft_nvrtc_module.F90:434-583) collapse into one pass over HBM that
// reads each element once and writes it once at its final position.
//
// Tiles: a CTA owns one TA x TB tile of one c-plane of one box.  It reads TB
// source rows of TA contiguous elements, stages them in padded shared memory
// (conflict-free for 4/8/16-byte elements) and writes TA destination rows of TB
// contiguous elements.  Every global access of a warp is one contiguous run.
#include <algorithm>
#include <cstdio>

#include "common.cuh"

namespace gb {

std::atomic<int64_t> g_launches{0};

__device__ __forceinline__ int find_box(const Box* __restrict__ boxes, int nboxes, i64 t) {
    int lo = 0, hi = nboxes - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (boxes[mid].tile_begin <= t) lo = mid; else hi = mid - 1;
    }
    return lo;
}

template <typename T, int TA, int TB, int ROWS>
__global__ void __launch_bounds__(32 * ROWS)
box_transpose_kernel(const T* __restrict__ in, T* __restrict__ out,
                     const Box* __restrict__ boxes, int nboxes) {
    __shared__ T tile[TB][TA + 1];
    const i64 t = (i64)blockIdx.x;
    const int bi = nboxes > 1 ? find_box(boxes, nboxes, t) : 0;
    const Box* bp = boxes + bi;
    const int tiles_a = __ldg(&bp->tiles_a);
    const int per_c = tiles_a * __ldg(&bp->tiles_b);
    const i64 lt = t - __ldg(&bp->tile_begin);
    const int c = (int)(lt / per_c);
    const int r = (int)(lt - (i64)c * per_c);
    const int a0 = (r % tiles_a) * TA;
    const int b0 = (r / tiles_a) * TB;
    const int tx = threadIdx.x, ty = threadIdx.y;
    // in-tile extents; offsets inside a box fit 32 bits (checked when the list is built)
    const int ra = min(TA, __ldg(&bp->na) - a0), rb = min(TB, __ldg(&bp->nb) - b0);
    const int sb = (int)__ldg(&bp->sb), da = (int)__ldg(&bp->da_or_db);
    const T* src = in + __ldg(&bp->src_off) + (i64)c * __ldg(&bp->sc) + a0 + (i64)b0 * sb;
    T* dst = out + __ldg(&bp->dst_off) + (i64)c * __ldg(&bp->dc) + b0 + (i64)a0 * da;
    if (ra == TA && rb == TB) {   // interior tile: no bounds checks
#pragma unroll
        for (int bb = ty; bb < TB; bb += ROWS)
#pragma unroll
            for (int aa = tx; aa < TA; aa += 32) tile[bb][aa] = src[aa + bb * sb];
        __syncthreads();
#pragma unroll
        for (int aa = ty; aa < TA; aa += ROWS)
#pragma unroll
            for (int bb = tx; bb < TB; bb += 32) dst[bb + aa * da] = tile[bb][aa];
        return;
    }
#pragma unroll
    for (int bb = ty; bb < TB; bb += ROWS)
#pragma unroll
        for (int aa = tx; aa < TA; aa += 32)
            if (aa < ra && bb < rb) tile[bb][aa] = src[aa + bb * sb];
    __syncthreads();
#pragma unroll
    for (int aa = ty; aa < TA; aa += ROWS)
#pragma unroll
        for (int bb = tx; bb < TB; bb += 32)
            if (aa < ra && bb < rb) dst[bb + aa * da] = tile[bb][aa];
}

// Copy boxes: the contiguous axis is the same on both sides, no staging.
template <typename T, int TA, int TB, int ROWS>
__global__ void __launch_bounds__(32 * ROWS)
box_copy_kernel(const T* __restrict__ in, T* __restrict__ out,
                const Box* __restrict__ boxes, int nboxes) {
    const i64 t = (i64)blockIdx.x;
    const int bi = nboxes > 1 ? find_box(boxes, nboxes, t) : 0;
    const Box& bx = boxes[bi];
    const i64 lt = t - bx.tile_begin;
    const int per_c = bx.tiles_a * bx.tiles_b;
    const int c = (int)(lt / per_c);
    const int r = (int)(lt - (i64)c * per_c);
    const int a0 = (r % bx.tiles_a) * TA;
    const int b0 = (r / bx.tiles_a) * TB;
    const T* src = in + bx.src_off + (i64)c * bx.sc;
    T* dst = out + bx.dst_off + (i64)c * bx.dc;
    for (int bb = threadIdx.y; bb < TB; bb += ROWS) {
        const int b = b0 + bb;
        if (b >= bx.nb) break;
        for (int aa = threadIdx.x; aa < TA; aa += 32) {
            const int a = a0 + aa;
            if (a < bx.na) dst[a + (i64)b * bx.da_or_db] = src[a + (i64)b * bx.sb];
        }
    }
}

dtfft_error_t boxes_upload(BoxList& bl) {
    boxes_free(bl);
    const int TA = bl.cfg.tile_a, TB = bl.cfg.tile_b;
    i64 tiles = 0;
    std::vector<Box> kept;
    for (Box b : bl.host) {
        if (b.na <= 0 || b.nb <= 0 || b.nc <= 0) continue;
        // in-tile offsets are 32-bit in the kernels
        if ((i64)(TB + 1) * b.sb >= 0x7fffffffLL || (i64)(TA + 1) * b.da_or_db >= 0x7fffffffLL)
            return DTFFT_ERROR_FFT_SIZE_NOT_SUPPORTED;
        b.tiles_a = (b.na + TA - 1) / TA;
        b.tiles_b = (b.nb + TB - 1) / TB;
        b.tile_begin = tiles;
        tiles += (i64)b.tiles_a * b.tiles_b * b.nc;
        kept.push_back(b);
    }
    bl.host.swap(kept);
    bl.total_tiles = tiles;
    GB_TRY(status_setup());
    if (bl.host.empty()) return DTFFT_SUCCESS;
    if (tiles > 0x7fffffffLL) return DTFFT_ERROR_FFT_SIZE_NOT_SUPPORTED;
    GB_CUDA_TRY(cudaMalloc((void**)&bl.dev, sizeof(Box) * bl.host.size()));
    GB_CUDA_TRY(cudaMemcpy(bl.dev, bl.host.data(), sizeof(Box) * bl.host.size(), cudaMemcpyHostToDevice));
    return DTFFT_SUCCESS;
}

void boxes_free(BoxList& bl) {
    if (bl.dev) cudaFree(bl.dev);
    bl.dev = nullptr;
    tma_cache_free(bl.tma_cache);
}

template <typename T, int TA, int TB, int ROWS>
static void launch_t(const BoxList& bl, const void* in, void* out, cudaStream_t s) {
    dim3 block(32, ROWS);
    const int nb = (int)bl.host.size();
    if (bl.copy)
        box_copy_kernel<T, TA, TB, ROWS><<<(unsigned)bl.total_tiles, block, 0, s>>>(
            (const T*)in, (T*)out, bl.dev, nb);
    else
        box_transpose_kernel<T, TA, TB, ROWS><<<(unsigned)bl.total_tiles, block, 0, s>>>(
            (const T*)in, (T*)out, bl.dev, nb);
}

template <typename T>
static bool launch_cfg(const BoxList& bl, const void* in, void* out, cudaStream_t s) {
    const TransposeConfig& c = bl.cfg;
#define GB_TILE(TA_, TB_, R_)                                              \
    if (c.tile_a == TA_ && c.tile_b == TB_ && c.rows == R_) {              \
        if constexpr (sizeof(T) * TB_ * (TA_ + 1) <= 48 * 1024) {          \
            launch_t<T, TA_, TB_, R_>(bl, in, out, s);                     \
            return true;                                                   \
        } else {                                                           \
            return false;                                                  \
        }                                                                  \
    }
    GB_TILE(32, 32, 8)
    GB_TILE(32, 32, 4)
    GB_TILE(64, 32, 8)
    GB_TILE(32, 64, 8)
    GB_TILE(64, 64, 8)
    GB_TILE(64, 64, 16)
#undef GB_TILE
    return false;
}

dtfft_error_t boxes_launch(const BoxList& bl, const void* in, void* out, cudaStream_t stream) {
    if (bl.total_tiles == 0) return DTFFT_SUCCESS;
    // TMA tensor loads when the list was tiled for the TMA kernel's extents
    // (a tensor map the driver refuses to encode leaves the list on the plain kernel)
    void* tok0 = nullptr;
    if (!bl.copy && bl.cfg.tile_a == tma_tile_a(bl.elem) && bl.cfg.tile_b == 32 && tma_eligible(bl) &&
        (tok0 = prof_begin(stream), tma_launch(bl, in, out, stream, gb_status_word(), bl.tma_cache)) == DTFFT_SUCCESS) {
        void* tok = tok0;
        if (tok)
            prof_end(tok, std::string("transpose_tma_e") + std::to_string(bl.elem) + "_t" + std::to_string(bl.cfg.tile_a) +
                              "x32", stream);
        count_launch();
        GB_CUDA_TRY(cudaGetLastError());
        return DTFFT_SUCCESS;
    }
    void* tok = prof_begin(stream);
    bool ok = false;
    switch (bl.elem) {
    case 4: ok = launch_cfg<uint32_t>(bl, in, out, stream); break;
    case 8: ok = launch_cfg<uint64_t>(bl, in, out, stream); break;
    case 16: ok = launch_cfg<e16>(bl, in, out, stream); break;
    default: return DTFFT_ERROR_INVALID_USAGE;
    }
    if (!ok) return DTFFT_ERROR_INVALID_USAGE;
    if (tok) {
        std::string nm = std::string(bl.copy ? "copy" : "transpose") + "_e" + std::to_string(bl.elem) + "_t" +
                         std::to_string(bl.cfg.tile_a) + "x" + std::to_string(bl.cfg.tile_b);
        prof_end(tok, nm, stream);
    }
    count_launch();
    GB_CUDA_TRY(cudaGetLastError());
    return DTFFT_SUCCESS;
}

}  // namespace gb
