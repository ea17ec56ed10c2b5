// Tile-kernel instantiations for double precision (complex128 rows).
#include "fft_tile.cuh"

namespace gb {

template <>
void* TilePtr<double>::get(int M, int sign, bool xpose, int ncw, int nsw) {
    // one warp split per kind: plain 8 warps, fused 4 compute + 4 store
    if (!xpose && ncw != 0 && ncw != 8) return nullptr;
    if (xpose && (ncw != 0 || nsw != 0) && !(ncw == 4 && nsw == 4)) return nullptr;
    if (!xpose) {
        switch (M) {
        case 256: return sign < 0 ? (void*)fft_tile_kernel<double, -1, 8, 8, 8, 8, 4> : (void*)fft_tile_kernel<double, 1, 8, 8, 8, 8, 4>;
        case 512: return sign < 0 ? (void*)fft_tile_kernel<double, -1, 8, 16, 16, 16, 2> : (void*)fft_tile_kernel<double, 1, 8, 16, 16, 16, 2>;
        }
        return nullptr;
    }
    switch (M) {
    case 256: return sign < 0 ? (void*)fft_tile_xpose_kernel<double, -1, 4, 4, 8, 8, 8, 4> : (void*)fft_tile_xpose_kernel<double, 1, 4, 4, 8, 8, 8, 4>;
    case 512: return sign < 0 ? (void*)fft_tile_xpose_kernel<double, -1, 4, 4, 16, 16, 16, 2> : (void*)fft_tile_xpose_kernel<double, 1, 4, 4, 16, 16, 16, 2>;
    }
    return nullptr;
}

// Fused passes with the tensor-store write-out: 4 compute warps (one row
// pair each of an 8-row tile, 128-byte lines) + 1 producer warp.
template <>
void* TilePtr<double>::get_tma(int M, int sign, int* rows, int* warps) {
    if (rows) *rows = 8;
    if (warps) *warps = 4;
    switch (M) {
    case 256:
        return sign < 0 ? (void*)fft_tile_xpose_tma_kernel<double, -1, 4, 2, 8, 8, 8, 4>
                        : (void*)fft_tile_xpose_tma_kernel<double, 1, 4, 2, 8, 8, 8, 4>;
    case 512:
        return sign < 0 ? (void*)fft_tile_xpose_tma_kernel<double, -1, 4, 2, 16, 16, 16, 2>
                        : (void*)fft_tile_xpose_tma_kernel<double, 1, 4, 2, 16, 16, 16, 2>;
    }
    return nullptr;
}

template <>
int TilePtr<double>::points_per_thread(int M) {
    switch (M) {
    case 256: return 8;
    case 512: return 16;
    }
    return 0;
}

template <>
int TilePtr<double>::default_threads(int M, bool xpose) {
    (void)xpose;
    switch (M) {
    case 256: case 512: return 256;
    }
    return 0;
}

}  // namespace gb
