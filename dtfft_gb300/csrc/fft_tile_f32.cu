// Tile-kernel instantiations for single precision (complex64 rows).
#include "fft_tile.cuh"

namespace gb {

// Warp counts compiled per row length: the first entry is the default, the
// others are selectable for measurements (DTFFT_GB_TILE_WARPS = <warps>,
// DTFFT_GB_XPOSE_WARPS = <compute>,<store>).
#define GB_PLAIN(NW_, E_, ...)                                                                   \
    if (nw == NW_ || (nw == 0 && first)) return sign < 0 ? (void*)fft_tile_kernel<float, -1, NW_, E_, __VA_ARGS__> \
                                                        : (void*)fft_tile_kernel<float, 1, NW_, E_, __VA_ARGS__>;  \
    first = false;
#define GB_XPOSE(C_, S_, E_, ...)                                                                \
    if ((ncw == C_ && nsw == S_) || (ncw == 0 && first))                                         \
        return sign < 0 ? (void*)fft_tile_xpose_kernel<float, -1, C_, S_, E_, __VA_ARGS__>       \
                        : (void*)fft_tile_xpose_kernel<float, 1, C_, S_, E_, __VA_ARGS__>;       \
    first = false;

template <>
void* TilePtr<float>::get(int M, int sign, bool xpose, int ncw, int nsw) {
    bool first = true;
    const int nw = ncw;
    if (!xpose) {
        switch (M) {
        case 256: GB_PLAIN(4, 8, 8, 8, 4) GB_PLAIN(8, 8, 8, 8, 4) break;
        case 512: GB_PLAIN(4, 16, 16, 16, 2) GB_PLAIN(8, 16, 16, 16, 2) break;
        case 768: GB_PLAIN(8, 24, 8, 8, 4, 3) GB_PLAIN(4, 24, 8, 8, 4, 3) break;
        case 1024: GB_PLAIN(8, 32, 16, 16, 4) GB_PLAIN(4, 32, 16, 16, 4) break;
        }
        return nullptr;
    }
    switch (M) {
    case 256: GB_XPOSE(3, 5, 8, 8, 8, 4) GB_XPOSE(4, 4, 8, 8, 8, 4) break;
    case 512: GB_XPOSE(3, 5, 16, 16, 16, 2) GB_XPOSE(4, 4, 16, 16, 16, 2) GB_XPOSE(4, 8, 16, 16, 16, 2) GB_XPOSE(4, 12, 16, 16, 16, 2) GB_XPOSE(6, 6, 16, 16, 16, 2) break;
    case 768: GB_XPOSE(4, 4, 24, 8, 8, 4, 3) GB_XPOSE(3, 5, 24, 8, 8, 4, 3) break;
    case 1024: GB_XPOSE(4, 4, 32, 16, 16, 4) GB_XPOSE(3, 5, 32, 16, 16, 4) break;
    }
    return nullptr;
}
#undef GB_PLAIN
#undef GB_XPOSE

// Fused passes with the tensor-store write-out, 8 compute warps + 1 producer
// warp: 256- and 512-point rows as 16-row tiles (a row pair per warp, 128-byte
// lines), 768- and 1024-point rows as 8-row tiles (a row per warp, 64-byte
// lines: two 768-point spectra per thread exceed the 168 registers of a
// 288-thread CTA).
#define GB_TMA(RPW_, E_, ...)                                                                    \
    if (rows) *rows = 8 * RPW_;                                                                  \
    if (warps) *warps = 8;                                                                       \
    return sign < 0 ? (void*)fft_tile_xpose_tma_kernel<float, -1, 8, RPW_, E_, __VA_ARGS__>      \
                    : (void*)fft_tile_xpose_tma_kernel<float, 1, 8, RPW_, E_, __VA_ARGS__>;
template <>
void* TilePtr<float>::get_tma(int M, int sign, int* rows, int* warps) {
    switch (M) {
    case 256: GB_TMA(2, 8, 8, 8, 4)
    case 512: GB_TMA(2, 16, 16, 16, 2)
    case 768: GB_TMA(1, 24, 8, 8, 4, 3)
    case 1024: GB_TMA(1, 32, 16, 16, 4)
    }
    return nullptr;
}
#undef GB_TMA

template <>
int TilePtr<float>::points_per_thread(int M) {
    switch (M) {
    case 256: return 8;
    case 512: return 16;
    case 768: return 24;
    case 1024: return 32;
    }
    return 0;
}

// Threads of the default variant.
template <>
int TilePtr<float>::default_threads(int M, bool xpose) {
    switch (M) {
    case 256: return xpose ? 32 * 8 : 32 * 4;
    case 512: return xpose ? 32 * 8 : 32 * 4;
    case 768: return xpose ? 32 * 8 : 32 * 8;
    case 1024: return xpose ? 32 * 8 : 32 * 8;
    }
    return 0;
}

}  // namespace gb
