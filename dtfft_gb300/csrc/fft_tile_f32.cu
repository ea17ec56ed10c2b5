// Tile-kernel instantiations for single precision (complex64 rows).
#include "fft_tile.cuh"

namespace gb {

template <int SG>
static void* tile_plain_f32(int M) {
    switch (M) {
    case 256: return (void*)fft_tile_kernel<float, SG, 8, 8, 8, 4>;
    case 512: return (void*)fft_tile_kernel<float, SG, 16, 16, 16, 2>;
    case 768: return (void*)fft_tile_kernel<float, SG, 24, 8, 8, 4, 3>;
    case 1024: return (void*)fft_tile_kernel<float, SG, 32, 16, 16, 4>;
    }
    return nullptr;
}

template <int SG>
static void* tile_xpose_f32(int M) {
    switch (M) {
    case 256: return (void*)fft_tile_xpose_kernel<float, SG, 8, 8, 8, 4>;
    case 512: return (void*)fft_tile_xpose_kernel<float, SG, 16, 16, 16, 2>;
    case 768: return (void*)fft_tile_xpose_kernel<float, SG, 24, 8, 8, 4, 3>;
    case 1024: return (void*)fft_tile_xpose_kernel<float, SG, 32, 16, 16, 4>;
    }
    return nullptr;
}

template <>
void* TilePtr<float>::get(int M, int sign, bool xpose) {
    if (sign < 0) return xpose ? tile_xpose_f32<-1>(M) : tile_plain_f32<-1>(M);
    return xpose ? tile_xpose_f32<1>(M) : tile_plain_f32<1>(M);
}

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

}  // namespace gb
