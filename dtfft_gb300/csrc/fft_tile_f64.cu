// Tile-kernel instantiations for double precision (complex128 rows).
#include "fft_tile.cuh"

namespace gb {

template <int SG>
static void* tile_plain_f64(int M) {
    switch (M) {
    case 256: return (void*)fft_tile_kernel<double, SG, 8, 8, 8, 4>;
    case 512: return (void*)fft_tile_kernel<double, SG, 16, 16, 16, 2>;
    }
    return nullptr;
}

template <int SG>
static void* tile_xpose_f64(int M) {
    switch (M) {
    case 256: return (void*)fft_tile_xpose_kernel<double, SG, 8, 8, 8, 4>;
    case 512: return (void*)fft_tile_xpose_kernel<double, SG, 16, 16, 16, 2>;
    }
    return nullptr;
}

template <>
void* TilePtr<double>::get(int M, int sign, bool xpose) {
    if (sign < 0) return xpose ? tile_xpose_f64<-1>(M) : tile_plain_f64<-1>(M);
    return xpose ? tile_xpose_f64<1>(M) : tile_plain_f64<1>(M);
}

template <>
int TilePtr<double>::points_per_thread(int M) {
    switch (M) {
    case 256: return 8;
    case 512: return 16;
    }
    return 0;
}

}  // namespace gb
