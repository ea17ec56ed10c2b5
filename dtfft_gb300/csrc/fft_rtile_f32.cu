// Runtime-schedule tile-kernel instantiations for single precision (complex64),
// one per points-per-thread count E.
#include "fft_rtile.cuh"

namespace gb {

#define GB_RT_E(E_)                                                                                               \
    case E_:                                                                                                      \
        if (xpose) return sign < 0 ? (void*)fft_rtile_xpose_kernel<float, -1, kRtileComputeWarps, kRtileStoreWarps, E_> \
                                   : (void*)fft_rtile_xpose_kernel<float, 1, kRtileComputeWarps, kRtileStoreWarps, E_>;  \
        return sign < 0 ? (void*)fft_rtile_kernel<float, -1, kRtilePlainWarps, E_>                               \
                        : (void*)fft_rtile_kernel<float, 1, kRtilePlainWarps, E_>;

template <>
void* RtilePtr<float>::get(int E, int sign, bool xpose) {
    switch (E) {
        GB_RT_E(6) GB_RT_E(7) GB_RT_E(8) GB_RT_E(9) GB_RT_E(10) GB_RT_E(12) GB_RT_E(14) GB_RT_E(15)
        GB_RT_E(16) GB_RT_E(18) GB_RT_E(20) GB_RT_E(21) GB_RT_E(24) GB_RT_E(25) GB_RT_E(27) GB_RT_E(28)
        GB_RT_E(30)
    }
    return nullptr;
}
#undef GB_RT_E

template <>
bool RtilePtr<float>::has(int E) { return get(E, -1, false) != nullptr; }

}  // namespace gb

namespace gb {
// No double-precision runtime-schedule variants: complex128 rows take the
// compile-time tile kernels or the register kernels.
template <>
void* RtilePtr<double>::get(int, int, bool) { return nullptr; }
template <>
bool RtilePtr<double>::has(int) { return false; }
}  // namespace gb
