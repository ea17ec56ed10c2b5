// Kernel instantiations for double precision (built in parallel with the other translation units).
#include "fft_kernels.cuh"

namespace gb {

void* reg_kernel_ext_f64(int E, bool cols, bool c2c);

template <>
void* KPtr<double>::reg(int E, bool cols, bool c2c) {
#define GB_R(E_) \
    case E_: \
        if (cols) return c2c ? (void*)fft_reg_kernel<double, E_, true, true> : (void*)fft_reg_kernel<double, E_, true, false>; \
        return c2c ? (void*)fft_reg_kernel<double, E_, false, true> : (void*)fft_reg_kernel<double, E_, false, false>;
    switch (E) {
        GB_R(8) GB_R(16) GB_R(24) GB_R(20) GB_R(28)
    }
#undef GB_R
    return reg_kernel_ext_f64(E, cols, c2c);
}

template <>
void* KPtr<double>::generic(bool cols) {
    return cols ? (void*)fft_kernel<double, true> : (void*)fft_kernel<double, false>;
}

template <>
void* KPtr<double>::xpose(int E) {
    switch (E) {
    case 8: return (void*)fft_xpose_kernel<double, 8>;
    case 16: return (void*)fft_xpose_kernel<double, 16>;
    case 24: return (void*)fft_xpose_kernel<double, 24>;
    case 20: return (void*)fft_xpose_kernel<double, 20>;
    case 28: return (void*)fft_xpose_kernel<double, 28>;
    }
    return nullptr;
}

}  // namespace gb
