// Register FFT kernels for the 7-smooth points-per-thread counts (float):
// rows whose length has the prime factors 3, 5 or 7 in combinations the
// power-of-two-heavy counts of the main instantiation unit cannot hold.
#include "fft_kernels.cuh"

namespace gb {

void* reg_kernel_ext_f32(int E, bool cols, bool c2c) {
#define GB_R(E_) \
    case E_: \
        if (cols) return c2c ? (void*)fft_reg_kernel<float, E_, true, true> : (void*)fft_reg_kernel<float, E_, true, false>; \
        return c2c ? (void*)fft_reg_kernel<float, E_, false, true> : (void*)fft_reg_kernel<float, E_, false, false>;
    switch (E) {
    GB_R(7)
    GB_R(9)
    GB_R(10)
    GB_R(12)
    GB_R(14)
    GB_R(15)
    GB_R(18)
    GB_R(21)
    GB_R(25)
    GB_R(30)
    GB_R(35)
    GB_R(42)
    }
#undef GB_R
    return nullptr;
}

}  // namespace gb
