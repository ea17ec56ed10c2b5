// Two-factor FFT kernels (fft_2f.cuh), float rows of the real modes, cores of
// 720..1008 points: R2C / C2R of even n (core n/2) for every core, of odd n
// (full-length core) for the odd cores.  Split m = M1 * M2 as in the C2C units.
#include "fft_2f.cuh"

namespace gb {

void* f2_kernel_f32_f_real(int m, bool cols, int mode, int* m1, int* m2) {
    if (cols) return nullptr;
#define GB_F2(M_, A_, B_)                                                                        \
    case M_:                                                                                    \
        *m1 = A_; *m2 = B_;                                                                     \
        if (mode == M_R2C_HALF) return (void*)fft2f_kernel<float, A_, B_, M_R2C_HALF, false>;  \
        if (mode == M_C2R_HALF) return (void*)fft2f_kernel<float, A_, B_, M_C2R_HALF, false>;  \
        return nullptr;
#define GB_F2ODD(M_, A_, B_)                                                                     \
    case M_:                                                                                    \
        *m1 = A_; *m2 = B_;                                                                     \
        if (mode == M_R2C_HALF) return (void*)fft2f_kernel<float, A_, B_, M_R2C_HALF, false>;  \
        if (mode == M_C2R_HALF) return (void*)fft2f_kernel<float, A_, B_, M_C2R_HALF, false>;  \
        if (mode == M_R2C_FULL) return (void*)fft2f_kernel<float, A_, B_, M_R2C_FULL, false>;  \
        if (mode == M_C2R_FULL) return (void*)fft2f_kernel<float, A_, B_, M_C2R_FULL, false>;  \
        return nullptr;
    switch (m) {
    GB_F2(720, 24, 30)
    GB_F2ODD(729, 27, 27)
    GB_F2ODD(735, 21, 35)
    GB_F2(750, 25, 30)
    GB_F2(756, 27, 28)
    GB_F2(784, 28, 28)
    GB_F2(800, 25, 32)
    GB_F2(810, 27, 30)
    GB_F2(840, 28, 30)
    GB_F2(864, 27, 32)
    GB_F2ODD(875, 25, 35)
    GB_F2(882, 21, 42)
    GB_F2(896, 28, 32)
    GB_F2(900, 30, 30)
    GB_F2ODD(945, 27, 35)
    GB_F2(960, 30, 32)
    GB_F2(972, 27, 36)
    GB_F2(980, 28, 35)
    GB_F2(1000, 25, 40)
    GB_F2(1008, 28, 36)
    }
#undef GB_F2
#undef GB_F2ODD
    return nullptr;
}

}  // namespace gb
