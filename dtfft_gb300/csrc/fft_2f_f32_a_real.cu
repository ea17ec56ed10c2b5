// Two-factor FFT kernels (fft_2f.cuh), float rows of the real modes, cores of
// 40..100 points: R2C / C2R of even n (core n/2) for every core, of odd n
// (full-length core) for the odd cores.  Split m = M1 * M2 as in the C2C units.
#include "fft_2f.cuh"

namespace gb {

void* f2_kernel_f32_a_real(int m, bool cols, int mode, int* m1, int* m2) {
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
    GB_F2(40, 5, 8)
    GB_F2(42, 6, 7)
    GB_F2ODD(45, 5, 9)
    GB_F2(48, 6, 8)
    GB_F2ODD(49, 7, 7)
    GB_F2(50, 5, 10)
    GB_F2(54, 6, 9)
    GB_F2(56, 7, 8)
    GB_F2(60, 6, 10)
    GB_F2ODD(63, 7, 9)
    GB_F2(70, 7, 10)
    GB_F2(72, 8, 9)
    GB_F2ODD(75, 5, 15)
    GB_F2(80, 8, 10)
    GB_F2ODD(81, 9, 9)
    GB_F2(84, 7, 12)
    GB_F2(90, 9, 10)
    GB_F2(96, 8, 12)
    GB_F2(98, 7, 14)
    GB_F2(100, 10, 10)
    }
#undef GB_F2
#undef GB_F2ODD
    return nullptr;
}

}  // namespace gb
