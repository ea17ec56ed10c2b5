// Two-factor FFT kernels (fft_2f.cuh), float rows of the real modes, cores of
// 105..196 points: R2C / C2R of even n (core n/2) for every core, of odd n
// (full-length core) for the odd cores.  Split m = M1 * M2 as in the C2C units.
#include "fft_2f.cuh"

namespace gb {

void* f2_kernel_f32_b_real(int m, bool cols, int mode, int* m1, int* m2) {
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
    GB_F2ODD(105, 7, 15)
    GB_F2(108, 9, 12)
    GB_F2(112, 8, 14)
    GB_F2(120, 10, 12)
    GB_F2ODD(125, 5, 25)
    GB_F2(126, 9, 14)
    GB_F2ODD(135, 9, 15)
    GB_F2(140, 10, 14)
    GB_F2(144, 12, 12)
    GB_F2ODD(147, 7, 21)
    GB_F2(150, 10, 15)
    GB_F2(160, 10, 16)
    GB_F2(162, 9, 18)
    GB_F2(168, 12, 14)
    GB_F2ODD(175, 7, 25)
    GB_F2(180, 12, 15)
    GB_F2ODD(189, 9, 21)
    GB_F2(192, 12, 16)
    GB_F2(196, 14, 14)
    }
#undef GB_F2
#undef GB_F2ODD
    return nullptr;
}

}  // namespace gb
