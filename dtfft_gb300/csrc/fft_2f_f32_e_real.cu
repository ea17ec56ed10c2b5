// Two-factor FFT kernels (fft_2f.cuh), float rows of the real modes, cores of
// 405..700 points: R2C / C2R of even n (core n/2) for every core, of odd n
// (full-length core) for the odd cores.  Split m = M1 * M2 as in the C2C units.
#include "fft_2f.cuh"

namespace gb {

void* f2_kernel_f32_e_real(int m, bool cols, int mode, int* m1, int* m2) {
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
    GB_F2ODD(405, 15, 27)
    GB_F2(420, 20, 21)
    GB_F2(432, 18, 24)
    GB_F2ODD(441, 21, 21)
    GB_F2(448, 16, 28)
    GB_F2(450, 18, 25)
    GB_F2(480, 20, 24)
    GB_F2(486, 18, 27)
    GB_F2(490, 14, 35)
    GB_F2(500, 20, 25)
    GB_F2(504, 21, 24)
    GB_F2ODD(525, 21, 25)
    GB_F2(540, 20, 27)
    GB_F2(560, 20, 28)
    GB_F2ODD(567, 21, 27)
    GB_F2(576, 24, 24)
    GB_F2(588, 21, 28)
    GB_F2(600, 24, 25)
    GB_F2ODD(625, 25, 25)
    GB_F2(630, 21, 30)
    GB_F2(640, 20, 32)
    GB_F2(648, 24, 27)
    GB_F2(672, 24, 28)
    GB_F2ODD(675, 25, 27)
    GB_F2(686, 14, 49)
    GB_F2(700, 25, 28)
    }
#undef GB_F2
#undef GB_F2ODD
    return nullptr;
}

}  // namespace gb
