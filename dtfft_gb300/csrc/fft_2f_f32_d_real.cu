// Two-factor FFT kernels (fft_2f.cuh), float rows of the real modes, cores of
// 300..400 points: R2C / C2R of even n (core n/2) for every core, of odd n
// (full-length core) for the odd cores.  Split m = M1 * M2 as in the C2C units.
#include "fft_2f.cuh"

namespace gb {

void* f2_kernel_f32_d_real(int m, bool cols, int mode, int* m1, int* m2) {
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
    GB_F2(300, 15, 20)
    GB_F2ODD(315, 15, 21)
    GB_F2(320, 16, 20)
    GB_F2(324, 18, 18)
    GB_F2(336, 16, 21)
    GB_F2ODD(343, 7, 49)
    GB_F2(350, 14, 25)
    GB_F2(360, 18, 20)
    GB_F2ODD(375, 15, 25)
    GB_F2(378, 18, 21)
    GB_F2(384, 16, 24)
    GB_F2(392, 14, 28)
    GB_F2(400, 20, 20)
    }
#undef GB_F2
#undef GB_F2ODD
    return nullptr;
}

}  // namespace gb
