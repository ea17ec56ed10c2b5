// Two-factor FFT kernels (fft_2f.cuh), float C2C rows and columns, pipelined
// rows and the fused rows + box-list transpose, lengths 200..294: the most balanced split
// m = M1 * M2 with both factors at most 49.
#include "fft_2f.cuh"

namespace gb {

void* f2_kernel_f32_c(int m, bool cols, int mode, int* m1, int* m2) {
    if (mode != M_C2C) return nullptr;
#define GB_F2(M_, A_, B_)                                                                        \
    case M_:                                                                                    \
        *m1 = A_; *m2 = B_;                                                                     \
        return cols ? (void*)fft2f_kernel<float, A_, B_, M_C2C, true>                         \
                    : (void*)fft2f_kernel<float, A_, B_, M_C2C, false>;
    switch (m) {
    GB_F2(200, 10, 20)
    GB_F2(210, 14, 15)
    GB_F2(216, 12, 18)
    GB_F2(224, 14, 16)
    GB_F2(225, 15, 15)
    GB_F2(240, 15, 16)
    GB_F2(243, 9, 27)
    GB_F2(245, 7, 35)
    GB_F2(250, 10, 25)
    GB_F2(252, 14, 18)
    GB_F2(270, 15, 18)
    GB_F2(280, 14, 20)
    GB_F2(288, 16, 18)
    GB_F2(294, 14, 21)
    }
#undef GB_F2
    return nullptr;
}

void* f2_xpose_kernel_f32_c(int m, int* m1, int* m2) {
#define GB_F2X(M_, A_, B_)                                                                       \
    case M_:                                                                                    \
        *m1 = A_; *m2 = B_;                                                                     \
        return (void*)fft2f_xpose_kernel<float, A_, B_>;
    switch (m) {
    GB_F2X(200, 10, 20)
    GB_F2X(210, 14, 15)
    GB_F2X(216, 12, 18)
    GB_F2X(224, 14, 16)
    GB_F2X(225, 15, 15)
    GB_F2X(240, 15, 16)
    GB_F2X(243, 9, 27)
    GB_F2X(245, 7, 35)
    GB_F2X(250, 10, 25)
    GB_F2X(252, 14, 18)
    GB_F2X(270, 15, 18)
    GB_F2X(280, 14, 20)
    GB_F2X(288, 16, 18)
    GB_F2X(294, 14, 21)
    }
#undef GB_F2X
    return nullptr;
}

void* f2_pipe_kernel_f32_c(int m, int* m1, int* m2) {
#define GB_F2P(M_, A_, B_)                                                                       \
    case M_:                                                                                    \
        *m1 = A_; *m2 = B_;                                                                     \
        return (void*)fft2f_pipe_kernel<float, A_, B_>;
    switch (m) {
    GB_F2P(200, 10, 20)
    GB_F2P(210, 14, 15)
    GB_F2P(216, 12, 18)
    GB_F2P(224, 14, 16)
    GB_F2P(225, 15, 15)
    GB_F2P(240, 15, 16)
    GB_F2P(243, 9, 27)
    GB_F2P(245, 7, 35)
    GB_F2P(250, 10, 25)
    GB_F2P(252, 14, 18)
    GB_F2P(270, 15, 18)
    GB_F2P(280, 14, 20)
    GB_F2P(288, 16, 18)
    GB_F2P(294, 14, 21)
    }
#undef GB_F2P
    return nullptr;
}

}  // namespace gb
