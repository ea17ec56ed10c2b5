// Two-factor FFT kernels (fft_2f.cuh), float C2C rows and columns, pipelined
// rows and the fused rows + box-list transpose, lengths 105..196: the most balanced split
// m = M1 * M2 with both factors at most 49.
#include "fft_2f.cuh"

namespace gb {

void* f2_kernel_f32_b(int m, bool cols, int mode, int* m1, int* m2) {
    if (mode != M_C2C) return nullptr;
#define GB_F2(M_, A_, B_)                                                                        \
    case M_:                                                                                    \
        *m1 = A_; *m2 = B_;                                                                     \
        return cols ? (void*)fft2f_kernel<float, A_, B_, M_C2C, true>                         \
                    : (void*)fft2f_kernel<float, A_, B_, M_C2C, false>;
    switch (m) {
    GB_F2(105, 7, 15)
    GB_F2(108, 9, 12)
    GB_F2(112, 8, 14)
    GB_F2(120, 10, 12)
    GB_F2(125, 5, 25)
    GB_F2(126, 9, 14)
    GB_F2(128, 8, 16)
    GB_F2(135, 9, 15)
    GB_F2(140, 10, 14)
    GB_F2(144, 12, 12)
    GB_F2(147, 7, 21)
    GB_F2(150, 10, 15)
    GB_F2(160, 10, 16)
    GB_F2(162, 9, 18)
    GB_F2(168, 12, 14)
    GB_F2(175, 7, 25)
    GB_F2(180, 12, 15)
    GB_F2(189, 9, 21)
    GB_F2(192, 12, 16)
    GB_F2(196, 14, 14)
    }
#undef GB_F2
    return nullptr;
}

void* f2_xpose_kernel_f32_b(int m, int* m1, int* m2) {
#define GB_F2X(M_, A_, B_)                                                                       \
    case M_:                                                                                    \
        *m1 = A_; *m2 = B_;                                                                     \
        return (void*)fft2f_xpose_kernel<float, A_, B_>;
    switch (m) {
    GB_F2X(105, 7, 15)
    GB_F2X(108, 9, 12)
    GB_F2X(112, 8, 14)
    GB_F2X(120, 10, 12)
    GB_F2X(125, 5, 25)
    GB_F2X(126, 9, 14)
    GB_F2X(128, 8, 16)
    GB_F2X(135, 9, 15)
    GB_F2X(140, 10, 14)
    GB_F2X(144, 12, 12)
    GB_F2X(147, 7, 21)
    GB_F2X(150, 10, 15)
    GB_F2X(160, 10, 16)
    GB_F2X(162, 9, 18)
    GB_F2X(168, 12, 14)
    GB_F2X(175, 7, 25)
    GB_F2X(180, 12, 15)
    GB_F2X(189, 9, 21)
    GB_F2X(192, 12, 16)
    GB_F2X(196, 14, 14)
    }
#undef GB_F2X
    return nullptr;
}

void* f2_pipe_kernel_f32_b(int m, int* m1, int* m2) {
#define GB_F2P(M_, A_, B_)                                                                       \
    case M_:                                                                                    \
        *m1 = A_; *m2 = B_;                                                                     \
        return (void*)fft2f_pipe_kernel<float, A_, B_>;
    switch (m) {
    GB_F2P(105, 7, 15)
    GB_F2P(108, 9, 12)
    GB_F2P(112, 8, 14)
    GB_F2P(120, 10, 12)
    GB_F2P(125, 5, 25)
    GB_F2P(126, 9, 14)
    GB_F2P(128, 8, 16)
    GB_F2P(135, 9, 15)
    GB_F2P(140, 10, 14)
    GB_F2P(144, 12, 12)
    GB_F2P(147, 7, 21)
    GB_F2P(150, 10, 15)
    GB_F2P(160, 10, 16)
    GB_F2P(162, 9, 18)
    GB_F2P(168, 12, 14)
    GB_F2P(175, 7, 25)
    GB_F2P(180, 12, 15)
    GB_F2P(189, 9, 21)
    GB_F2P(192, 12, 16)
    GB_F2P(196, 14, 14)
    }
#undef GB_F2P
    return nullptr;
}

}  // namespace gb
