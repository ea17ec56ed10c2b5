// Two-factor FFT kernels (fft_2f.cuh), float C2C rows and columns, pipelined
// rows and the fused rows + box-list transpose, lengths 720..1008 (7-smooth, no
// tile kernel): the most balanced split m = M1 * M2 with both factors at most 49.
#include "fft_2f.cuh"

namespace gb {

void* f2_kernel_f32_f(int m, bool cols, int mode, int* m1, int* m2) {
    if (mode != M_C2C) return nullptr;
#define GB_F2(M_, A_, B_)                                                                        \
    case M_:                                                                                    \
        *m1 = A_; *m2 = B_;                                                                     \
        return cols ? (void*)fft2f_kernel<float, A_, B_, M_C2C, true>                         \
                    : (void*)fft2f_kernel<float, A_, B_, M_C2C, false>;
    switch (m) {
    GB_F2(720, 24, 30)
    GB_F2(729, 27, 27)
    GB_F2(735, 21, 35)
    GB_F2(750, 25, 30)
    GB_F2(756, 27, 28)
    GB_F2(784, 28, 28)
    GB_F2(800, 25, 32)
    GB_F2(810, 27, 30)
    GB_F2(840, 28, 30)
    GB_F2(864, 27, 32)
    GB_F2(875, 25, 35)
    GB_F2(882, 21, 42)
    GB_F2(896, 28, 32)
    GB_F2(900, 30, 30)
    GB_F2(945, 27, 35)
    GB_F2(960, 30, 32)
    GB_F2(972, 27, 36)
    GB_F2(980, 28, 35)
    GB_F2(1000, 25, 40)
    GB_F2(1008, 28, 36)
    }
#undef GB_F2
    return nullptr;
}

void* f2_xpose_kernel_f32_f(int m, int* m1, int* m2) {
#define GB_F2X(M_, A_, B_)                                                                       \
    case M_:                                                                                    \
        *m1 = A_; *m2 = B_;                                                                     \
        return (void*)fft2f_xpose_kernel<float, A_, B_>;
    switch (m) {
    GB_F2X(720, 24, 30)
    GB_F2X(729, 27, 27)
    GB_F2X(735, 21, 35)
    GB_F2X(750, 25, 30)
    GB_F2X(756, 27, 28)
    GB_F2X(784, 28, 28)
    GB_F2X(800, 25, 32)
    GB_F2X(810, 27, 30)
    GB_F2X(840, 28, 30)
    GB_F2X(864, 27, 32)
    GB_F2X(875, 25, 35)
    GB_F2X(882, 21, 42)
    GB_F2X(896, 28, 32)
    GB_F2X(900, 30, 30)
    GB_F2X(945, 27, 35)
    GB_F2X(960, 30, 32)
    GB_F2X(972, 27, 36)
    GB_F2X(980, 28, 35)
    GB_F2X(1000, 25, 40)
    GB_F2X(1008, 28, 36)
    }
#undef GB_F2X
    return nullptr;
}

void* f2_pipe_kernel_f32_f(int m, int* m1, int* m2) {
#define GB_F2P(M_, A_, B_)                                                                       \
    case M_:                                                                                    \
        *m1 = A_; *m2 = B_;                                                                     \
        return (void*)fft2f_pipe_kernel<float, A_, B_>;
    switch (m) {
    GB_F2P(720, 24, 30)
    GB_F2P(729, 27, 27)
    GB_F2P(735, 21, 35)
    GB_F2P(750, 25, 30)
    GB_F2P(756, 27, 28)
    GB_F2P(784, 28, 28)
    GB_F2P(800, 25, 32)
    GB_F2P(810, 27, 30)
    GB_F2P(840, 28, 30)
    GB_F2P(864, 27, 32)
    GB_F2P(875, 25, 35)
    GB_F2P(882, 21, 42)
    GB_F2P(896, 28, 32)
    GB_F2P(900, 30, 30)
    GB_F2P(945, 27, 35)
    GB_F2P(960, 30, 32)
    GB_F2P(972, 27, 36)
    GB_F2P(980, 28, 35)
    GB_F2P(1000, 25, 40)
    GB_F2P(1008, 28, 36)
    }
#undef GB_F2P
    return nullptr;
}

}  // namespace gb
