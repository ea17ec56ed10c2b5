// Two-factor FFT kernels (fft_2f.cuh), float C2C rows and columns, pipelined
// rows and the fused rows + box-list transpose, lengths 405..700 (7-smooth, no
// tile kernel): the most balanced split m = M1 * M2 with both factors at most 49.
#include "fft_2f.cuh"

namespace gb {

void* f2_kernel_f32_e(int m, bool cols, int mode, int* m1, int* m2) {
    if (mode != M_C2C) return nullptr;
#define GB_F2(M_, A_, B_)                                                                        \
    case M_:                                                                                    \
        *m1 = A_; *m2 = B_;                                                                     \
        return cols ? (void*)fft2f_kernel<float, A_, B_, M_C2C, true>                         \
                    : (void*)fft2f_kernel<float, A_, B_, M_C2C, false>;
    switch (m) {
    GB_F2(405, 15, 27)
    GB_F2(420, 20, 21)
    GB_F2(432, 18, 24)
    GB_F2(441, 21, 21)
    GB_F2(448, 16, 28)
    GB_F2(450, 18, 25)
    GB_F2(480, 20, 24)
    GB_F2(486, 18, 27)
    GB_F2(490, 14, 35)
    GB_F2(500, 20, 25)
    GB_F2(504, 21, 24)
    GB_F2(525, 21, 25)
    GB_F2(540, 20, 27)
    GB_F2(560, 20, 28)
    GB_F2(567, 21, 27)
    GB_F2(576, 24, 24)
    GB_F2(588, 21, 28)
    GB_F2(600, 24, 25)
    GB_F2(625, 25, 25)
    GB_F2(630, 21, 30)
    GB_F2(640, 20, 32)
    GB_F2(648, 24, 27)
    GB_F2(672, 24, 28)
    GB_F2(675, 25, 27)
    GB_F2(686, 14, 49)
    GB_F2(700, 25, 28)
    }
#undef GB_F2
    return nullptr;
}

void* f2_xpose_kernel_f32_e(int m, int* m1, int* m2) {
#define GB_F2X(M_, A_, B_)                                                                       \
    case M_:                                                                                    \
        *m1 = A_; *m2 = B_;                                                                     \
        return (void*)fft2f_xpose_kernel<float, A_, B_>;
    switch (m) {
    GB_F2X(405, 15, 27)
    GB_F2X(420, 20, 21)
    GB_F2X(432, 18, 24)
    GB_F2X(441, 21, 21)
    GB_F2X(448, 16, 28)
    GB_F2X(450, 18, 25)
    GB_F2X(480, 20, 24)
    GB_F2X(486, 18, 27)
    GB_F2X(490, 14, 35)
    GB_F2X(500, 20, 25)
    GB_F2X(504, 21, 24)
    GB_F2X(525, 21, 25)
    GB_F2X(540, 20, 27)
    GB_F2X(560, 20, 28)
    GB_F2X(567, 21, 27)
    GB_F2X(576, 24, 24)
    GB_F2X(588, 21, 28)
    GB_F2X(600, 24, 25)
    GB_F2X(625, 25, 25)
    GB_F2X(630, 21, 30)
    GB_F2X(640, 20, 32)
    GB_F2X(648, 24, 27)
    GB_F2X(672, 24, 28)
    GB_F2X(675, 25, 27)
    GB_F2X(686, 14, 49)
    GB_F2X(700, 25, 28)
    }
#undef GB_F2X
    return nullptr;
}

void* f2_pipe_kernel_f32_e(int m, int* m1, int* m2) {
#define GB_F2P(M_, A_, B_)                                                                       \
    case M_:                                                                                    \
        *m1 = A_; *m2 = B_;                                                                     \
        return (void*)fft2f_pipe_kernel<float, A_, B_>;
    switch (m) {
    GB_F2P(405, 15, 27)
    GB_F2P(420, 20, 21)
    GB_F2P(432, 18, 24)
    GB_F2P(441, 21, 21)
    GB_F2P(448, 16, 28)
    GB_F2P(450, 18, 25)
    GB_F2P(480, 20, 24)
    GB_F2P(486, 18, 27)
    GB_F2P(490, 14, 35)
    GB_F2P(500, 20, 25)
    GB_F2P(504, 21, 24)
    GB_F2P(525, 21, 25)
    GB_F2P(540, 20, 27)
    GB_F2P(560, 20, 28)
    GB_F2P(567, 21, 27)
    GB_F2P(576, 24, 24)
    GB_F2P(588, 21, 28)
    GB_F2P(600, 24, 25)
    GB_F2P(625, 25, 25)
    GB_F2P(630, 21, 30)
    GB_F2P(640, 20, 32)
    GB_F2P(648, 24, 27)
    GB_F2P(672, 24, 28)
    GB_F2P(675, 25, 27)
    GB_F2P(686, 14, 49)
    GB_F2P(700, 25, 28)
    }
#undef GB_F2P
    return nullptr;
}

}  // namespace gb
