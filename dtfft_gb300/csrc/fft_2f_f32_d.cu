// Two-factor FFT kernels (fft_2f.cuh), float C2C rows and columns, pipelined
// rows and the fused rows + box-list transpose, lengths 300..400: the most balanced split
// m = M1 * M2 with both factors at most 49.
#include "fft_2f.cuh"

namespace gb {

void* f2_kernel_f32_d(int m, bool cols, int mode, int* m1, int* m2) {
    if (mode != M_C2C) return nullptr;
#define GB_F2(M_, A_, B_)                                                                        \
    case M_:                                                                                    \
        *m1 = A_; *m2 = B_;                                                                     \
        return cols ? (void*)fft2f_kernel<float, A_, B_, M_C2C, true>                         \
                    : (void*)fft2f_kernel<float, A_, B_, M_C2C, false>;
    switch (m) {
    GB_F2(300, 15, 20)
    GB_F2(315, 15, 21)
    GB_F2(320, 16, 20)
    GB_F2(324, 18, 18)
    GB_F2(336, 16, 21)
    GB_F2(343, 7, 49)
    GB_F2(350, 14, 25)
    GB_F2(360, 18, 20)
    GB_F2(375, 15, 25)
    GB_F2(378, 18, 21)
    GB_F2(384, 16, 24)
    GB_F2(392, 14, 28)
    GB_F2(400, 20, 20)
    }
#undef GB_F2
    return nullptr;
}

void* f2_xpose_kernel_f32_d(int m, int* m1, int* m2) {
#define GB_F2X(M_, A_, B_)                                                                       \
    case M_:                                                                                    \
        *m1 = A_; *m2 = B_;                                                                     \
        return (void*)fft2f_xpose_kernel<float, A_, B_>;
    switch (m) {
    GB_F2X(300, 15, 20)
    GB_F2X(315, 15, 21)
    GB_F2X(320, 16, 20)
    GB_F2X(324, 18, 18)
    GB_F2X(336, 16, 21)
    GB_F2X(343, 7, 49)
    GB_F2X(350, 14, 25)
    GB_F2X(360, 18, 20)
    GB_F2X(375, 15, 25)
    GB_F2X(378, 18, 21)
    GB_F2X(384, 16, 24)
    GB_F2X(392, 14, 28)
    GB_F2X(400, 20, 20)
    }
#undef GB_F2X
    return nullptr;
}

void* f2_pipe_kernel_f32_d(int m, int* m1, int* m2) {
#define GB_F2P(M_, A_, B_)                                                                       \
    case M_:                                                                                    \
        *m1 = A_; *m2 = B_;                                                                     \
        return (void*)fft2f_pipe_kernel<float, A_, B_>;
    switch (m) {
    GB_F2P(300, 15, 20)
    GB_F2P(315, 15, 21)
    GB_F2P(320, 16, 20)
    GB_F2P(324, 18, 18)
    GB_F2P(336, 16, 21)
    GB_F2P(343, 7, 49)
    GB_F2P(350, 14, 25)
    GB_F2P(360, 18, 20)
    GB_F2P(375, 15, 25)
    GB_F2P(378, 18, 21)
    GB_F2P(384, 16, 24)
    GB_F2P(392, 14, 28)
    GB_F2P(400, 20, 20)
    }
#undef GB_F2P
    return nullptr;
}

}  // namespace gb
