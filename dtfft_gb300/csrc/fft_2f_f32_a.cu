// Two-factor FFT kernels (fft_2f.cuh), float C2C rows and columns, pipelined
// rows and the fused rows + box-list transpose, lengths 40..100: the most balanced split
// m = M1 * M2 with both factors at most 49.
#include "fft_2f.cuh"

namespace gb {

void* f2_kernel_f32_a(int m, bool cols, int mode, int* m1, int* m2) {
    if (mode != M_C2C) return nullptr;
#define GB_F2(M_, A_, B_)                                                                        \
    case M_:                                                                                    \
        *m1 = A_; *m2 = B_;                                                                     \
        return cols ? (void*)fft2f_kernel<float, A_, B_, M_C2C, true>                         \
                    : (void*)fft2f_kernel<float, A_, B_, M_C2C, false>;
    switch (m) {
    GB_F2(40, 5, 8)
    GB_F2(42, 6, 7)
    GB_F2(45, 5, 9)
    GB_F2(48, 6, 8)
    GB_F2(49, 7, 7)
    GB_F2(50, 5, 10)
    GB_F2(54, 6, 9)
    GB_F2(56, 7, 8)
    GB_F2(60, 6, 10)
    GB_F2(63, 7, 9)
    GB_F2(64, 8, 8)
    GB_F2(70, 7, 10)
    GB_F2(72, 8, 9)
    GB_F2(75, 5, 15)
    GB_F2(80, 8, 10)
    GB_F2(81, 9, 9)
    GB_F2(84, 7, 12)
    GB_F2(90, 9, 10)
    GB_F2(96, 8, 12)
    GB_F2(98, 7, 14)
    GB_F2(100, 10, 10)
    }
#undef GB_F2
    return nullptr;
}

void* f2_xpose_kernel_f32_a(int m, int* m1, int* m2) {
#define GB_F2X(M_, A_, B_)                                                                       \
    case M_:                                                                                    \
        *m1 = A_; *m2 = B_;                                                                     \
        return (void*)fft2f_xpose_kernel<float, A_, B_>;
    switch (m) {
    GB_F2X(40, 5, 8)
    GB_F2X(42, 6, 7)
    GB_F2X(45, 5, 9)
    GB_F2X(48, 6, 8)
    GB_F2X(49, 7, 7)
    GB_F2X(50, 5, 10)
    GB_F2X(54, 6, 9)
    GB_F2X(56, 7, 8)
    GB_F2X(60, 6, 10)
    GB_F2X(63, 7, 9)
    GB_F2X(64, 8, 8)
    GB_F2X(70, 7, 10)
    GB_F2X(72, 8, 9)
    GB_F2X(75, 5, 15)
    GB_F2X(80, 8, 10)
    GB_F2X(81, 9, 9)
    GB_F2X(84, 7, 12)
    GB_F2X(90, 9, 10)
    GB_F2X(96, 8, 12)
    GB_F2X(98, 7, 14)
    GB_F2X(100, 10, 10)
    }
#undef GB_F2X
    return nullptr;
}

void* f2_pipe_kernel_f32_a(int m, int* m1, int* m2) {
#define GB_F2P(M_, A_, B_)                                                                       \
    case M_:                                                                                    \
        *m1 = A_; *m2 = B_;                                                                     \
        return (void*)fft2f_pipe_kernel<float, A_, B_>;
    switch (m) {
    GB_F2P(40, 5, 8)
    GB_F2P(42, 6, 7)
    GB_F2P(45, 5, 9)
    GB_F2P(48, 6, 8)
    GB_F2P(49, 7, 7)
    GB_F2P(50, 5, 10)
    GB_F2P(54, 6, 9)
    GB_F2P(56, 7, 8)
    GB_F2P(60, 6, 10)
    GB_F2P(63, 7, 9)
    GB_F2P(64, 8, 8)
    GB_F2P(70, 7, 10)
    GB_F2P(72, 8, 9)
    GB_F2P(75, 5, 15)
    GB_F2P(80, 8, 10)
    GB_F2P(81, 9, 9)
    GB_F2P(84, 7, 12)
    GB_F2P(90, 9, 10)
    GB_F2P(96, 8, 12)
    GB_F2P(98, 7, 14)
    GB_F2P(100, 10, 10)
    }
#undef GB_F2P
    return nullptr;
}

void* f2_kernel_f32_b(int m, bool cols, int mode, int* m1, int* m2);
void* f2_kernel_f32_c(int m, bool cols, int mode, int* m1, int* m2);
void* f2_kernel_f32_d(int m, bool cols, int mode, int* m1, int* m2);
void* f2_kernel_f32_e(int m, bool cols, int mode, int* m1, int* m2);
void* f2_kernel_f32_f(int m, bool cols, int mode, int* m1, int* m2);
void* f2_kernel_f32_a_real(int m, bool cols, int mode, int* m1, int* m2);
void* f2_kernel_f32_b_real(int m, bool cols, int mode, int* m1, int* m2);
void* f2_kernel_f32_c_real(int m, bool cols, int mode, int* m1, int* m2);
void* f2_kernel_f32_d_real(int m, bool cols, int mode, int* m1, int* m2);
void* f2_kernel_f32_e_real(int m, bool cols, int mode, int* m1, int* m2);
void* f2_kernel_f32_f_real(int m, bool cols, int mode, int* m1, int* m2);
void* f2_xpose_kernel_f32_b(int m, int* m1, int* m2);
void* f2_pipe_kernel_f32_b(int m, int* m1, int* m2);
void* f2_pipe_kernel_f32_c(int m, int* m1, int* m2);
void* f2_pipe_kernel_f32_d(int m, int* m1, int* m2);
void* f2_pipe_kernel_f32_e(int m, int* m1, int* m2);
void* f2_pipe_kernel_f32_f(int m, int* m1, int* m2);
void* f2_xpose_kernel_f32_c(int m, int* m1, int* m2);
void* f2_xpose_kernel_f32_d(int m, int* m1, int* m2);
void* f2_xpose_kernel_f32_e(int m, int* m1, int* m2);
void* f2_xpose_kernel_f32_f(int m, int* m1, int* m2);

void* f2_kernel_f32(int m, bool cols, int mode, int* m1, int* m2) {
    typedef void* (*Fn)(int, bool, int, int*, int*);
    static const Fn units[12] = {f2_kernel_f32_a,      f2_kernel_f32_b,      f2_kernel_f32_c,
                                 f2_kernel_f32_d,      f2_kernel_f32_e,      f2_kernel_f32_f,
                                 f2_kernel_f32_a_real, f2_kernel_f32_b_real, f2_kernel_f32_c_real,
                                 f2_kernel_f32_d_real, f2_kernel_f32_e_real, f2_kernel_f32_f_real};
    int a = 0, b = 0;
    void* k = nullptr;
    for (int i = 0; i < 12 && !k; ++i) k = units[i](m, cols, mode, &a, &b);
    if (m1) *m1 = a;
    if (m2) *m2 = b;
    return k;
}

void* f2_xpose_kernel_f32(int m, int* m1, int* m2) {
    typedef void* (*Fn)(int, int*, int*);
    static const Fn units[6] = {f2_xpose_kernel_f32_a, f2_xpose_kernel_f32_b, f2_xpose_kernel_f32_c,
                                f2_xpose_kernel_f32_d, f2_xpose_kernel_f32_e, f2_xpose_kernel_f32_f};
    int a = 0, b = 0;
    void* k = nullptr;
    for (int i = 0; i < 6 && !k; ++i) k = units[i](m, &a, &b);
    if (m1) *m1 = a;
    if (m2) *m2 = b;
    return k;
}

void* f2_pipe_kernel_f32(int m, int* m1, int* m2) {
    typedef void* (*Fn)(int, int*, int*);
    static const Fn units[6] = {f2_pipe_kernel_f32_a, f2_pipe_kernel_f32_b, f2_pipe_kernel_f32_c,
                                f2_pipe_kernel_f32_d, f2_pipe_kernel_f32_e, f2_pipe_kernel_f32_f};
    int a = 0, b = 0;
    void* k = nullptr;
    for (int i = 0; i < 6 && !k; ++i) k = units[i](m, &a, &b);
    if (m1) *m1 = a;
    if (m2) *m2 = b;
    return k;
}

}  // namespace gb
