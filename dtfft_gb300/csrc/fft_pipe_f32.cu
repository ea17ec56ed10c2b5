// Pipelined-kernel instantiations for single precision.
#include "fft_kernels.cuh"

namespace gb {

template <bool F>
static void* pipe_ptr(int m, int E) {
    if (E == ct_points_per_thread(m)) {
        switch (m) {
        case 8: return (void*)fft_pipe_kernel<float, CtSch<8, 8>, F>;
        case 16: return (void*)fft_pipe_kernel<float, CtSch<16, 16>, F>;
        case 32: return (void*)fft_pipe_kernel<float, CtSch<8, 8, 4>, F>;
        case 64: return (void*)fft_pipe_kernel<float, CtSch<8, 8, 8>, F>;
        case 128: return (void*)fft_pipe_kernel<float, CtSch<16, 16, 8>, F>;
        case 256: return (void*)fft_pipe_kernel<float, CtSch<16, 16, 16>, F>;
        case 512: return (void*)fft_pipe_kernel<float, CtSch<8, 8, 8, 8>, F>;
        case 1024: return (void*)fft_pipe_kernel<float, CtSch<16, 16, 8, 8>, F>;
        case 2048: return (void*)fft_pipe_kernel<float, CtSch<16, 16, 16, 8>, F>;
        case 4096: return (void*)fft_pipe_kernel<float, CtSch<16, 16, 16, 16>, F>;
        case 96: return (void*)fft_pipe_kernel<float, CtSch<24, 8, 4, 3>, F>;
        case 384: return (void*)fft_pipe_kernel<float, CtSch<24, 8, 8, 2, 3>, F>;
        case 768: return (void*)fft_pipe_kernel<float, CtSch<24, 8, 8, 4, 3>, F>;
        }
    }
    switch (E) {
    case 8: return (void*)fft_pipe_kernel<float, RtSch<8>, F>;
    case 16: return (void*)fft_pipe_kernel<float, RtSch<16>, F>;
    case 24: return (void*)fft_pipe_kernel<float, RtSch<24>, F>;
    case 20: return (void*)fft_pipe_kernel<float, RtSch<20>, F>;
    case 28: return (void*)fft_pipe_kernel<float, RtSch<28>, F>;
    }
    // plain rows only: the other points-per-thread counts of the register schedules
    if (!F) switch (E) {
    case 7: return (void*)fft_pipe_kernel<float, RtSch<7>, false>;
    case 9: return (void*)fft_pipe_kernel<float, RtSch<9>, false>;
    case 10: return (void*)fft_pipe_kernel<float, RtSch<10>, false>;
    case 12: return (void*)fft_pipe_kernel<float, RtSch<12>, false>;
    case 14: return (void*)fft_pipe_kernel<float, RtSch<14>, false>;
    case 15: return (void*)fft_pipe_kernel<float, RtSch<15>, false>;
    case 18: return (void*)fft_pipe_kernel<float, RtSch<18>, false>;
    case 21: return (void*)fft_pipe_kernel<float, RtSch<21>, false>;
    case 25: return (void*)fft_pipe_kernel<float, RtSch<25>, false>;
    case 30: return (void*)fft_pipe_kernel<float, RtSch<30>, false>;
    }
    return nullptr;
}

template <>
void* KPtr<float>::pipe(int m, int E, bool fused) {
    return fused ? pipe_ptr<true>(m, E) : pipe_ptr<false>(m, E);
}

}  // namespace gb
