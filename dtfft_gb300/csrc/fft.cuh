// Batched FFT executor of the GB300 execute path (replaces the cuFFT / VkFFT
// executors of src/interfaces/fft/ behind src/dtfft_abstract_executor.F90).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "common.cuh"

namespace gb {

enum FftType { FFT_C2C = 0, FFT_R2C = 1, FFT_R2R = 2 };
enum { FFT_FWD = -1, FFT_BWD = 1 };  // src/include/_dtfft_private.h:27-28

// One batched transform of rank 1 or 2 over contiguous rows.
//  rank 1: `batch` signals of n_fast points, consecutive signals idist/odist
//          elements apart (elements of the input / output type).
//  rank 2: `batch` planes of n_slow x n_fast points (n_fast contiguous).
//  R2C: input real rows of n_fast, output complex rows of n_fast/2+1; the
//       backward direction is C2R.
struct FftDesc {
    int type = FFT_C2C;
    int dbl = 0;
    int rank = 1;
    int n_fast = 1, n_slow = 1;
    i64 batch = 0;
    i64 idist = 0, odist = 0;
    int kind_fast = 0, kind_slow = 0;  // dtfft_r2r_kind_t for FFT_R2R
};

// Radix schedule of one complex transform of length m (Stockham stages).
struct Schedule {
    int m = 1;
    std::vector<int> radix;
    std::string str() const;
};
bool make_schedule(int m, Schedule& s);

struct FftStep;  // one kernel launch of a plan

// Arithmetic form of the C2C FP32 row passes: 0 = FP32 Stockham kernels,
// 1 = tensor-core DFT-matrix GEMM stages with FP16 hi/lo operands (fft_tc.cu)
// for the row lengths that have one.  Read when a plan is built.
int fft_form();
bool tc_supported(int m);
dtfft_error_t tc_create(int m, void** out);
void tc_destroy(void* tc);
dtfft_error_t tc_execute(void* tc, const void* in, void* out, i64 nsig, int sign, int* status, cudaStream_t s);

// Bluestein form of a batched transform whose length has a prime factor
// above 127 (fft_bluestein.cu).  kind: 0 C2C, 1 real input (R2C, odd n),
// 2 Hermitian half input (C2R, odd n), 3 R2R: the length-m core of mode
// r2r_mode (M_DCT1 .. M_DST4) for r2r_n reals, with that mode's tables ta/tb.
// Geometry as in the kernels' steps: rows signal s at s*idist / s*odist, or
// columns (cols != 0) of planes.
dtfft_error_t blue_create(int dbl, int m, int sign, int kind, i64 nsig, i64 idist, i64 odist, i64 plane, int ld,
                          int ncols, int cols, void** out, int r2r_mode = 0, int r2r_n = 0,
                          const void* ta = nullptr, const void* tb = nullptr);
dtfft_error_t blue_execute(void* b, const void* in, void* out, cudaStream_t s);
void blue_destroy(void* b);

class FftPlan {
public:
    static dtfft_error_t create(const FftDesc& d, FftPlan** out);
    ~FftPlan();
    // in -> out; in == out allowed except for R2C / C2R.
    dtfft_error_t execute(const void* in, void* out, int sign, cudaStream_t s);
    const FftDesc& desc() const { return d_; }
    int launches_per_execute() const { return launches_; }
    // Measured choice of each step's kernel, tile shape and radix schedule
    // (EXHAUSTIVE plans); cached per GPU and step geometry.
    dtfft_error_t autotune(cudaStream_t s, int warmup, int iters, bool log);

private:
    FftDesc d_;
    std::vector<FftStep*> fwd_, bwd_;
    std::vector<void*> tables_;
    int launches_ = 0;
    dtfft_error_t build(int sign, std::vector<FftStep*>& steps);
    dtfft_error_t twiddles(int m, const void** table);
};

// Batched C2C along the source layout's aligned axis fused with the transpose
// described by a box list: one HBM pass instead of two.
class FusedFT {
public:
    // Fails (without side effects) when the boxes do not give every source
    // rank whole rows of the transform axis or the length has no register
    // schedule; with tile_only, also when neither the tile kernel nor the
    // two-factor kernel (float) can take the rows.
    static dtfft_error_t create(const BoxList& bl, int m, int dbl, bool tile_only, FusedFT** out);
    ~FusedFT();
    dtfft_error_t execute(const void* in, void* out, int sign, cudaStream_t s);
    // False when this pass cannot run on these buffers (the tile kernel's bulk
    // copies need 16-byte aligned rows); the caller then runs FFT + transpose.
    bool usable(const void* in, const void* out) const {
        return !tile_ || (((uintptr_t)in % 16) == 0 && ((uintptr_t)out % 16) == 0);
    }
    // Measured choice of the tile kernel's warp split (compute / store warps):
    // every compiled split is timed with CUDA events on scratch buffers of
    // max_elems elements and the fastest is kept; choices are cached per
    // (device, row length, precision, pass geometry) for the process.
    dtfft_error_t autotune(i64 max_elems, cudaStream_t s, int warmup, int iters, bool log);

private:
    int m_ = 0, dbl_ = 0, E_ = 0, T_ = 0, S_ = 1, pitch_ = 0, ngroups_ = 0;
    i64 ctas_ = 0;
    size_t smem_ = 0;
    size_t pipe_smem_ = 0;   // TMA-pipelined persistent variant (0 CTAs/SM = not used)
    int pipe_per_sm_ = 0;
    // warp-per-row tile kernel (fft_tile.cuh): used when tile_ is set
    bool tile_ = false;
    int tile_nst_ = 0, tile_threads_ = 0, pair_ok_ = 0, ncw_ = 0, nsw_ = 0;
    int wfast_ = 0;          // tile order of the pass: w first (1) or u first (0)
    const void* tw_bwd_ = nullptr;
    // tensor-store write-out of the tile pass (fft_tile_xpose_tma_kernel);
    // null when the pass's segments do not fit it or `use_xtma_` is off
    struct XTma* xtma_ = nullptr;
    bool use_xtma_ = false;
    // two-factor kernel fused with the transpose (fft_2f.cuh), tiles of S_ rows
    void* f2_ = nullptr;
    int f2_threads_ = 128;
    Schedule sched_;
    const void* tw_ = nullptr;
    const void* groups_ = nullptr;
    const void* segs_ = nullptr;
    std::vector<void*> owned_;
};

}  // namespace gb
