/*
 * Helpers that dtFFT's C and C++ integration programs call around the dtFFT
 * calls: test values, host->device copies, scaling of unnormalised results,
 * the round-trip check and its report, the GPU choice and a block of a
 * cartesian split.  The reference declares them in tests/c/test_utils.h and
 * implements them in Fortran (tests/test_utils.F90, with
 * tests/include/{h2d,scale,check_and_report}.inc); this is a C implementation
 * of the same interface for one process on one GPU, so those programs link
 * against libdtfft_gb300 without the reference's Fortran test library.
 *
 * Test infrastructure: only tests/ builds it.
 */
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "dtfft.h"
#include "mpi.h"

/* uniform [0, 1) values from a fixed-seed xorshift generator (the reference
 * draws them with Fortran's random_number) */
static uint64_t g_rng = 0x2545F4914F6CDD1DULL;

static double next_uniform(void) {
    g_rng ^= g_rng << 13;
    g_rng ^= g_rng >> 7;
    g_rng ^= g_rng << 17;
    return (double)(g_rng >> 11) * (1.0 / 9007199254740992.0);
}

void setTestValuesDouble(void* buf, size_t n) {
    double* b = (double*)buf;
    for (size_t i = 0; i < n; ++i) b[i] = next_uniform();
}

void setTestValuesFloat(void* buf, size_t n) {
    float* b = (float*)buf;
    for (size_t i = 0; i < n; ++i) b[i] = (float)next_uniform();
}

void setTestValuesComplexDouble(void* buf, size_t n) { setTestValuesDouble(buf, 2 * n); }
void setTestValuesComplexFloat(void* buf, size_t n) { setTestValuesFloat(buf, 2 * n); }

/* Block of this process in a balanced cartesian split of `dims` (fastest
 * first); the last coordinate of each axis takes the remainder. */
void createGridDims(int32_t ndims, int32_t* dims, int32_t* grid, int32_t* starts, int32_t* counts) {
    int size = 1, rank = 0;
    MPI_Comm_size(MPI_COMM_WORLD, &size);
    MPI_Comm_rank(MPI_COMM_WORLD, &rank);
    int g[3] = {0, 0, 0};
    for (int i = 0; i < ndims; ++i) g[i] = grid[i];
    MPI_Dims_create(size, ndims, g);
    int r = rank;
    for (int i = 0; i < ndims; ++i) {
        grid[i] = g[i];
        const int coord = r % g[i];
        r /= g[i];
        counts[i] = dims[i] / g[i];
        starts[i] = coord * counts[i];
        if (coord == g[i] - 1) counts[i] += dims[i] % g[i];
    }
}

void attach_gpu_to_process(void) {
    const char* env = getenv("DTFFT_PLATFORM");
    if (env && strcmp(env, "host") == 0) return;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) { cudaGetLastError(); return; }
    cudaSetDevice(0);
}

static void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        fprintf(stderr, "Cuda error in %s : %s.\n", what, cudaGetErrorString(e));
        MPI_Abort(MPI_COMM_WORLD, (int)e);
    }
}

/* ---- host -> device copies ---- */
static void h2d(void* src, void* dst, size_t bytes, int32_t platform) {
    if (platform == DTFFT_PLATFORM_CUDA) cuda_check(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice), "h2d");
    else memcpy(dst, src, bytes);
}
void complexDoubleH2D(void* s, void* d, size_t n, int32_t p) { h2d(s, d, n * 16, p); }
void complexFloatH2D(void* s, void* d, size_t n, int32_t p) { h2d(s, d, n * 8, p); }
void doubleH2D(void* s, void* d, size_t n, int32_t p) { h2d(s, d, n * 8, p); }
void floatH2D(void* s, void* d, size_t n, int32_t p) { h2d(s, d, n * 4, p); }

/* ---- scaling of unnormalised results; transpose-only plans are not scaled ---- */
static void scale(int32_t executor, void* buf, size_t nreal, size_t by, int32_t platform, int single) {
    if (executor == DTFFT_EXECUTOR_NONE) return;
    const size_t bytes = nreal * (single ? 4 : 8);
    void* h = buf;
    int copy = 0;
    if (platform == DTFFT_PLATFORM_CUDA) {
        cuda_check(cudaDeviceSynchronize(), "scale");
        struct cudaPointerAttributes at;
        cuda_check(cudaPointerGetAttributes(&at, buf), "scale");
        if (at.type == cudaMemoryTypeDevice) {   /* plain device memory: scale a host copy */
            h = malloc(bytes);
            cuda_check(cudaMemcpy(h, buf, bytes, cudaMemcpyDeviceToHost), "scale");
            copy = 1;
        }
    }
    if (single) {
        float* b = (float*)h;
        for (size_t i = 0; i < nreal; ++i) b[i] /= (float)by;
    } else {
        double* b = (double*)h;
        for (size_t i = 0; i < nreal; ++i) b[i] /= (double)by;
    }
    if (copy) {
        cuda_check(cudaMemcpy(buf, h, bytes, cudaMemcpyHostToDevice), "scale");
        free(h);
    }
}
void scaleComplexDouble(int32_t e, void* b, size_t n, size_t s, int32_t p, dtfft_stream_t st) { (void)st; scale(e, b, 2 * n, s, p, 0); }
void scaleComplexFloat(int32_t e, void* b, size_t n, size_t s, int32_t p, dtfft_stream_t st) { (void)st; scale(e, b, 2 * n, s, p, 1); }
void scaleDouble(int32_t e, void* b, size_t n, size_t s, int32_t p, dtfft_stream_t st) { (void)st; scale(e, b, n, s, p, 0); }
void scaleFloat(int32_t e, void* b, size_t n, size_t s, int32_t p, dtfft_stream_t st) { (void)st; scale(e, b, n, s, p, 1); }

/* ---- round-trip check: max |check - result| against 5 log2(N) eps ---- */
static void check_and_report(size_t n_global, double tf, double tb, void* buf, size_t nreal, void* check,
                             int32_t platform, int single) {
    const size_t bytes = nreal * (single ? 4 : 8);
    void* h = buf;
    if (platform == DTFFT_PLATFORM_CUDA) {
        h = malloc(bytes);
        cuda_check(cudaMemcpy(h, buf, bytes, cudaMemcpyDefault), "check");
    }
    double err = 0.0;
    for (size_t i = 0; i < nreal; ++i) {
        const double d = single ? fabs((double)((float*)check)[i] - (double)((float*)h)[i])
                                : fabs(((double*)check)[i] - ((double*)h)[i]);
        if (single && d > 1e-3) {
            fprintf(stderr, "i = %zu: %g vs %g\n", i + 1, (double)((float*)check)[i], (double)((float*)h)[i]);
            MPI_Abort(MPI_COMM_WORLD, -1);
        }
        if (d > err || d != d) err = d;
    }
    if (h != buf) free(h);
    /* spacing of the numbers around 1: nearest(1, 1) - nearest(1, -1) */
    const double eps = single ? 1.5 * 1.1920928955078125e-07 : 1.5 * 2.220446049250313e-16;
    const double thr = 5.0 * log((double)n_global) / log(2.0) * eps;
    printf("****************************************\n");
    if (err <= thr && err >= 0.0) {
        printf("            Test PASSED!\n");
    } else {
        printf("Test FAILED... error = %16.5e threshold = %16.5e\n", err, thr);
        MPI_Abort(MPI_COMM_WORLD, -1);
    }
    printf("****************************************\n");
    printf("Forward execution time\n  max: %g [s]\n", tf);
    printf("----------------------------------------\n");
    printf("Backward execution time\n  max: %g [s]\n", tb);
    printf("****************************************\n");
}
void checkAndReportComplexDouble(size_t n, double tf, double tb, void* b, size_t c, void* k, int32_t p) { check_and_report(n, tf, tb, b, 2 * c, k, p, 0); }
void checkAndReportComplexFloat(size_t n, double tf, double tb, void* b, size_t c, void* k, int32_t p) { check_and_report(n, tf, tb, b, 2 * c, k, p, 1); }
void checkAndReportDouble(size_t n, double tf, double tb, void* b, size_t c, void* k, int32_t p) { check_and_report(n, tf, tb, b, c, k, p, 0); }
void checkAndReportFloat(size_t n, double tf, double tb, void* b, size_t c, void* k, int32_t p) { check_and_report(n, tf, tb, b, c, k, p, 1); }
