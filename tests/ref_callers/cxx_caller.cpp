/*
 * A C++ program that uses dtFFT's C++ interface (include/dtfft.hpp) the way
 * the reference's C++ integration tests do: dtfft::Config and set_config,
 * PlanR2R / PlanC2C / PlanR2C from dims and from a Pencil, get_local_sizes,
 * typed mem_alloc, forward / backward through the template overloads, the
 * round-trip check, and dtfft::Exception for a refused call.  Built with g++
 * against the include directory and libdtfft_gb300.so.
 *
 * Test infrastructure: tests/test_ref_callers_gpu.py builds and runs it.
 */
#include <mpi.h>

#include <complex>
#include <cstdio>
#include <iostream>
#include <vector>

#include <cuda_runtime.h>

#include "dtfft.hpp"
#include "helpers.h"

using namespace dtfft;

static void r2r_float_3d() {
    const std::vector<int32_t> dims = {20, 24, 32};   // dims[0] is the fastest axis
    const std::vector<R2RKind> kinds = {R2RKind::DCT_2, R2RKind::DST_2, R2RKind::DCT_3};
    PlanR2R plan(dims, kinds, MPI_COMM_WORLD, Precision::SINGLE, Effort::ESTIMATE, Executor::VKFFT);
    if (plan.get_precision() != Precision::SINGLE || plan.get_executor() != Executor::VKFFT) MPI_Abort(MPI_COMM_WORLD, 11);
    std::vector<int32_t> in_starts, in_counts, out_starts, out_counts;
    size_t alloc_size = 0;
    DTFFT_CXX_CALL(plan.get_local_sizes(in_starts, in_counts, out_starts, out_counts, &alloc_size))
    const size_t in_size = (size_t)in_counts[0] * in_counts[1] * in_counts[2];
    const size_t out_size = (size_t)out_counts[0] * out_counts[1] * out_counts[2];
    float* in = plan.mem_alloc<float>(alloc_size);
    float* out = plan.mem_alloc<float>(alloc_size);
    std::vector<float> check(in_size);
    setTestValuesFloat(check.data(), in_size);
    floatH2D(check.data(), in, in_size, static_cast<int32_t>(Platform::CUDA));
    double tf = -MPI_Wtime();
    DTFFT_CXX_CALL(plan.forward(in, out, nullptr))
    cudaDeviceSynchronize();
    tf += MPI_Wtime();
    scaleFloat(static_cast<int32_t>(Executor::VKFFT), out, out_size, (size_t)8 * 20 * 24 * 32,
               static_cast<int32_t>(Platform::CUDA), nullptr);
    double tb = -MPI_Wtime();
    DTFFT_CXX_CALL(plan.backward(out, in, nullptr))
    cudaDeviceSynchronize();
    tb += MPI_Wtime();
    checkAndReportFloat((size_t)20 * 24 * 32, tf, tb, in, in_size, check.data(), static_cast<int32_t>(Platform::CUDA));
    DTFFT_CXX_CALL(plan.mem_free(in))
    DTFFT_CXX_CALL(plan.mem_free(out))
}

static void c2c_double_2d_from_pencil() {
    // one process holds the whole domain: its pencil starts at zero
    const std::vector<int32_t> starts = {0, 0}, counts = {48, 40};
    Pencil pencil(starts, counts);
    PlanC2C plan(pencil, MPI_COMM_WORLD, Precision::DOUBLE, Effort::MEASURE, Executor::CUFFT);
    const Pencil px = plan.get_pencil(Layout::X_PENCILS);
    if (px.get_ndims() != 2 || px.get_dim() != 1 || px.get_size() != (size_t)48 * 40) MPI_Abort(MPI_COMM_WORLD, 12);
    const size_t n = plan.get_alloc_size();
    auto* in = plan.mem_alloc<std::complex<double>>(n);
    auto* out = plan.mem_alloc<std::complex<double>>(n);
    std::vector<std::complex<double>> check(n);
    setTestValuesComplexDouble(check.data(), n);
    complexDoubleH2D(check.data(), in, n, static_cast<int32_t>(Platform::CUDA));
    DTFFT_CXX_CALL(plan.execute(in, out, Execute::FORWARD))
    scaleComplexDouble(static_cast<int32_t>(Executor::CUFFT), out, n, (size_t)48 * 40,
                       static_cast<int32_t>(Platform::CUDA), nullptr);
    DTFFT_CXX_CALL(plan.execute(out, in, Execute::BACKWARD))
    cudaDeviceSynchronize();
    checkAndReportComplexDouble((size_t)48 * 40, 0.0, 0.0, in, n, check.data(), static_cast<int32_t>(Platform::CUDA));
    // a refused call throws with the C error code
    bool thrown = false;
    try {
        plan.transpose_start(in, out, Transpose::Y_TO_Z);
    } catch (const Exception& e) {
        thrown = e.get_error_code() == Error::INVALID_TRANSPOSE_TYPE;
    }
    if (!thrown) MPI_Abort(MPI_COMM_WORLD, 13);
    DTFFT_CXX_CALL(plan.mem_free(in))
    DTFFT_CXX_CALL(plan.mem_free(out))
}

static void r2c_float_inplace_grid() {
    // a 2 x 2 cartesian grid of virtual ranks
    int cdims[2] = {0, 0};
    const int periods[2] = {0, 0};
    MPI_Dims_create(1, 2, cdims);
    MPI_Comm grid;
    MPI_Cart_create(MPI_COMM_WORLD, 2, cdims, periods, 1, &grid);
    PlanR2C plan({16, 24, 64}, grid, Precision::SINGLE, Effort::ESTIMATE, Executor::CUFFT);
    const size_t n = plan.get_alloc_size();
    float* in = plan.mem_alloc<float>(n);
    auto* out = plan.mem_alloc<std::complex<float>>(n / 2);
    int32_t in_counts[3];
    DTFFT_CXX_CALL(plan.get_local_sizes(nullptr, in_counts, nullptr, nullptr, nullptr))
    const size_t in_size = (size_t)in_counts[0] * in_counts[1] * in_counts[2];
    std::vector<float> check(in_size);
    setTestValuesFloat(check.data(), in_size);
    floatH2D(check.data(), in, in_size, static_cast<int32_t>(Platform::CUDA));
    DTFFT_CXX_CALL(plan.forward(in, out, nullptr))
    DTFFT_CXX_CALL(plan.backward(out, in, nullptr))
    cudaDeviceSynchronize();
    // unnormalised round trip: scale the real result
    scaleFloat(static_cast<int32_t>(Executor::CUFFT), in, in_size, (size_t)16 * 24 * 64,
               static_cast<int32_t>(Platform::CUDA), nullptr);
    checkAndReportFloat((size_t)16 * 24 * 64, 0.0, 0.0, in, in_size, check.data(), static_cast<int32_t>(Platform::CUDA));
    DTFFT_CXX_CALL(plan.mem_free(in))
    DTFFT_CXX_CALL(plan.mem_free(out))
    MPI_Comm_free(&grid);
}

int main(int argc, char* argv[]) {
    MPI_Init(&argc, &argv);
    attach_gpu_to_process();
    try {
        Config conf;
        conf.set_platform(Platform::CUDA).set_enable_z_slab(true);
        DTFFT_CXX_CALL(set_config(conf))
        if (Version::get() != Version::CODE) MPI_Abort(MPI_COMM_WORLD, 10);
        r2r_float_3d();
        c2c_double_2d_from_pencil();
        r2c_float_inplace_grid();
    } catch (const Exception& e) {
        std::cerr << e.what() << std::endl;
        MPI_Abort(MPI_COMM_WORLD, 1);
    }
    MPI_Finalize();
    return 0;
}
