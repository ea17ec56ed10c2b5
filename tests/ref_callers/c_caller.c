/*
 * A C program that uses dtFFT the way the reference's C integration tests do
 * (MPI_Init, dtfft_config_t, plan creation, local sizes, dtfft_mem_alloc,
 * forward execute, scaling, backward execute, the round-trip check, destroy),
 * built with a plain C compiler against include/dtfft.h, the single-process
 * mpi.h and libdtfft_gb300.so.  Four plans: C2C double 3D, R2C float 3D,
 * R2R double 3D (DCT-II / DST-III / DCT-IV) and a transpose-only C2C plan on a
 * 2 x 2 grid of virtual ranks whose X->Y->Z->Y->X transposes must return the
 * input bit for bit.  Exit status 0 and "Test PASSED!" per plan on success.
 *
 * Test infrastructure: tests/test_ref_callers_gpu.py builds and runs it.
 */
#include <mpi.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime.h>

#include "dtfft.h"
#include "helpers.h"

static void c2c_double(void) {
    int32_t dims[3] = {40, 48, 64};   /* dims[0] is the fastest axis, as in dtFFT's C API */
    dtfft_plan_t plan;
    DTFFT_CALL(dtfft_create_plan_c2c(3, dims, MPI_COMM_WORLD, DTFFT_DOUBLE, DTFFT_ESTIMATE, DTFFT_EXECUTOR_VKFFT, &plan))
    int32_t in_counts[3], out_counts[3];
    size_t alloc_size, alloc_bytes, aux_bytes, el;
    DTFFT_CALL(dtfft_get_local_sizes(plan, NULL, in_counts, NULL, out_counts, &alloc_size))
    DTFFT_CALL(dtfft_get_alloc_bytes(plan, &alloc_bytes))
    DTFFT_CALL(dtfft_get_aux_bytes(plan, &aux_bytes))
    DTFFT_CALL(dtfft_get_element_size(plan, &el))
    if (el != 16 || alloc_bytes != alloc_size * el) MPI_Abort(MPI_COMM_WORLD, 1);
    const size_t in_size = (size_t)in_counts[0] * in_counts[1] * in_counts[2];
    const size_t out_size = (size_t)out_counts[0] * out_counts[1] * out_counts[2];
    void *in, *out, *aux;
    DTFFT_CALL(dtfft_mem_alloc(plan, alloc_bytes, &in))
    DTFFT_CALL(dtfft_mem_alloc(plan, alloc_bytes, &out))
    DTFFT_CALL(dtfft_mem_alloc(plan, aux_bytes, &aux))
    double* check = (double*)malloc(16 * in_size);
    setTestValuesComplexDouble(check, in_size);
    complexDoubleH2D(check, in, in_size, DTFFT_PLATFORM_CUDA);
    double tf = -MPI_Wtime();
    DTFFT_CALL(dtfft_execute(plan, in, out, DTFFT_EXECUTE_FORWARD, aux))
    cudaDeviceSynchronize();
    tf += MPI_Wtime();
    scaleComplexDouble(DTFFT_EXECUTOR_VKFFT, out, out_size, (size_t)40 * 48 * 64, DTFFT_PLATFORM_CUDA, NULL);
    double tb = -MPI_Wtime();
    DTFFT_CALL(dtfft_execute(plan, out, in, DTFFT_EXECUTE_BACKWARD, aux))
    cudaDeviceSynchronize();
    tb += MPI_Wtime();
    checkAndReportComplexDouble((size_t)40 * 48 * 64, tf, tb, in, in_size, check, DTFFT_PLATFORM_CUDA);
    free(check);
    DTFFT_CALL(dtfft_mem_free(plan, in))
    DTFFT_CALL(dtfft_mem_free(plan, out))
    DTFFT_CALL(dtfft_mem_free(plan, aux))
    DTFFT_CALL(dtfft_destroy(&plan))
}

static void r2c_float(void) {
    int32_t dims[3] = {32, 64, 96};
    dtfft_plan_t plan;
    DTFFT_CALL(dtfft_create_plan_r2c(3, dims, MPI_COMM_WORLD, DTFFT_SINGLE, DTFFT_ESTIMATE, DTFFT_EXECUTOR_CUFFT, &plan))
    int32_t in_counts[3], out_counts[3];
    size_t alloc_bytes;
    DTFFT_CALL(dtfft_get_local_sizes(plan, NULL, in_counts, NULL, out_counts, NULL))
    DTFFT_CALL(dtfft_get_alloc_bytes(plan, &alloc_bytes))
    const size_t in_size = (size_t)in_counts[0] * in_counts[1] * in_counts[2];
    const size_t out_size = (size_t)out_counts[0] * out_counts[1] * out_counts[2];
    /* dims[0] is the fastest axis: the Fourier-space layout holds 32 / 2 + 1 points of it */
    if (out_counts[0] != 32 / 2 + 1 && out_counts[1] != 32 / 2 + 1 && out_counts[2] != 32 / 2 + 1)
        MPI_Abort(MPI_COMM_WORLD, 2);
    float *in, *out;
    cudaMallocManaged((void**)&in, alloc_bytes, cudaMemAttachGlobal);
    cudaMallocManaged((void**)&out, alloc_bytes, cudaMemAttachGlobal);
    float* check = (float*)malloc(4 * in_size);
    setTestValuesFloat(check, in_size);
    floatH2D(check, in, in_size, DTFFT_PLATFORM_CUDA);
    double tf = -MPI_Wtime();
    DTFFT_CALL(dtfft_execute(plan, in, out, DTFFT_EXECUTE_FORWARD, NULL))
    cudaDeviceSynchronize();
    tf += MPI_Wtime();
    scaleComplexFloat(DTFFT_EXECUTOR_CUFFT, out, out_size, (size_t)32 * 64 * 96, DTFFT_PLATFORM_CUDA, NULL);
    double tb = -MPI_Wtime();
    DTFFT_CALL(dtfft_execute(plan, out, in, DTFFT_EXECUTE_BACKWARD, NULL))
    cudaDeviceSynchronize();
    tb += MPI_Wtime();
    checkAndReportFloat((size_t)32 * 64 * 96, tf, tb, in, in_size, check, DTFFT_PLATFORM_CUDA);
    free(check);
    cudaFree(in);
    cudaFree(out);
    DTFFT_CALL(dtfft_destroy(&plan))
}

static void r2r_double(void) {
    int32_t dims[3] = {30, 36, 40};
    dtfft_r2r_kind_t kinds[3] = {DTFFT_DCT_2, DTFFT_DST_3, DTFFT_DCT_4};
    dtfft_plan_t plan;
    DTFFT_CALL(dtfft_create_plan_r2r(3, dims, kinds, MPI_COMM_WORLD, DTFFT_DOUBLE, DTFFT_ESTIMATE, DTFFT_EXECUTOR_VKFFT,
                                     &plan))
    int32_t in_counts[3], out_counts[3];
    size_t alloc_bytes;
    DTFFT_CALL(dtfft_get_local_sizes(plan, NULL, in_counts, NULL, out_counts, NULL))
    DTFFT_CALL(dtfft_get_alloc_bytes(plan, &alloc_bytes))
    const size_t in_size = (size_t)in_counts[0] * in_counts[1] * in_counts[2];
    const size_t out_size = (size_t)out_counts[0] * out_counts[1] * out_counts[2];
    double *in, *out;
    DTFFT_CALL(dtfft_mem_alloc(plan, alloc_bytes, (void**)&in))
    DTFFT_CALL(dtfft_mem_alloc(plan, alloc_bytes, (void**)&out))
    double* check = (double*)malloc(8 * in_size);
    setTestValuesDouble(check, in_size);
    doubleH2D(check, in, in_size, DTFFT_PLATFORM_CUDA);
    DTFFT_CALL(dtfft_execute(plan, in, out, DTFFT_EXECUTE_FORWARD, NULL))
    /* FFTW's round-trip factor of these kinds: 2n each */
    scaleDouble(DTFFT_EXECUTOR_VKFFT, out, out_size, (size_t)8 * 30 * 36 * 40, DTFFT_PLATFORM_CUDA, NULL);
    DTFFT_CALL(dtfft_execute(plan, out, in, DTFFT_EXECUTE_BACKWARD, NULL))
    cudaDeviceSynchronize();
    checkAndReportDouble((size_t)30 * 36 * 40, 0.0, 0.0, in, in_size, check, DTFFT_PLATFORM_CUDA);
    free(check);
    DTFFT_CALL(dtfft_mem_free(plan, in))
    DTFFT_CALL(dtfft_mem_free(plan, out))
    DTFFT_CALL(dtfft_destroy(&plan))
}

static void transposes_on_virtual_grid(void) {
    /* a 1 x 2 x 2 cartesian grid of virtual ranks in this one process */
    int cdims[3] = {1, 2, 2}, periods[3] = {0, 0, 0};
    MPI_Comm grid;
    if (MPI_Cart_create(MPI_COMM_WORLD, 3, cdims, periods, 0, &grid) != MPI_SUCCESS) MPI_Abort(MPI_COMM_WORLD, 3);
    int gsize = 0;
    MPI_Comm_size(grid, &gsize);
    if (gsize != 4) MPI_Abort(MPI_COMM_WORLD, 4);
    int32_t dims[3] = {24, 20, 36};
    dtfft_plan_t plan;
    DTFFT_CALL(dtfft_create_plan_c2c(3, dims, grid, DTFFT_SINGLE, DTFFT_ESTIMATE, DTFFT_EXECUTOR_NONE, &plan))
    const int32_t* gd;
    int8_t nd;
    DTFFT_CALL(dtfft_get_grid_dims(plan, &nd, &gd))
    if (nd != 3 || gd[0] != 1 || gd[1] != 2 || gd[2] != 2) MPI_Abort(MPI_COMM_WORLD, 5);
    size_t alloc_bytes, n;
    DTFFT_CALL(dtfft_get_alloc_bytes(plan, &alloc_bytes))
    n = alloc_bytes / 8;
    float *a, *b;
    cudaMallocManaged((void**)&a, alloc_bytes, cudaMemAttachGlobal);
    cudaMallocManaged((void**)&b, alloc_bytes, cudaMemAttachGlobal);
    float* check = (float*)malloc(alloc_bytes);
    setTestValuesComplexFloat(check, n);
    complexFloatH2D(check, a, n, DTFFT_PLATFORM_CUDA);
    DTFFT_CALL(dtfft_transpose(plan, a, b, DTFFT_TRANSPOSE_X_TO_Y, NULL))
    DTFFT_CALL(dtfft_transpose(plan, b, a, DTFFT_TRANSPOSE_Y_TO_Z, NULL))
    dtfft_request_t req;
    DTFFT_CALL(dtfft_transpose_start(plan, a, b, DTFFT_TRANSPOSE_Z_TO_Y, NULL, &req))
    DTFFT_CALL(dtfft_transpose_end(plan, req))
    DTFFT_CALL(dtfft_transpose(plan, b, a, DTFFT_TRANSPOSE_Y_TO_X, NULL))
    cudaDeviceSynchronize();
    /* the total of the packed blocks is the global size: compare the whole cycle bit for bit */
    const size_t total = (size_t)24 * 20 * 36;
    if (memcmp(a, check, total * 8) != 0) {
        fprintf(stderr, "transpose cycle changed the data\n");
        MPI_Abort(MPI_COMM_WORLD, 6);
    }
    printf("****************************************\n            Test PASSED!\n");
    printf("****************************************\n");
    free(check);
    cudaFree(a);
    cudaFree(b);
    DTFFT_CALL(dtfft_destroy(&plan))
    MPI_Comm_free(&grid);
}

int main(int argc, char* argv[]) {
    MPI_Init(&argc, &argv);
    int rank, size;
    MPI_Comm_rank(MPI_COMM_WORLD, &rank);
    MPI_Comm_size(MPI_COMM_WORLD, &size);
    if (rank != 0 || size != 1) MPI_Abort(MPI_COMM_WORLD, 7);
    attach_gpu_to_process();
    dtfft_config_t conf;
    DTFFT_CALL(dtfft_create_config(&conf))
    conf.platform = DTFFT_PLATFORM_CUDA;
    conf.enable_z_slab = true;
    DTFFT_CALL(dtfft_set_config(&conf))
    c2c_double();
    r2c_float();
    r2r_double();
    transposes_on_virtual_grid();
    MPI_Finalize();
    return 0;
}
