/*
 * mpi.h for single-process callers of libdtfft_gb300.
 *
 * Programs written for dtFFT include <mpi.h> and call a handful of MPI
 * functions around the dtFFT calls (init and finalize, their rank and size,
 * wall-clock timers, abort, and a cartesian communicator for the plan).  This
 * library runs every rank of a decomposition on one GPU in one process and
 * never calls MPI, so such a program can run unchanged without an MPI
 * library: put this directory first on the include path and it gets these
 * functions for one process.
 *
 *   MPI_Init / MPI_Finalize / MPI_Initialized / MPI_Finalized
 *   MPI_Comm_rank (always 0) / MPI_Comm_size (1 for MPI_COMM_WORLD and
 *     MPI_COMM_SELF, the grid's rank count for a cartesian handle)
 *   MPI_Wtime (wall clock, seconds)
 *   MPI_Abort (exits the process with the code, 1 when it is 0 or negative)
 *   MPI_Dims_create (balanced factorisation, as MPI defines it)
 *   MPI_Cart_create (a grid of virtual ranks: dtfft_vgrid_cart_create)
 *   MPI_Comm_free (releases such a grid)
 *
 * MPI_Comm and MPI_COMM_WORLD come from dtfft_mpi_shim.h, so dtfft.h and this
 * header may be included in either order.
 */
#ifndef DTFFT_SINGLE_PROCESS_MPI_H
#define DTFFT_SINGLE_PROCESS_MPI_H

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <time.h>

#include "dtfft_mpi_shim.h"

#ifdef __cplusplus
extern "C" {
#endif

#define MPI_SUCCESS 0
#define MPI_ERR_ARG 12
#define MPI_ERR_COMM 5

int32_t dtfft_vgrid_comm_size(MPI_Comm comm, int32_t* size);

static int dtfft_spmpi_state_ = 0;   /* 0 before init, 1 initialised, 2 finalised */

static inline int MPI_Init(int* argc, char*** argv) {
    (void)argc;
    (void)argv;
    dtfft_spmpi_state_ = 1;
    return MPI_SUCCESS;
}

static inline int MPI_Finalize(void) {
    dtfft_spmpi_state_ = 2;
    return MPI_SUCCESS;
}

static inline int MPI_Initialized(int* flag) {
    *flag = dtfft_spmpi_state_ >= 1;
    return MPI_SUCCESS;
}

static inline int MPI_Finalized(int* flag) {
    *flag = dtfft_spmpi_state_ == 2;
    return MPI_SUCCESS;
}

static inline int MPI_Comm_rank(MPI_Comm comm, int* rank) {
    (void)comm;
    *rank = 0;
    return MPI_SUCCESS;
}

static inline int MPI_Comm_size(MPI_Comm comm, int* size) {
    int32_t n = 1;
    if (comm != MPI_COMM_WORLD && comm != MPI_COMM_SELF && dtfft_vgrid_comm_size(comm, &n) != 0) return MPI_ERR_COMM;
    *size = (int)n;
    return MPI_SUCCESS;
}

static inline double MPI_Wtime(void) {
    struct timespec ts;
    timespec_get(&ts, TIME_UTC);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static inline int MPI_Abort(MPI_Comm comm, int errorcode) {
    (void)comm;
    fflush(stdout);
    fprintf(stderr, "MPI_Abort (single process): error code %d\n", errorcode);
    exit(errorcode > 0 ? errorcode : 1);
    return errorcode;
}

/* Fills the zero entries of dims with a factorisation of nnodes that is as
 * balanced as possible, in non-increasing order (MPI-4.0, section 8.5.2). */
static inline int MPI_Dims_create(int nnodes, int ndims, int dims[]) {
    int fixed = 1, nfree = 0;
    for (int i = 0; i < ndims; ++i) {
        if (dims[i] < 0) return MPI_ERR_ARG;
        if (dims[i] > 0) fixed *= dims[i]; else ++nfree;
    }
    if (fixed <= 0 || nnodes % fixed) return MPI_ERR_ARG;
    int rest = nnodes / fixed;
    if (nfree == 0) return rest == 1 ? MPI_SUCCESS : MPI_ERR_ARG;
    int f[64];
    for (int i = 0; i < nfree; ++i) f[i] = 1;
    /* largest prime factors first, each to the currently smallest entry */
    int primes[64], np = 0, r = rest;
    for (int p = 2; p * p <= r; ++p)
        while (r % p == 0) { primes[np++] = p; r /= p; }
    if (r > 1) primes[np++] = r;
    for (int k = np - 1; k >= 0; --k) {
        int m = 0;
        for (int i = 1; i < nfree; ++i) if (f[i] < f[m]) m = i;
        f[m] *= primes[k];
    }
    /* non-increasing order */
    for (int i = 0; i < nfree; ++i)
        for (int j = i + 1; j < nfree; ++j)
            if (f[j] > f[i]) { int t = f[i]; f[i] = f[j]; f[j] = t; }
    for (int i = 0, k = 0; i < ndims; ++i)
        if (dims[i] == 0) dims[i] = f[k++];
    return MPI_SUCCESS;
}

static inline int MPI_Cart_create(MPI_Comm comm_old, int ndims, const int dims[], const int periods[], int reorder,
                                  MPI_Comm* comm_cart) {
    (void)comm_old;
    (void)periods;
    (void)reorder;
    int32_t d[3] = {1, 1, 1};
    if (ndims < 1 || ndims > 3) return MPI_ERR_ARG;
    for (int i = 0; i < ndims; ++i) d[i] = (int32_t)dims[i];
    return dtfft_vgrid_cart_create((int32_t)ndims, d, comm_cart) == 0 ? MPI_SUCCESS : MPI_ERR_ARG;
}

static inline int MPI_Comm_free(MPI_Comm* comm) {
    if (*comm == MPI_COMM_WORLD || *comm == MPI_COMM_SELF) return MPI_ERR_COMM;
    return dtfft_vgrid_free(comm) == 0 ? MPI_SUCCESS : MPI_ERR_COMM;
}

#ifdef __cplusplus
}
#endif
#endif /* DTFFT_SINGLE_PROCESS_MPI_H */
