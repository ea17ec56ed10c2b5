/*
 * dtfft_mpi_shim.h -- the MPI names dtfft.h needs, for a library that runs
 * every rank of a decomposition on one GPU.
 *
 * dtFFT's C ABI takes an `MPI_Comm` (include/dtfft.h:397-515 of the
 * reference).  This library is a single process: it never calls MPI, so a
 * communicator is only a handle that names a decomposition grid.
 *
 *   MPI_COMM_WORLD            one process, the grid is chosen by the planner
 *   dtfft_vgrid_cart_create   a cartesian grid of virtual ranks, the way
 *                             MPI_Cart_create(MPI_COMM_WORLD, ndims, dims, ...)
 *                             would build it for prod(dims) processes
 *
 * Handles follow the MPICH ABI (MPI_Comm is a 32-bit int), which is also what
 * the reference's Fortran layer receives (MPI_Comm_c2f, dtfft_api_c.c:42).
 * Define DTFFT_HAVE_REAL_MPI and include <mpi.h> first to use a real MPI's
 * MPI_Comm type instead; handles are then compared by value only.
 */
#ifndef DTFFT_MPI_SHIM_H
#define DTFFT_MPI_SHIM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifndef DTFFT_HAVE_REAL_MPI
typedef int MPI_Comm;
#ifndef MPI_COMM_WORLD
#define MPI_COMM_WORLD ((MPI_Comm)0x44000000)
#endif
#ifndef MPI_COMM_SELF
#define MPI_COMM_SELF ((MPI_Comm)0x44000001)
#endif
#endif

/**
 * Creates a handle for a cartesian grid of virtual ranks.
 *
 * @param[in]  ndims  number of grid dimensions (1, 2 or 3)
 * @param[in]  dims   grid sizes in the order MPI_Cart_create takes them;
 *                    when ndims equals the plan's rank, dims[0] describes the
 *                    fastest (X) axis and must be 1 for a plan (dtFFT's rule)
 * @param[out] comm   handle to pass to dtfft_create_plan_*
 * @return 0 on success, DTFFT_ERROR_INVALID_COMM_DIMS-like code otherwise
 *
 * Virtual rank r has cartesian coordinates in row-major order, exactly as
 * MPI numbers the ranks of a cartesian communicator.
 */
int32_t dtfft_vgrid_cart_create(int32_t ndims, const int32_t* dims, MPI_Comm* comm);

/**
 * Creates a handle for `nprocs` virtual ranks without a topology, the way
 * MPI_COMM_WORLD of an `nprocs`-process run looks to the planner: the plan
 * then chooses the grid itself (Z-slab, Y-slab or a balanced P1 x P2 grid)
 * by the reference's rules.
 */
int32_t dtfft_vgrid_world_create(int32_t nprocs, MPI_Comm* comm);

/**
 * Creates a handle for `nprocs` virtual ranks without a topology, each owning
 * its own block of the global domain: what `nprocs` MPI processes that each
 * pass their dtfft_pencil_t to dtfft_create_plan_*_pencil describe together
 * (dtfft_plan.F90:2014-2089 and dtfft_pencil.F90:777-908 of the reference).
 *
 * @param[in]  nprocs  number of virtual ranks
 * @param[in]  ndims   2 or 3
 * @param[in]  starts  nprocs x ndims block starts, rank-major, in the order of
 *                     dtfft_pencil_t::starts (dims[0] is the fastest axis)
 * @param[in]  counts  nprocs x ndims block counts, same order
 * @param[out] comm    handle to pass to dtfft_create_plan_*_pencil together
 *                     with virtual rank 0's block
 *
 * The blocks are checked when the plan is created, with the reference's error
 * codes (DTFFT_ERROR_PENCIL_*).  Blocks that split the fastest axis are bricks:
 * the plan then provides dtfft_reshape between them and X pencils, and
 * dtfft_execute starts from (and returns to) the bricks.  Virtual rank r's
 * block of any layout sits at the offset dtfft_vgrid_get_pencil reports.
 */
int32_t dtfft_vgrid_pencils_create(int32_t nprocs, int32_t ndims, const int32_t* starts, const int32_t* counts,
                                   MPI_Comm* comm);

/**
 * Number of virtual ranks a handle stands for: 1 for MPI_COMM_WORLD and
 * MPI_COMM_SELF, prod(dims) for a cartesian grid, `nprocs` for the others.
 * DTFFT_ERROR_INVALID_COMM_TYPE for an unknown handle.
 */
int32_t dtfft_vgrid_comm_size(MPI_Comm comm, int32_t* size);

/** Releases a handle made by dtfft_vgrid_cart_create or dtfft_vgrid_world_create. */
int32_t dtfft_vgrid_free(MPI_Comm* comm);

#ifdef __cplusplus
}
#endif
#endif /* DTFFT_MPI_SHIM_H */
