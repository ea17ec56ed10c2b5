/*
 * dtfft_gb300.h -- entry points of libdtfft_gb300.so beyond the public
 * dtfft.h ABI.
 *
 * 1. Kernel and executor plug-ins.  These are the two seams inside the
 *    reference where its Fortran plan code calls into device code; a
 *    Fortran build of dtFFT binds them with iso_c_binding interface blocks
 *    in place of its NVRTC kernels and its cuFFT / VkFFT executors.
 *
 * 2. Virtual-rank queries for plans whose communicator is a grid made by
 *    dtfft_vgrid_cart_create: where each rank's block sits in the one device
 *    buffer that holds all ranks.
 *
 * All functions return dtfft_error_t codes (dtfft.h).
 */
#ifndef DTFFT_GB300_H
#define DTFFT_GB300_H

#include "dtfft.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* Kernel plug-in                                                            */
/* Replaces kernel_device (src/dtfft_kernel_device.F90:61-178) behind        */
/* abstract_kernel%create/execute/destroy (src/dtfft_abstract_kernel.F90).   */
/* ------------------------------------------------------------------------ */

/** Kernel types, numbered as the reference's kernel_type_t
 * (src/dtfft_abstract_kernel.F90:61-97). */
typedef enum {
    GB_KERNEL_DUMMY = -1,
    GB_KERNEL_PACK = 1,
    GB_KERNEL_COPY_PIPELINED = 2,
    GB_KERNEL_UNPACK = 3,
    GB_KERNEL_COPY = 4,
    GB_KERNEL_UNPACK_PIPELINED = 5,
    GB_KERNEL_PACK_PIPELINED = 6,
    GB_KERNEL_PERMUTE_FORWARD = 7,
    GB_KERNEL_PERMUTE_BACKWARD = 8,
    GB_KERNEL_PERMUTE_BACKWARD_START = 9,
    GB_KERNEL_PERMUTE_BACKWARD_END = 10,
    GB_KERNEL_PERMUTE_BACKWARD_END_PIPELINED = 11
} gb_kernel_type_t;

typedef struct gb_kernel_s* gb_kernel_t;

/**
 * Creates a local data-movement kernel.
 * Reference: abstract_kernel%create(dims, effort, base_storage, kernel_type,
 * neighbor_data, force_effort), src/dtfft_abstract_kernel.F90:220-285.
 *
 * @param ndims          2 or 3
 * @param dims           local dims, fastest first
 * @param base_storage   element size in bytes: 4, 8 or 16
 * @param kernel_type    gb_kernel_type_t
 * @param neighbor_data  5 x n_neighbors ints {n1, n2, n3, in_displ, out_displ}
 *                       per neighbour (src/dtfft_reshape_handle_generic.F90:401-410),
 *                       NULL for the permute kernels
 * @param n_neighbors    number of neighbour columns
 * @param effort         dtfft_effort_t; DTFFT_EXHAUSTIVE times the tile candidates
 */
dtfft_error_t gb_kernel_create(int32_t ndims, const int32_t* dims, int32_t base_storage,
                               int32_t kernel_type, const int32_t* neighbor_data,
                               int32_t n_neighbors, int32_t effort, gb_kernel_t* kernel);

/**
 * Enqueues the kernel on `stream` (a cudaStream_t, NULL = legacy default).
 * Reference: abstract_kernel%execute(in, out, stream, neighbor),
 * src/dtfft_abstract_kernel.F90:287-330.  `neighbor` is 1-based for the
 * *_PIPELINED kernels and ignored otherwise.
 */
dtfft_error_t gb_kernel_execute(gb_kernel_t kernel, const void* in, void* out, void* stream, int32_t neighbor);

dtfft_error_t gb_kernel_destroy(gb_kernel_t* kernel);

/* ------------------------------------------------------------------------ */
/* FFT executor plug-in                                                      */
/* Replaces cufft_executor / vkfft_executor behind abstract_executor         */
/* (src/dtfft_abstract_executor.F90:47-112, create_private/execute_private). */
/* ------------------------------------------------------------------------ */

typedef enum { GB_FFT_C2C = 0, GB_FFT_R2C = 1, GB_FFT_R2R = 2 } gb_fft_type_t;
typedef enum { GB_FFT_FORWARD = -1, GB_FFT_BACKWARD = 1 } gb_fft_sign_t;

typedef struct gb_fft_s* gb_fft_t;

/**
 * Creates a batched FFT along contiguous data, with the arguments the
 * reference hands to its executors (src/dtfft_abstract_executor.F90:115-216):
 * fft_sizes/inembed/onembed in FFTW's slowest-first order, unit stride,
 * `idist`/`odist` between consecutive transforms.
 *
 * @param fft_rank    1 or 2
 * @param fft_type    gb_fft_type_t
 * @param precision   dtfft_precision_t
 * @param r2r_kinds   fft_rank kinds for GB_FFT_R2R (slowest first), else NULL
 * @param stream      cudaStream_t the transforms are enqueued on
 */
dtfft_error_t gb_fft_create(int32_t fft_rank, int32_t fft_type, int32_t precision, int32_t idist,
                            int32_t odist, int32_t how_many, const int32_t* fft_sizes,
                            const int32_t* inembed, const int32_t* onembed,
                            const int32_t* r2r_kinds, void* stream, gb_fft_t* fft);

/**
 * Runs the transform a -> b (a == b allowed except for R2C/C2R).
 * sign = GB_FFT_FORWARD: C2C forward, R2C, or R2R with the plan's kinds;
 * sign = GB_FFT_BACKWARD: C2C backward, C2R, or R2R with the inverse kinds.
 * Unnormalised, like FFTW.
 */
dtfft_error_t gb_fft_execute(gb_fft_t fft, void* a, void* b, int32_t sign);

dtfft_error_t gb_fft_destroy(gb_fft_t* fft);

/* ------------------------------------------------------------------------ */
/* Virtual ranks                                                             */
/* ------------------------------------------------------------------------ */

/** Number of virtual ranks of the plan's grid (1 for MPI_COMM_WORLD plans). */
dtfft_error_t dtfft_vgrid_get_nranks(dtfft_plan_t plan, int32_t* nranks);

/**
 * Pencil of virtual rank `vrank` in `layout` (what dtfft_get_pencil returns on
 * that rank of an MPI run) and the element offset of that rank's block in a
 * buffer holding `layout` for all ranks.  For R2C plans the X_PENCILS offset
 * counts real elements and the others complex elements.
 */
dtfft_error_t dtfft_vgrid_get_pencil(dtfft_plan_t plan, dtfft_layout_t layout, int32_t vrank,
                                     dtfft_pencil_t* pencil, size_t* offset);

/* ------------------------------------------------------------------------ */
/* Execute without allocating                                                */
/* ------------------------------------------------------------------------ */

/**
 * dtfft_execute for callers that cannot allocate device memory.  No
 * counterpart in the reference.
 *
 * dtfft_execute with aux = NULL allocates its scratch (dtfft_get_aux_bytes)
 * with cudaMalloc on the first call.  Callers whose device memory belongs to
 * another allocator (a framework's caching allocator, a fixed pool that
 * forbids raw cudaMalloc) or that cannot take a first-use allocation and its
 * possible device synchronisation use this entry point instead: it takes the
 * scratch from a fixed 16 MiB buffer compiled into the library
 * (dtfft_execute_noalloc_max_bytes) and calls no allocating routine.
 *
 * - Plans with dtfft_get_aux_bytes > 16 MiB are refused with
 *   DTFFT_ERROR_NOALLOC_SCRATCH_TOO_SMALL.
 * - The first call on a device looks the buffer's device address up
 *   (cudaGetSymbolAddress); make that first call before any stream capture.
 *   The lookup is repeated when the device's context has changed
 *   (cudaDeviceReset frees the buffer with the context; the next context
 *   holds a new one).  Plans do not survive a reset: create them again.
 * - Every call on a device shares the one buffer, which keeps what the last
 *   call left in it: calls whose kernels overlap on the GPU (different
 *   streams without ordering) race on it.
 * - Each GPU that loads this code holds the 16 MiB until the process exits.
 */
dtfft_error_t dtfft_execute_noalloc(dtfft_plan_t plan, void* in, void* out, dtfft_execute_t execute_type);

/** Size in bytes of the fixed scratch buffer of dtfft_execute_noalloc. */
size_t dtfft_execute_noalloc_max_bytes(void);

/* ------------------------------------------------------------------------ */
/* Batches of independent plans (no counterpart in the reference, whose      */
/* callers run one dtfft_execute per plan).                                  */
/* ------------------------------------------------------------------------ */
typedef struct gb_batch_s* dtfft_gb_batch_t;

/**
 * Groups `n` existing plans (any kinds, shapes, precisions and grids) so that
 * dtfft_gb_batch_execute runs all of them with one CUDA graph launch.  The
 * plans stay owned by the caller and must outlive the batch.  `lanes` (<= 0:
 * 8) is the number of graph branches the plans are spread over, so the
 * kernels of small transforms run side by side.
 */
dtfft_error_t dtfft_gb_batch_create(int32_t n, const dtfft_plan_t* plans, int32_t lanes, dtfft_gb_batch_t* batch);

/**
 * Same results as dtfft_execute(plans[i], ins[i], outs[i], execute_type,
 * auxs ? auxs[i] : NULL) for every i, launched as one graph on `stream`
 * (NULL: the legacy default stream).  The first call with a given set of
 * buffers checks them, allocates the plans' aux buffers where `auxs` gives
 * none and captures the graph (no other work may be captured on this thread
 * meanwhile); later calls with the same buffers and direction only launch it.
 * The batch keeps the graphs of its 4 most recently used buffer sets and
 * directions; other calls capture again.
 */
dtfft_error_t dtfft_gb_batch_execute(dtfft_gb_batch_t batch, void* const* ins, void* const* outs, void* const* auxs,
                                     dtfft_execute_t execute_type, void* stream);

/** Nodes of the graph the last dtfft_gb_batch_execute launched (0 before the first). */
dtfft_error_t dtfft_gb_batch_graph_nodes(dtfft_gb_batch_t batch, int64_t* nodes);

/** Waits for the device, destroys the graph and the batch; the plans stay. */
dtfft_error_t dtfft_gb_batch_destroy(dtfft_gb_batch_t* batch);

/**
 * Arithmetic form of the complex FP32 row FFT passes of plans created from now
 * on (no counterpart in the reference, whose FFTs come from cuFFT / VkFFT):
 *   0  FP32 Stockham kernels (default)
 *   1  tensor-core form: the row FFT of length 256, 512, 768 or 1024 runs as
 *      two DFT-matrix GEMM stages on tcgen05 with FP16 hi + lo operands
 *      (three products) accumulated in FP32, FP32 twiddles between the stages;
 *      other lengths, FP64 and real transforms keep the FP32 kernels.
 * The environment variable DTFFT_GB_FFT_FORM gives the initial value.
 * Returns DTFFT_ERROR_INVALID_USAGE for any other value.
 */
int32_t dtfft_gb_set_fft_form(int32_t form);
int32_t dtfft_gb_get_fft_form(void);

/** Number of launches of this library's kernels since load (for benchmarks). */
int64_t dtfft_gb_kernel_launch_count(void);

/**
 * Status of the bounded waits on the current device: 0 = fine, else the code
 * of a kernel that gave up waiting for its data (1 tile FFT kernels, 2
 * tensor-core form, 3 TMA transpose) after draining its own copies; that
 * launch's output is incomplete.  The word lives in pinned host memory, so
 * every public entry point (dtfft_execute, dtfft_execute_noalloc,
 * dtfft_transpose[_start], dtfft_reshape[_start], dtfft_gb_batch_execute,
 * gb_kernel_execute, gb_fft_execute) reads it without synchronising and, if
 * it is set, clears it and returns DTFFT_ERROR_GPU_WAIT_TIMEOUT before
 * launching anything: a timeout is reported by the first call after the
 * failed kernel has run.  This function synchronises the device first, so it
 * reports a timeout of any kernel enqueued before it; `reset` != 0 clears the
 * word afterwards.  -1 if the word could not be set up or the device failed.
 */
int32_t dtfft_gb_device_status(int32_t reset);

/**
 * Iteration limit of the waits of the tile FFT kernels and the TMA transpose
 * for their bulk copies, for kernels launched from now on (default 4194304,
 * well over a second).  0 makes every such wait give up at once: the kernels
 * then record status 1 or 3, wait (with the default bound) for the copies
 * they issued and return, which is how the failure path is tested.  Returns
 * DTFFT_ERROR_INVALID_USAGE for a negative value.
 */
int32_t dtfft_gb_set_wait_limit(int32_t iterations);

/* ------------------------------------------------------------------------ */
/* Kernel timing (for benchmarks)                                            */
/* Between start and stop every launch is bracketed by CUDA events on its    */
/* stream; durations are summed per kernel name.                             */
/* ------------------------------------------------------------------------ */
void dtfft_gb_profile_start(void);
void dtfft_gb_profile_stop(void);
int32_t dtfft_gb_profile_count(void);
int32_t dtfft_gb_profile_get(int32_t index, char* name, int32_t name_len, int64_t* launches, double* total_ms);

/**
 * Choices of the FFT step autotuner so far in this process (plans created with
 * DTFFT_EXHAUSTIVE or enable_kernel_autotune time every candidate kernel, tile
 * shape and radix schedule of each FFT step): a JSON array of
 * {"step", "chosen", "chosen_ms", "runner_up", "runner_up_ms", "candidates"}.
 * `len` receives the bytes needed (with the terminating zero); buf = NULL only
 * queries it.  DTFFT_ERROR_INVALID_USAGE when `cap` is too small.
 */
int32_t dtfft_gb_tune_records(char* buf, size_t cap, size_t* len);

/**
 * Measured FP64 FMA throughput of the current device in TFLOP/s (independent
 * FMA chains on every SM, best of 4 timed launches): the roofline of the
 * complex128 / float64 transforms, whose kernels are bound by the FP64 pipe.
 * Synchronises the device.
 */
int32_t dtfft_gb_measure_fp64_fma(double* tflops);

#ifdef __cplusplus
}
#endif
#endif /* DTFFT_GB300_H */
