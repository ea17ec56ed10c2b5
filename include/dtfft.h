/*
 * dtfft.h -- C ABI of the GB300 execute path of dtFFT.
 *
 * Drop-in for the reference's public C header (include/dtfft.h of dtFFT
 * v3.2.0): every function below has the reference's name, argument list and
 * meaning, and every enum the reference's numeric value
 * (include/dtfft_config.h.in:35-186), so a program written against the
 * reference recompiles against this header and links to libdtfft_gb300.so.
 *
 * What differs, by design:
 *   - The only platform is CUDA (one GB300).  DTFFT_PLATFORM_HOST plans are
 *     rejected with DTFFT_ERROR_INVALID_PLATFORM.
 *   - A decomposition of P processes runs as P virtual ranks on one GPU; the
 *     ranks' local blocks sit one after another in one device buffer, in
 *     cartesian rank order (see dtfft_gb300.h for per-rank offsets).  Make the
 *     grid with dtfft_vgrid_cart_create (dtfft_mpi_shim.h).
 *   - FFTs run on this library's own kernels.  DTFFT_EXECUTOR_CUFFT and
 *     DTFFT_EXECUTOR_VKFFT both select them; like the reference, R2R plans
 *     are refused for CUFFT (DTFFT_ERROR_R2R_FFT_NOT_SUPPORTED) and accepted
 *     for VKFFT.  FFTW3 / MKL are host executors and are refused.
 */
#ifndef DTFFT_H
#define DTFFT_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>

#include "dtfft_mpi_shim.h"

/* What the reference's generated dtfft_config.h defines for a CUDA build with
 * both GPU executors: both executor names select this library's kernels. */
#ifndef DTFFT_WITH_CUDA
#define DTFFT_WITH_CUDA
#endif
#ifndef DTFFT_WITH_CUFFT
#define DTFFT_WITH_CUFFT
#endif
#ifndef DTFFT_WITH_VKFFT
#define DTFFT_WITH_VKFFT
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define DTFFT_VERSION_MAJOR 3
#define DTFFT_VERSION_MINOR 2
#define DTFFT_VERSION_PATCH 0
#define DTFFT_VERSION(X, Y, Z) ((X) * 100000 + (Y) * 1000 + (Z))
#define DTFFT_VERSION_CODE DTFFT_VERSION(DTFFT_VERSION_MAJOR, DTFFT_VERSION_MINOR, DTFFT_VERSION_PATCH)

/** Library version code (reference: include/dtfft.h:52). */
int32_t dtfft_get_version(void);

/** Error codes (reference: include/dtfft.h:78-215, values from dtfft_config.h.in:84-145). */
typedef enum {
    DTFFT_SUCCESS = 0,
    DTFFT_ERROR_MPI_FINALIZED = -1,
    DTFFT_ERROR_PLAN_NOT_CREATED = 1,
    DTFFT_ERROR_INVALID_TRANSPOSE_TYPE = 2,
    DTFFT_ERROR_INVALID_N_DIMENSIONS = 3,
    DTFFT_ERROR_INVALID_DIMENSION_SIZE = 4,
    DTFFT_ERROR_INVALID_COMM_TYPE = 5,
    DTFFT_ERROR_INVALID_PRECISION = 6,
    DTFFT_ERROR_INVALID_EFFORT = 7,
    DTFFT_ERROR_INVALID_EXECUTOR = 8,
    DTFFT_ERROR_INVALID_COMM_DIMS = 9,
    DTFFT_ERROR_INVALID_COMM_FAST_DIM = 10,
    DTFFT_ERROR_MISSING_R2R_KINDS = 11,
    DTFFT_ERROR_INVALID_R2R_KINDS = 12,
    DTFFT_ERROR_R2C_TRANSPOSE_PLAN = 13,
    DTFFT_ERROR_INPLACE_TRANSPOSE = 14,
    DTFFT_ERROR_INVALID_AUX = 15,
    DTFFT_ERROR_INVALID_LAYOUT = 16,
    DTFFT_ERROR_INVALID_USAGE = 17,
    DTFFT_ERROR_PLAN_IS_CREATED = 18,
    DTFFT_ERROR_ALLOC_FAILED = 19,
    DTFFT_ERROR_FREE_FAILED = 20,
    DTFFT_ERROR_INVALID_ALLOC_BYTES = 21,
    DTFFT_ERROR_DLOPEN_FAILED = 22,
    DTFFT_ERROR_DLSYM_FAILED = 23,
    DTFFT_ERROR_PENCIL_ARRAYS_SIZE_MISMATCH = 25,
    DTFFT_ERROR_PENCIL_ARRAYS_INVALID_SIZES = 26,
    DTFFT_ERROR_PENCIL_INVALID_COUNTS = 27,
    DTFFT_ERROR_PENCIL_INVALID_STARTS = 28,
    DTFFT_ERROR_PENCIL_SHAPE_MISMATCH = 29,
    DTFFT_ERROR_PENCIL_OVERLAP = 30,
    DTFFT_ERROR_PENCIL_NOT_CONTINUOUS = 31,
    DTFFT_ERROR_PENCIL_NOT_INITIALIZED = 32,
    DTFFT_ERROR_INVALID_MEASURE_WARMUP_ITERS = 33,
    DTFFT_ERROR_INVALID_MEASURE_ITERS = 34,
    DTFFT_ERROR_INVALID_REQUEST = 35,
    DTFFT_ERROR_TRANSPOSE_ACTIVE = 36,
    DTFFT_ERROR_TRANSPOSE_NOT_ACTIVE = 37,
    DTFFT_ERROR_INVALID_RESHAPE_TYPE = 38,
    DTFFT_ERROR_RESHAPE_ACTIVE = 39,
    DTFFT_ERROR_RESHAPE_NOT_ACTIVE = 40,
    DTFFT_ERROR_INPLACE_RESHAPE = 41,
    DTFFT_ERROR_INVALID_EXECUTE_TYPE = 43,
    DTFFT_ERROR_RESHAPE_NOT_SUPPORTED = 44,
    DTFFT_ERROR_R2C_EXECUTE_CALLED = 45,
    DTFFT_ERROR_INVALID_CART_COMM = 46,
    DTFFT_ERROR_INVALID_TRANSPOSE_MODE = 47,
    DTFFT_ERROR_INVALID_ACCESS_MODE = 48,
    DTFFT_ERROR_R2R_FFT_NOT_SUPPORTED = 101,
    DTFFT_ERROR_GPU_INVALID_STREAM = 201,
    DTFFT_ERROR_INVALID_BACKEND = 202,
    DTFFT_ERROR_GPU_NOT_SET = 203,
    DTFFT_ERROR_VKFFT_R2R_2D_PLAN = 204,
    DTFFT_ERROR_BACKENDS_DISABLED = 205,
    DTFFT_ERROR_NOT_DEVICE_PTR = 300,
    DTFFT_ERROR_NOT_NVSHMEM_PTR = 301,
    DTFFT_ERROR_INVALID_PLATFORM = 400,
    DTFFT_ERROR_INVALID_PLATFORM_EXECUTOR = 401,
    DTFFT_ERROR_INVALID_PLATFORM_BACKEND = 402,
    DTFFT_ERROR_COMPRESSION_CUDA_NOT_SUPPORTED = 500,
    DTFFT_ERROR_COMPRESSION_INVALID_RATE = 501,
    DTFFT_ERROR_COMPRESSION_INVALID_PRECISION = 502,
    DTFFT_ERROR_COMPRESSION_INVALID_TOLERANCE = 503,
    DTFFT_ERROR_COMPRESSION_INVALID_MODE = 504,
    DTFFT_ERROR_COMPRESSION_INVALID_LIBRARY = 505,
    DTFFT_ERROR_COMPRESSION_NOT_USED = 506,
    /* Library-specific: a CUDA call failed; the plan stays usable. */
    DTFFT_ERROR_GPU_CALL_FAILED = 600,
    /* Library-specific: a transform size this library's FFT kernels cannot run. */
    DTFFT_ERROR_FFT_SIZE_NOT_SUPPORTED = 601,
    /* Library-specific: the plan needs more scratch than the fixed buffer of
     * dtfft_execute_noalloc holds (dtfft_gb300.h). */
    DTFFT_ERROR_NOALLOC_SCRATCH_TOO_SMALL = 602,
    /* Library-specific: a kernel launched by an earlier call on this device
     * gave up a bounded wait and left its output incomplete (reported once,
     * by the next call on the device; dtfft_gb300.h). */
    DTFFT_ERROR_GPU_WAIT_TIMEOUT = 603
} dtfft_error_t;

/** Prints the failing call and aborts (reference: include/dtfft.h:62-70, which calls MPI_Abort). */
#define DTFFT_CALL(call)                                                     \
    do {                                                                     \
        dtfft_error_t ierr_ = (call);                                        \
        if (ierr_ != DTFFT_SUCCESS) {                                        \
            fprintf(stderr, "dtFFT error in file '%s:%i': %s.\n", __FILE__,  \
                    __LINE__, dtfft_get_error_string(ierr_));                \
            abort();                                                         \
        }                                                                    \
    } while (0);

typedef enum { DTFFT_EXECUTE_FORWARD = 11, DTFFT_EXECUTE_BACKWARD = 12 } dtfft_execute_t;

typedef enum {
    DTFFT_TRANSPOSE_X_TO_Y = 1,
    DTFFT_TRANSPOSE_Y_TO_X = -1,
    DTFFT_TRANSPOSE_Y_TO_Z = 2,
    DTFFT_TRANSPOSE_Z_TO_Y = -2,
    DTFFT_TRANSPOSE_X_TO_Z = 3,
    DTFFT_TRANSPOSE_Z_TO_X = -3
} dtfft_transpose_t;

typedef enum {
    DTFFT_RESHAPE_X_BRICKS_TO_PENCILS = 11,
    DTFFT_RESHAPE_X_PENCILS_TO_BRICKS = 12,
    DTFFT_RESHAPE_Z_PENCILS_TO_BRICKS = 13,
    DTFFT_RESHAPE_Z_BRICKS_TO_PENCILS = 14,
    DTFFT_RESHAPE_Y_BRICKS_TO_PENCILS = 14,
    DTFFT_RESHAPE_Y_PENCILS_TO_BRICKS = 13
} dtfft_reshape_t;

typedef enum { DTFFT_SINGLE = 0, DTFFT_DOUBLE = 1 } dtfft_precision_t;

typedef enum { DTFFT_ESTIMATE = 0, DTFFT_MEASURE = 1, DTFFT_PATIENT = 2, DTFFT_EXHAUSTIVE = 3 } dtfft_effort_t;

typedef enum {
    DTFFT_EXECUTOR_NONE = 0,
    DTFFT_EXECUTOR_FFTW3 = 1,
    DTFFT_EXECUTOR_MKL = 2,
    DTFFT_EXECUTOR_CUFFT = 3,
    DTFFT_EXECUTOR_VKFFT = 4
} dtfft_executor_t;

/** R2R kinds: FFTW's REDFT00..RODFT11 numbering (reference include/dtfft.h:310-336). */
typedef enum {
    DTFFT_DCT_1 = 3,
    DTFFT_DCT_2 = 5,
    DTFFT_DCT_3 = 4,
    DTFFT_DCT_4 = 6,
    DTFFT_DST_1 = 7,
    DTFFT_DST_2 = 9,
    DTFFT_DST_3 = 8,
    DTFFT_DST_4 = 10
} dtfft_r2r_kind_t;

typedef void* dtfft_plan_t;

/** Local box of one layout, fastest axis first (reference include/dtfft.h:354-371). */
typedef struct {
    uint8_t dim;
    uint8_t ndims;
    int32_t starts[3];
    int32_t counts[3];
    size_t size;
} dtfft_pencil_t;

/* ---- plan constructors (reference include/dtfft.h:397-515) ---- */
dtfft_error_t dtfft_create_plan_r2r(int8_t ndims, const int32_t* dims, const dtfft_r2r_kind_t* kinds,
                                    MPI_Comm comm, dtfft_precision_t precision, dtfft_effort_t effort,
                                    dtfft_executor_t executor, dtfft_plan_t* plan);
dtfft_error_t dtfft_create_plan_r2r_pencil(const dtfft_pencil_t* pencil, const dtfft_r2r_kind_t* kinds,
                                           MPI_Comm comm, dtfft_precision_t precision, dtfft_effort_t effort,
                                           dtfft_executor_t executor, dtfft_plan_t* plan);
dtfft_error_t dtfft_create_plan_c2c(int8_t ndims, const int32_t* dims, MPI_Comm comm,
                                    dtfft_precision_t precision, dtfft_effort_t effort,
                                    dtfft_executor_t executor, dtfft_plan_t* plan);
dtfft_error_t dtfft_create_plan_c2c_pencil(const dtfft_pencil_t* pencil, MPI_Comm comm,
                                           dtfft_precision_t precision, dtfft_effort_t effort,
                                           dtfft_executor_t executor, dtfft_plan_t* plan);
dtfft_error_t dtfft_create_plan_r2c(int8_t ndims, const int32_t* dims, MPI_Comm comm,
                                    dtfft_precision_t precision, dtfft_effort_t effort,
                                    dtfft_executor_t executor, dtfft_plan_t* plan);
dtfft_error_t dtfft_create_plan_r2c_pencil(const dtfft_pencil_t* pencil, MPI_Comm comm,
                                           dtfft_precision_t precision, dtfft_effort_t effort,
                                           dtfft_executor_t executor, dtfft_plan_t* plan);

/* ---- slab queries (reference include/dtfft.h:524-534) ---- */
dtfft_error_t dtfft_get_z_slab_enabled(dtfft_plan_t plan, bool* is_z_slab_enabled);
dtfft_error_t dtfft_get_y_slab_enabled(dtfft_plan_t plan, bool* is_y_slab_enabled);

/* ---- execution (reference include/dtfft.h:554-645) ----
 * All calls are asynchronous on the plan's stream.  `in` may be overwritten
 * by execute; transposes need in != out. */
dtfft_error_t dtfft_execute(dtfft_plan_t plan, void* in, void* out, dtfft_execute_t execute_type, void* aux);
dtfft_error_t dtfft_transpose(dtfft_plan_t plan, void* in, void* out, dtfft_transpose_t transpose_type, void* aux);

typedef void* dtfft_request_t;
dtfft_error_t dtfft_transpose_start(dtfft_plan_t plan, void* in, void* out, dtfft_transpose_t transpose_type,
                                    void* aux, dtfft_request_t* request);
dtfft_error_t dtfft_transpose_end(dtfft_plan_t plan, dtfft_request_t request);
dtfft_error_t dtfft_reshape(dtfft_plan_t plan, void* in, void* out, dtfft_reshape_t reshape_type, void* aux);
dtfft_error_t dtfft_reshape_start(dtfft_plan_t plan, void* in, void* out, dtfft_reshape_t reshape_type,
                                  void* aux, dtfft_request_t* request);
dtfft_error_t dtfft_reshape_end(dtfft_plan_t plan, dtfft_request_t request);

dtfft_error_t dtfft_destroy(dtfft_plan_t* plan);

/* ---- sizes (reference include/dtfft.h:667-760) ---- */
dtfft_error_t dtfft_get_local_sizes(dtfft_plan_t plan, int32_t* in_starts, int32_t* in_counts,
                                    int32_t* out_starts, int32_t* out_counts, size_t* alloc_size);
dtfft_error_t dtfft_get_alloc_size(dtfft_plan_t plan, size_t* alloc_size);
dtfft_error_t dtfft_get_aux_size(dtfft_plan_t plan, size_t* aux_size);
dtfft_error_t dtfft_get_aux_bytes(dtfft_plan_t plan, size_t* aux_bytes);
dtfft_error_t dtfft_get_aux_size_reshape(dtfft_plan_t plan, size_t* aux_size);
dtfft_error_t dtfft_get_aux_bytes_reshape(dtfft_plan_t plan, size_t* aux_bytes);
dtfft_error_t dtfft_get_aux_size_transpose(dtfft_plan_t plan, size_t* aux_size);
dtfft_error_t dtfft_get_aux_bytes_transpose(dtfft_plan_t plan, size_t* aux_bytes);

const char* dtfft_get_error_string(dtfft_error_t error_code);
const char* dtfft_get_precision_string(dtfft_precision_t precision);
const char* dtfft_get_executor_string(dtfft_executor_t executor);

typedef enum {
    DTFFT_LAYOUT_X_BRICKS = 1,
    DTFFT_LAYOUT_X_PENCILS = 2,
    DTFFT_LAYOUT_X_PENCILS_FOURIER = 3,
    DTFFT_LAYOUT_Y_PENCILS = 4,
    DTFFT_LAYOUT_Z_PENCILS = 5,
    DTFFT_LAYOUT_Z_BRICKS = 6
} dtfft_layout_t;

/* ---- plan properties (reference include/dtfft.h:797-890) ---- */
dtfft_error_t dtfft_get_pencil(dtfft_plan_t plan, dtfft_layout_t layout, dtfft_pencil_t* pencil);
dtfft_error_t dtfft_get_element_size(dtfft_plan_t plan, size_t* element_size);
dtfft_error_t dtfft_get_alloc_bytes(dtfft_plan_t plan, size_t* alloc_bytes);
dtfft_error_t dtfft_mem_alloc(dtfft_plan_t plan, size_t alloc_bytes, void** ptr);
dtfft_error_t dtfft_mem_free(dtfft_plan_t plan, void* ptr);
dtfft_error_t dtfft_report(dtfft_plan_t plan);
dtfft_error_t dtfft_get_executor(dtfft_plan_t plan, dtfft_executor_t* executor);
dtfft_error_t dtfft_get_precision(dtfft_plan_t plan, dtfft_precision_t* precision);
dtfft_error_t dtfft_get_dims(dtfft_plan_t plan, int8_t* ndims, const int32_t* dims[]);
dtfft_error_t dtfft_get_grid_dims(dtfft_plan_t plan, int8_t* ndims, const int32_t* grid_dims[]);

/** Exchange backends (values from dtfft_config.h.in:147-166).  One GPU has no
 * exchange, so plans report DTFFT_BACKEND_NONE. */
typedef enum {
    DTFFT_BACKEND_MPI_DATATYPE = 21,
    DTFFT_BACKEND_MPI_P2P = 22,
    DTFFT_BACKEND_MPI_P2P_PIPELINED = 26,
    DTFFT_BACKEND_MPI_A2A = 23,
    DTFFT_BACKEND_MPI_RMA = 29,
    DTFFT_BACKEND_MPI_RMA_PIPELINED = 30,
    DTFFT_BACKEND_MPI_P2P_SCHEDULED = 31,
    DTFFT_BACKEND_MPI_P2P_FUSED = 32,
    DTFFT_BACKEND_MPI_RMA_FUSED = 33,
    DTFFT_BACKEND_MPI_P2P_COMPRESSED = 34,
    DTFFT_BACKEND_MPI_RMA_COMPRESSED = 35,
    DTFFT_BACKEND_NCCL = 24,
    DTFFT_BACKEND_NCCL_PIPELINED = 27,
    DTFFT_BACKEND_NCCL_COMPRESSED = 37,
    DTFFT_BACKEND_CUFFTMP = 25,
    DTFFT_BACKEND_CUFFTMP_PIPELINED = 28,
    DTFFT_BACKEND_ADAPTIVE = 36,
    DTFFT_BACKEND_NONE = -111
} dtfft_backend_t;

typedef enum { DTFFT_TRANSPOSE_MODE_PACK = 15, DTFFT_TRANSPOSE_MODE_UNPACK = 16 } dtfft_transpose_mode_t;
typedef enum { DTFFT_ACCESS_MODE_WRITE = -1, DTFFT_ACCESS_MODE_READ = 1 } dtfft_access_mode_t;

typedef void* dtfft_stream_t;
typedef enum { DTFFT_PLATFORM_HOST = 1, DTFFT_PLATFORM_CUDA = 2 } dtfft_platform_t;

dtfft_error_t dtfft_get_stream(dtfft_plan_t plan, dtfft_stream_t* stream);
dtfft_error_t dtfft_get_platform(dtfft_plan_t plan, dtfft_platform_t* platform);
dtfft_error_t dtfft_get_backend(dtfft_plan_t plan, dtfft_backend_t* backend);
dtfft_error_t dtfft_get_reshape_backend(dtfft_plan_t plan, dtfft_backend_t* backend);
const char* dtfft_get_backend_string(dtfft_backend_t backend);
dtfft_error_t dtfft_get_backend_pipelined(const dtfft_backend_t backend, bool* is_pipe);

/** Configuration; same fields and order as the reference's CUDA build
 * without compression (reference include/dtfft.h:1159-1395). */
typedef struct {
    bool enable_log;
    bool enable_z_slab;
    bool enable_y_slab;
    int32_t n_measure_warmup_iters;
    int32_t n_measure_iters;
    dtfft_platform_t platform;
    dtfft_stream_t stream;
    dtfft_backend_t backend;
    dtfft_backend_t reshape_backend;
    bool enable_datatype_backend;
    bool enable_mpi_backends;
    bool enable_pipelined_backends;
    bool enable_rma_backends;
    bool enable_fused_backends;
    bool enable_nccl_backends;
    bool enable_nvshmem_backends;
    bool enable_kernel_autotune;
    bool enable_fourier_reshape;
    dtfft_transpose_mode_t transpose_mode;
    dtfft_access_mode_t access_mode;
} dtfft_config_t;

dtfft_error_t dtfft_create_config(dtfft_config_t* config);
dtfft_error_t dtfft_set_config(const dtfft_config_t* config);

#ifdef __cplusplus
}
#endif
#endif /* DTFFT_H */
