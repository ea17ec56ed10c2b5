/*
 * dtfft.hpp -- C++ interface of the GB300 execute path of dtFFT.
 *
 * Drop-in for the reference's C++ header (include/dtfft.hpp of dtFFT
 * v3.2.0): the same namespace, class and enum names, member signatures and
 * class layouts, so a C++ program written against the reference recompiles
 * against this header (or keeps the reference's header) and links to
 * libdtfft_gb300.so, which implements the out-of-line members
 * (dtfft_gb300/csrc/api_cxx.cpp) on top of the C ABI of dtfft.h.
 *
 * Errors: members returning `Error` never throw; the value-returning
 * overloads and the constructors throw dtfft::Exception.
 */
#ifndef DTFFT_HPP
#define DTFFT_HPP

#include "dtfft.h"

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#define DTFFT_THROW_EXCEPTION(error_code, msg)                       \
    do {                                                             \
        throw dtfft::Exception(error_code, msg, __FILE__, __LINE__); \
    } while (false);

#define DTFFT_CXX_CALL(call)                                           \
    do {                                                               \
        dtfft::Error ierr = call;                                      \
        if (ierr != dtfft::Error::SUCCESS) {                           \
            DTFFT_THROW_EXCEPTION(ierr, dtfft::get_error_string(ierr)) \
        }                                                              \
    } while (false);

namespace dtfft {

/** Library version (reference include/dtfft.hpp, struct Version). */
struct Version {
public:
    static constexpr int32_t MAJOR = DTFFT_VERSION_MAJOR;
    static constexpr int32_t MINOR = DTFFT_VERSION_MINOR;
    static constexpr int32_t PATCH = DTFFT_VERSION_PATCH;
    static constexpr int32_t CODE = DTFFT_VERSION_CODE;
    static int32_t get() noexcept { return dtfft_get_version(); }
    static constexpr int32_t get(int32_t major, int32_t minor, int32_t patch) noexcept
    {
        return DTFFT_VERSION(major, minor, patch);
    }
};

/** Error codes: the values of dtfft_error_t. */
enum class Error {
    SUCCESS = DTFFT_SUCCESS,
    MPI_FINALIZED = DTFFT_ERROR_MPI_FINALIZED,
    PLAN_NOT_CREATED = DTFFT_ERROR_PLAN_NOT_CREATED,
    INVALID_TRANSPOSE_TYPE = DTFFT_ERROR_INVALID_TRANSPOSE_TYPE,
    INVALID_N_DIMENSIONS = DTFFT_ERROR_INVALID_N_DIMENSIONS,
    INVALID_DIMENSION_SIZE = DTFFT_ERROR_INVALID_DIMENSION_SIZE,
    INVALID_COMM_TYPE = DTFFT_ERROR_INVALID_COMM_TYPE,
    INVALID_PRECISION = DTFFT_ERROR_INVALID_PRECISION,
    INVALID_EFFORT = DTFFT_ERROR_INVALID_EFFORT,
    INVALID_EXECUTOR = DTFFT_ERROR_INVALID_EXECUTOR,
    INVALID_COMM_DIMS = DTFFT_ERROR_INVALID_COMM_DIMS,
    INVALID_COMM_FAST_DIM = DTFFT_ERROR_INVALID_COMM_FAST_DIM,
    MISSING_R2R_KINDS = DTFFT_ERROR_MISSING_R2R_KINDS,
    INVALID_R2R_KINDS = DTFFT_ERROR_INVALID_R2R_KINDS,
    R2C_TRANSPOSE_PLAN = DTFFT_ERROR_R2C_TRANSPOSE_PLAN,
    INPLACE_TRANSPOSE = DTFFT_ERROR_INPLACE_TRANSPOSE,
    INVALID_AUX = DTFFT_ERROR_INVALID_AUX,
    INVALID_LAYOUT = DTFFT_ERROR_INVALID_LAYOUT,
    INVALID_USAGE = DTFFT_ERROR_INVALID_USAGE,
    PLAN_IS_CREATED = DTFFT_ERROR_PLAN_IS_CREATED,
    R2R_FFT_NOT_SUPPORTED = DTFFT_ERROR_R2R_FFT_NOT_SUPPORTED,
    ALLOC_FAILED = DTFFT_ERROR_ALLOC_FAILED,
    FREE_FAILED = DTFFT_ERROR_FREE_FAILED,
    INVALID_ALLOC_BYTES = DTFFT_ERROR_INVALID_ALLOC_BYTES,
    DLOPEN_FAILED = DTFFT_ERROR_DLOPEN_FAILED,
    DLSYM_FAILED = DTFFT_ERROR_DLSYM_FAILED,
    PENCIL_ARRAYS_SIZE_MISMATCH = DTFFT_ERROR_PENCIL_ARRAYS_SIZE_MISMATCH,
    PENCIL_ARRAYS_INVALID_SIZES = DTFFT_ERROR_PENCIL_ARRAYS_INVALID_SIZES,
    PENCIL_INVALID_COUNTS = DTFFT_ERROR_PENCIL_INVALID_COUNTS,
    PENCIL_INVALID_STARTS = DTFFT_ERROR_PENCIL_INVALID_STARTS,
    PENCIL_SHAPE_MISMATCH = DTFFT_ERROR_PENCIL_SHAPE_MISMATCH,
    PENCIL_OVERLAP = DTFFT_ERROR_PENCIL_OVERLAP,
    PENCIL_NOT_CONTINUOUS = DTFFT_ERROR_PENCIL_NOT_CONTINUOUS,
    PENCIL_NOT_INITIALIZED = DTFFT_ERROR_PENCIL_NOT_INITIALIZED,
    INVALID_MEASURE_WARMUP_ITERS = DTFFT_ERROR_INVALID_MEASURE_WARMUP_ITERS,
    INVALID_MEASURE_ITERS = DTFFT_ERROR_INVALID_MEASURE_ITERS,
    INVALID_REQUEST = DTFFT_ERROR_INVALID_REQUEST,
    TRANSPOSE_ACTIVE = DTFFT_ERROR_TRANSPOSE_ACTIVE,
    TRANSPOSE_NOT_ACTIVE = DTFFT_ERROR_TRANSPOSE_NOT_ACTIVE,
    INVALID_RESHAPE_TYPE = DTFFT_ERROR_INVALID_RESHAPE_TYPE,
    RESHAPE_ACTIVE = DTFFT_ERROR_RESHAPE_ACTIVE,
    RESHAPE_NOT_ACTIVE = DTFFT_ERROR_RESHAPE_NOT_ACTIVE,
    INPLACE_RESHAPE = DTFFT_ERROR_INPLACE_RESHAPE,
    INVALID_EXECUTE_TYPE = DTFFT_ERROR_INVALID_EXECUTE_TYPE,
    RESHAPE_NOT_SUPPORTED = DTFFT_ERROR_RESHAPE_NOT_SUPPORTED,
    R2C_EXECUTE_CALLED = DTFFT_ERROR_R2C_EXECUTE_CALLED,
    INVALID_CART_COMM = DTFFT_ERROR_INVALID_CART_COMM,
    INVALID_TRANSPOSE_MODE = DTFFT_ERROR_INVALID_TRANSPOSE_MODE,
    INVALID_ACCESS_MODE = DTFFT_ERROR_INVALID_ACCESS_MODE,
    GPU_INVALID_STREAM = DTFFT_ERROR_GPU_INVALID_STREAM,
    INVALID_BACKEND = DTFFT_ERROR_INVALID_BACKEND,
    GPU_NOT_SET = DTFFT_ERROR_GPU_NOT_SET,
    VKFFT_R2R_2D_PLAN = DTFFT_ERROR_VKFFT_R2R_2D_PLAN,
    BACKENDS_DISABLED = DTFFT_ERROR_BACKENDS_DISABLED,
    NOT_DEVICE_PTR = DTFFT_ERROR_NOT_DEVICE_PTR,
    NOT_NVSHMEM_PTR = DTFFT_ERROR_NOT_NVSHMEM_PTR,
    INVALID_PLATFORM = DTFFT_ERROR_INVALID_PLATFORM,
    INVALID_PLATFORM_EXECUTOR = DTFFT_ERROR_INVALID_PLATFORM_EXECUTOR,
    INVALID_PLATFORM_BACKEND = DTFFT_ERROR_INVALID_PLATFORM_BACKEND,
    COMPRESSION_CUDA_NOT_SUPPORTED = DTFFT_ERROR_COMPRESSION_CUDA_NOT_SUPPORTED,
    COMPRESSION_INVALID_RATE = DTFFT_ERROR_COMPRESSION_INVALID_RATE,
    COMPRESSION_INVALID_PRECISION = DTFFT_ERROR_COMPRESSION_INVALID_PRECISION,
    COMPRESSION_INVALID_TOLERANCE = DTFFT_ERROR_COMPRESSION_INVALID_TOLERANCE,
    COMPRESSION_INVALID_MODE = DTFFT_ERROR_COMPRESSION_INVALID_MODE,
    COMPRESSION_INVALID_LIBRARY = DTFFT_ERROR_COMPRESSION_INVALID_LIBRARY,
    COMPRESSION_NOT_USED = DTFFT_ERROR_COMPRESSION_NOT_USED,
    GPU_CALL_FAILED = DTFFT_ERROR_GPU_CALL_FAILED,
    FFT_SIZE_NOT_SUPPORTED = DTFFT_ERROR_FFT_SIZE_NOT_SUPPORTED,
    NOALLOC_SCRATCH_TOO_SMALL = DTFFT_ERROR_NOALLOC_SCRATCH_TOO_SMALL,
    GPU_WAIT_TIMEOUT = DTFFT_ERROR_GPU_WAIT_TIMEOUT
};

/** Text of an error code (dtfft_get_error_string). */
std::string get_error_string(Error error_code) noexcept;

enum class Execute { FORWARD = DTFFT_EXECUTE_FORWARD, BACKWARD = DTFFT_EXECUTE_BACKWARD };

enum class Transpose {
    X_TO_Y = DTFFT_TRANSPOSE_X_TO_Y,
    Y_TO_X = DTFFT_TRANSPOSE_Y_TO_X,
    Y_TO_Z = DTFFT_TRANSPOSE_Y_TO_Z,
    Z_TO_Y = DTFFT_TRANSPOSE_Z_TO_Y,
    X_TO_Z = DTFFT_TRANSPOSE_X_TO_Z,
    Z_TO_X = DTFFT_TRANSPOSE_Z_TO_X
};

enum class Reshape {
    X_BRICKS_TO_PENCILS = DTFFT_RESHAPE_X_BRICKS_TO_PENCILS,
    X_PENCILS_TO_BRICKS = DTFFT_RESHAPE_X_PENCILS_TO_BRICKS,
    Z_BRICKS_TO_PENCILS = DTFFT_RESHAPE_Z_BRICKS_TO_PENCILS,
    Z_PENCILS_TO_BRICKS = DTFFT_RESHAPE_Z_PENCILS_TO_BRICKS,
    Y_BRICKS_TO_PENCILS = DTFFT_RESHAPE_Y_BRICKS_TO_PENCILS,
    Y_PENCILS_TO_BRICKS = DTFFT_RESHAPE_Y_PENCILS_TO_BRICKS,
};

enum class Layout {
    X_BRICKS = DTFFT_LAYOUT_X_BRICKS,
    X_PENCILS = DTFFT_LAYOUT_X_PENCILS,
    X_PENCILS_FOURIER = DTFFT_LAYOUT_X_PENCILS_FOURIER,
    Y_PENCILS = DTFFT_LAYOUT_Y_PENCILS,
    Z_PENCILS = DTFFT_LAYOUT_Z_PENCILS,
    Z_BRICKS = DTFFT_LAYOUT_Z_BRICKS
};

enum class Precision { SINGLE = DTFFT_SINGLE, DOUBLE = DTFFT_DOUBLE };

std::string get_precision_string(Precision precision) noexcept;

enum class Effort {
    ESTIMATE = DTFFT_ESTIMATE,
    MEASURE = DTFFT_MEASURE,
    PATIENT = DTFFT_PATIENT,
    EXHAUSTIVE = DTFFT_EXHAUSTIVE
};

enum class Executor {
    NONE = DTFFT_EXECUTOR_NONE,
    FFTW3 = DTFFT_EXECUTOR_FFTW3,
    MKL = DTFFT_EXECUTOR_MKL,
    CUFFT = DTFFT_EXECUTOR_CUFFT,
    VKFFT = DTFFT_EXECUTOR_VKFFT
};

std::string get_executor_string(Executor executor) noexcept;

enum class R2RKind {
    DCT_1 = DTFFT_DCT_1,
    DCT_2 = DTFFT_DCT_2,
    DCT_3 = DTFFT_DCT_3,
    DCT_4 = DTFFT_DCT_4,
    DST_1 = DTFFT_DST_1,
    DST_2 = DTFFT_DST_2,
    DST_3 = DTFFT_DST_3,
    DST_4 = DTFFT_DST_4
};

enum class Backend {
    MPI_DATATYPE = DTFFT_BACKEND_MPI_DATATYPE,
    MPI_P2P = DTFFT_BACKEND_MPI_P2P,
    MPI_P2P_PIPELINED = DTFFT_BACKEND_MPI_P2P_PIPELINED,
    MPI_A2A = DTFFT_BACKEND_MPI_A2A,
    MPI_RMA = DTFFT_BACKEND_MPI_RMA,
    MPI_RMA_PIPELINED = DTFFT_BACKEND_MPI_RMA_PIPELINED,
    MPI_P2P_SCHEDULED = DTFFT_BACKEND_MPI_P2P_SCHEDULED,
    MPI_P2P_FUSED = DTFFT_BACKEND_MPI_P2P_FUSED,
    MPI_RMA_FUSED = DTFFT_BACKEND_MPI_RMA_FUSED,
    MPI_P2P_COMPRESSED = DTFFT_BACKEND_MPI_P2P_COMPRESSED,
    MPI_RMA_COMPRESSED = DTFFT_BACKEND_MPI_RMA_COMPRESSED,
    NCCL = DTFFT_BACKEND_NCCL,
    NCCL_PIPELINED = DTFFT_BACKEND_NCCL_PIPELINED,
    NCCL_COMPRESSED = DTFFT_BACKEND_NCCL_COMPRESSED,
    CUFFTMP = DTFFT_BACKEND_CUFFTMP,
    CUFFTMP_PIPELINED = DTFFT_BACKEND_CUFFTMP_PIPELINED,
    ADAPTIVE = DTFFT_BACKEND_ADAPTIVE,
    NONE = DTFFT_BACKEND_NONE
};

std::string get_backend_string(Backend backend);
bool get_backend_pipelined(Backend backend);

enum class Platform {
    HOST = DTFFT_PLATFORM_HOST,
    CUDA = DTFFT_PLATFORM_CUDA,
};

/** Exception thrown by the throwing members; carries the dtFFT error code. */
class Exception final : public std::exception {
private:
    Error _error_code;
    std::string _message;
    std::string _file;
    int _line;
    mutable std::string _what_cache;

public:
    Exception(Error error_code, std::string msg, const char* file, int line);
    const char* what() const noexcept override;
    Error get_error_code() const noexcept;
    const std::string& get_message() const noexcept;
    const std::string& get_file() const noexcept;
    int get_line() const noexcept;
};

/** A local block: starts and counts per dimension (dtfft_pencil_t). */
struct Pencil {
private:
    bool is_created;
    bool is_obtained;
    dtfft_pencil_t pencil;
    explicit Pencil(dtfft_pencil_t& c_pencil);
    friend class Plan;

public:
    Pencil();
    explicit Pencil(int32_t n_dims, const int32_t* starts, const int32_t* counts);
    explicit Pencil(const std::vector<int32_t>& starts, const std::vector<int32_t>& counts);
    uint8_t get_ndims() const;
    uint8_t get_dim() const;
    std::vector<int32_t> get_starts() const;
    std::vector<int32_t> get_counts() const;
    size_t get_size() const;
    const dtfft_pencil_t& c_struct() const;
};

enum class TransposeMode { PACK = DTFFT_TRANSPOSE_MODE_PACK, UNPACK = DTFFT_TRANSPOSE_MODE_UNPACK };

enum class AccessMode { WRITE = DTFFT_ACCESS_MODE_WRITE, READ = DTFFT_ACCESS_MODE_READ };

/** Settings applied to plans created after set_config (dtfft_config_t). */
struct Config {
protected:
    dtfft_config_t config;

public:
    explicit Config() { DTFFT_CXX_CALL(static_cast<Error>(dtfft_create_config(&config))) }
    Config& set_enable_log(const bool v) noexcept { config.enable_log = v; return *this; }
    Config& set_enable_z_slab(bool v) noexcept { config.enable_z_slab = v; return *this; }
    Config& set_enable_y_slab(bool v) noexcept { config.enable_y_slab = v; return *this; }
    Config& set_measure_warmup_iters(int32_t v) noexcept { config.n_measure_warmup_iters = v; return *this; }
    Config& set_measure_iters(int32_t v) noexcept { config.n_measure_iters = v; return *this; }
    Config& set_platform(Platform v) noexcept { config.platform = static_cast<dtfft_platform_t>(v); return *this; }
    Config& set_stream(dtfft_stream_t v) noexcept { config.stream = v; return *this; }
    Config& set_backend(Backend v) noexcept { config.backend = static_cast<dtfft_backend_t>(v); return *this; }
    Config& set_reshape_backend(Backend v) noexcept
    {
        config.reshape_backend = static_cast<dtfft_backend_t>(v);
        return *this;
    }
    Config& set_enable_datatype_backend(bool v) noexcept { config.enable_datatype_backend = v; return *this; }
    Config& set_enable_mpi_backends(bool v) noexcept { config.enable_mpi_backends = v; return *this; }
    Config& set_enable_pipelined_backends(bool v) noexcept { config.enable_pipelined_backends = v; return *this; }
    Config& set_enable_rma_backends(bool v) noexcept { config.enable_rma_backends = v; return *this; }
    Config& set_enable_fused_backends(bool v) noexcept { config.enable_fused_backends = v; return *this; }
    Config& set_enable_nccl_backends(bool v) noexcept { config.enable_nccl_backends = v; return *this; }
    Config& set_enable_nvshmem_backends(bool v) noexcept { config.enable_nvshmem_backends = v; return *this; }
    Config& set_enable_kernel_autotune(bool v) noexcept { config.enable_kernel_autotune = v; return *this; }
    Config& set_enable_fourier_reshape(bool v) noexcept { config.enable_fourier_reshape = v; return *this; }
    Config& set_transpose_mode(TransposeMode v) noexcept
    {
        config.transpose_mode = static_cast<dtfft_transpose_mode_t>(v);
        return *this;
    }
    Config& set_access_mode(AccessMode v) noexcept
    {
        config.access_mode = static_cast<dtfft_access_mode_t>(v);
        return *this;
    }
    dtfft_config_t c_struct() const { return config; }
};

/** Makes `config` the settings of plans created from now on (dtfft_set_config). */
Error set_config(const Config& config) noexcept;

/** Base of the plan classes: execute, transpose, reshape and the queries.
 *  The destructor destroys the plan. */
class Plan {
protected:
    dtfft_plan_t _plan;

public:
    Error get_z_slab_enabled(bool* is_z_slab_enabled) const noexcept;
    bool get_z_slab_enabled() const;
    Error get_y_slab_enabled(bool* is_y_slab_enabled) const noexcept;
    bool get_y_slab_enabled() const;
    Error report() const noexcept;
    Error get_pencil(Layout layout, Pencil& pencil) const noexcept;
    Pencil get_pencil(Layout layout) const;

    Error execute(void* in, void* out, Execute execute_type, void* aux = nullptr) const noexcept;
    template <typename Tr>
    Tr* execute(void* inout, const Execute execute_type, void* aux = nullptr) const
    {
        DTFFT_CXX_CALL(execute(inout, inout, execute_type, aux))
        return static_cast<Tr*>(inout);
    }
    template <typename T, typename Tr = T>
    Tr* execute(T* inout, const Execute execute_type, void* aux = nullptr) const
    {
        return execute<Tr>(static_cast<void*>(inout), execute_type, aux);
    }

    Error forward(void* in, void* out, void* aux) const noexcept;
    template <typename Tr>
    Tr* forward(void* inout, void* aux = nullptr) const
    {
        return execute<Tr>(inout, Execute::FORWARD, aux);
    }
    template <typename T, typename Tr = T>
    Tr* forward(T* inout, void* aux = nullptr) const
    {
        return forward<Tr>(static_cast<void*>(inout), aux);
    }

    Error backward(void* in, void* out, void* aux) const noexcept;
    template <typename Tr>
    Tr* backward(void* inout, void* aux = nullptr) const
    {
        return execute<Tr>(inout, Execute::BACKWARD, aux);
    }
    template <typename T, typename Tr = T>
    Tr* backward(T* inout, void* aux = nullptr) const
    {
        return backward<Tr>(static_cast<void*>(inout), aux);
    }

    Error transpose(void* in, void* out, Transpose transpose_type, void* aux = nullptr) const noexcept;
    Error transpose_start(void* in, void* out, Transpose transpose_type, void* aux,
                          dtfft_request_t* request) const noexcept;
    Error transpose_start(void* in, void* out, Transpose transpose_type, dtfft_request_t* request) const noexcept;
    dtfft_request_t transpose_start(void* in, void* out, Transpose transpose_type, void* aux = nullptr) const;
    Error transpose_end(dtfft_request_t request) const noexcept;

    Error reshape(void* in, void* out, Reshape reshape_type, void* aux = nullptr) const noexcept;
    Error reshape_start(void* in, void* out, Reshape reshape_type, void* aux, dtfft_request_t* request) const noexcept;
    Error reshape_start(void* in, void* out, Reshape reshape_type, dtfft_request_t* request) const noexcept;
    dtfft_request_t reshape_start(void* in, void* out, Reshape reshape_type, void* aux = nullptr) const;
    Error reshape_end(dtfft_request_t request) const noexcept;

    Error get_alloc_size(size_t* alloc_size) const noexcept;
    std::size_t get_alloc_size() const;
    Error get_aux_size(std::size_t* aux_size) const noexcept;
    std::size_t get_aux_size() const;
    Error get_aux_bytes(std::size_t* aux_bytes) const noexcept;
    std::size_t get_aux_bytes() const;
    Error get_aux_size_reshape(std::size_t* aux_size) const noexcept;
    std::size_t get_aux_size_reshape() const;
    Error get_aux_bytes_reshape(std::size_t* aux_bytes) const noexcept;
    std::size_t get_aux_bytes_reshape() const;
    Error get_aux_size_transpose(std::size_t* aux_size) const noexcept;
    std::size_t get_aux_size_transpose() const;
    Error get_aux_bytes_transpose(std::size_t* aux_bytes) const noexcept;
    std::size_t get_aux_bytes_transpose() const;
    Error get_local_sizes(std::vector<int32_t>& in_starts, std::vector<int32_t>& in_counts,
                          std::vector<int32_t>& out_starts, std::vector<int32_t>& out_counts,
                          std::size_t* alloc_size) const noexcept;
    Error get_local_sizes(int32_t* in_starts = nullptr, int32_t* in_counts = nullptr, int32_t* out_starts = nullptr,
                          int32_t* out_counts = nullptr, size_t* alloc_size = nullptr) const noexcept;
    Error get_element_size(size_t* element_size) const noexcept;
    size_t get_element_size() const;
    Error get_alloc_bytes(size_t* alloc_bytes) const noexcept;
    size_t get_alloc_bytes() const;
    Error get_executor(Executor* executor) const noexcept;
    Executor get_executor() const;
    Error get_precision(Precision* precision) const noexcept;
    Precision get_precision() const;
    Error get_dims(int8_t* ndims, const int32_t* dims[]) const noexcept;
    std::vector<int32_t> get_dims() const;
    Error get_grid_dims(int8_t* ndims, const int32_t* grid_dims[]) const noexcept;
    std::vector<int32_t> get_grid_dims() const;

    Error mem_alloc(size_t alloc_bytes, void** ptr) const noexcept;
    void* mem_alloc(size_t alloc_bytes) const;
    template <typename T>
    T* mem_alloc(const size_t alloc_size) const
    {
        return static_cast<T*>(mem_alloc(alloc_size * sizeof(T)));
    }
    Error mem_free(void* ptr) const noexcept;
    Error destroy() noexcept;

    Error get_backend(Backend& backend) const noexcept;
    Backend get_backend() const;
    Error get_reshape_backend(Backend& backend) const noexcept;
    Backend get_reshape_backend() const;
    Error get_stream(dtfft_stream_t* stream) const noexcept;
    dtfft_stream_t get_stream() const;
    Error get_platform(Platform& platform) const noexcept;
    Platform get_platform() const;

    dtfft_plan_t c_struct() const { return _plan; }
    virtual ~Plan() noexcept = 0;
};

inline Plan::~Plan() noexcept { destroy(); }

/** Complex-to-complex plan (dtfft_create_plan_c2c[_pencil]). */
class PlanC2C final : public Plan {
public:
    explicit PlanC2C(const std::vector<int32_t>& dims, MPI_Comm comm = MPI_COMM_WORLD,
                     Precision precision = Precision::DOUBLE, Effort effort = Effort::ESTIMATE,
                     Executor executor = Executor::NONE);
    explicit PlanC2C(const std::vector<int32_t>& dims, Precision precision, Effort effort = Effort::ESTIMATE);
    explicit PlanC2C(int8_t ndims, const int32_t* dims, MPI_Comm comm = MPI_COMM_WORLD,
                     Precision precision = Precision::DOUBLE, Effort effort = Effort::ESTIMATE,
                     Executor executor = Executor::NONE);
    explicit PlanC2C(const Pencil& pencil, Precision precision, Effort effort = Effort::ESTIMATE);
    explicit PlanC2C(const Pencil& pencil, MPI_Comm comm = MPI_COMM_WORLD, Precision precision = Precision::DOUBLE,
                     Effort effort = Effort::ESTIMATE, Executor executor = Executor::NONE);
};

/** Real-to-complex plan (dtfft_create_plan_r2c[_pencil]). */
class PlanR2C final : public Plan {
public:
    explicit PlanR2C(const std::vector<int32_t>& dims, MPI_Comm comm = MPI_COMM_WORLD,
                     Precision precision = Precision::DOUBLE, Effort effort = Effort::ESTIMATE,
                     Executor executor = Executor::NONE);
    explicit PlanR2C(const std::vector<int32_t>& dims, Precision precision, Effort effort = Effort::ESTIMATE);
    explicit PlanR2C(int8_t ndims, const int32_t* dims, MPI_Comm comm = MPI_COMM_WORLD,
                     Precision precision = Precision::DOUBLE, Effort effort = Effort::ESTIMATE,
                     Executor executor = Executor::NONE);
    explicit PlanR2C(const Pencil& pencil, Precision precision, Effort effort = Effort::ESTIMATE);
    explicit PlanR2C(const Pencil& pencil, MPI_Comm comm = MPI_COMM_WORLD, Precision precision = Precision::DOUBLE,
                     Effort effort = Effort::ESTIMATE, Executor executor = Executor::NONE);
};

/** Real-to-real plan (dtfft_create_plan_r2r[_pencil]). */
class PlanR2R final : public Plan {
public:
    explicit PlanR2R(const std::vector<int32_t>& dims, const std::vector<R2RKind>& kinds = std::vector<R2RKind>(),
                     MPI_Comm comm = MPI_COMM_WORLD, Precision precision = Precision::DOUBLE,
                     Effort effort = Effort::ESTIMATE, Executor executor = Executor::NONE);
    explicit PlanR2R(const std::vector<int32_t>& dims, Precision precision, Effort effort = Effort::ESTIMATE);
    explicit PlanR2R(int8_t ndims, const int32_t* dims, const R2RKind* kinds = nullptr, MPI_Comm comm = MPI_COMM_WORLD,
                     Precision precision = Precision::DOUBLE, Effort effort = Effort::ESTIMATE,
                     Executor executor = Executor::NONE);
    explicit PlanR2R(const Pencil& pencil, Precision precision, Effort effort = Effort::ESTIMATE);
    explicit PlanR2R(const Pencil& pencil, const std::vector<R2RKind>& kinds, MPI_Comm comm = MPI_COMM_WORLD,
                     Precision precision = Precision::DOUBLE, Effort effort = Effort::ESTIMATE,
                     Executor executor = Executor::NONE);
    explicit PlanR2R(const Pencil& pencil, const R2RKind* kinds = nullptr, MPI_Comm comm = MPI_COMM_WORLD,
                     Precision precision = Precision::DOUBLE, Effort effort = Effort::ESTIMATE,
                     Executor executor = Executor::NONE);
};

}  // namespace dtfft
#endif  // DTFFT_HPP
