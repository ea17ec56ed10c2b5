// Out-of-line members of the C++ interface (include/dtfft.hpp): thin wrappers
// over the C ABI, so a C++ program built against dtFFT's C++ header links to
// this library.  Behaviour follows src/interfaces/api/dtfft_api_cxx.cpp of
// the reference: members returning Error never throw, the value-returning
// overloads and the constructors throw dtfft::Exception with the C call's
// error code, and a Pencil made by the caller has no aligned dim or size
// until a plan fills it in (get_pencil).
#include "dtfft.hpp"

namespace dtfft {

namespace {
inline Error E(dtfft_error_t e) { return static_cast<Error>(e); }

// Value form of a "query(T*) -> Error" member: throws on failure.
template <typename T, typename F>
T value_or_throw(F&& query) {
    T v{};
    DTFFT_CXX_CALL(query(&v))
    return v;
}
}  // namespace

// ---- Exception ----------------------------------------------------------------
Exception::Exception(Error error_code, std::string msg, const char* file, int line)
    : _error_code(error_code), _message(std::move(msg)), _file(file ? file : ""), _line(line) {}

const char* Exception::what() const noexcept {
    if (_what_cache.empty())
        _what_cache = "dtFFT Exception: '" + _message + "' (code: " + std::to_string(static_cast<int>(_error_code)) +
                      ") at " + _file + ":" + std::to_string(_line);
    return _what_cache.c_str();
}
Error Exception::get_error_code() const noexcept { return _error_code; }
const std::string& Exception::get_message() const noexcept { return _message; }
const std::string& Exception::get_file() const noexcept { return _file; }
int Exception::get_line() const noexcept { return _line; }

// ---- Pencil -------------------------------------------------------------------
Pencil::Pencil(dtfft_pencil_t& c_pencil) : is_created(true), is_obtained(true), pencil(c_pencil) {}

Pencil::Pencil() : is_created(false), is_obtained(false), pencil() {}

Pencil::Pencil(int32_t n_dims, const int32_t* starts, const int32_t* counts)
    : is_created(false), is_obtained(false), pencil() {
    if (!starts || !counts || n_dims < 2 || n_dims > 3) DTFFT_CXX_CALL(Error::INVALID_USAGE)
    pencil.ndims = static_cast<uint8_t>(n_dims);
    for (int32_t d = 0; d < n_dims; ++d) {
        pencil.starts[d] = starts[d];
        pencil.counts[d] = counts[d];
    }
    is_created = true;
}

Pencil::Pencil(const std::vector<int32_t>& starts, const std::vector<int32_t>& counts)
    : Pencil(static_cast<int8_t>(starts.size()), starts.data(), counts.data()) {}

uint8_t Pencil::get_ndims() const {
    if (!is_created) DTFFT_CXX_CALL(Error::INVALID_USAGE)
    return pencil.ndims;
}
uint8_t Pencil::get_dim() const {
    if (!is_obtained) DTFFT_CXX_CALL(Error::INVALID_USAGE)
    return pencil.dim;
}
std::vector<int32_t> Pencil::get_starts() const {
    if (!is_obtained) DTFFT_CXX_CALL(Error::INVALID_USAGE)
    return std::vector<int32_t>(pencil.starts, pencil.starts + pencil.ndims);
}
std::vector<int32_t> Pencil::get_counts() const {
    if (!is_obtained) DTFFT_CXX_CALL(Error::INVALID_USAGE)
    return std::vector<int32_t>(pencil.counts, pencil.counts + pencil.ndims);
}
size_t Pencil::get_size() const {
    if (!is_obtained) DTFFT_CXX_CALL(Error::INVALID_USAGE)
    return pencil.size;
}
const dtfft_pencil_t& Pencil::c_struct() const {
    if (!is_created) DTFFT_CXX_CALL(Error::INVALID_USAGE)
    return pencil;
}

// ---- free functions -----------------------------------------------------------
std::string get_error_string(Error e) noexcept { return dtfft_get_error_string(static_cast<dtfft_error_t>(e)); }
std::string get_precision_string(Precision p) noexcept {
    return dtfft_get_precision_string(static_cast<dtfft_precision_t>(p));
}
std::string get_executor_string(Executor x) noexcept {
    return dtfft_get_executor_string(static_cast<dtfft_executor_t>(x));
}
std::string get_backend_string(Backend b) { return dtfft_get_backend_string(static_cast<dtfft_backend_t>(b)); }
bool get_backend_pipelined(Backend b) {
    bool v = false;
    dtfft_get_backend_pipelined(static_cast<dtfft_backend_t>(b), &v);
    return v;
}
Error set_config(const Config& config) noexcept {
    const dtfft_config_t c = config.c_struct();
    return E(dtfft_set_config(&c));
}

// ---- Plan: queries ------------------------------------------------------------
Error Plan::get_z_slab_enabled(bool* v) const noexcept { return E(dtfft_get_z_slab_enabled(_plan, v)); }
bool Plan::get_z_slab_enabled() const {
    return value_or_throw<bool>([this](bool* v) { return get_z_slab_enabled(v); });
}
Error Plan::get_y_slab_enabled(bool* v) const noexcept { return E(dtfft_get_y_slab_enabled(_plan, v)); }
bool Plan::get_y_slab_enabled() const {
    return value_or_throw<bool>([this](bool* v) { return get_y_slab_enabled(v); });
}
Error Plan::report() const noexcept { return E(dtfft_report(_plan)); }

Error Plan::get_pencil(Layout layout, Pencil& pencil) const noexcept {
    dtfft_pencil_t c;
    const dtfft_error_t e = dtfft_get_pencil(_plan, static_cast<dtfft_layout_t>(layout), &c);
    if (e == DTFFT_SUCCESS) pencil = Pencil(c);
    return E(e);
}
Pencil Plan::get_pencil(Layout layout) const {
    Pencil p;
    DTFFT_CXX_CALL(get_pencil(layout, p))
    return p;
}

#define GB_SIZE_QUERY(member, cfn)                                                  \
    Error Plan::member(size_t* v) const noexcept { return E(cfn(_plan, v)); }       \
    size_t Plan::member() const {                                                   \
        return value_or_throw<size_t>([this](size_t* v) { return member(v); });     \
    }
GB_SIZE_QUERY(get_alloc_size, dtfft_get_alloc_size)
GB_SIZE_QUERY(get_aux_size, dtfft_get_aux_size)
GB_SIZE_QUERY(get_aux_bytes, dtfft_get_aux_bytes)
GB_SIZE_QUERY(get_aux_size_reshape, dtfft_get_aux_size_reshape)
GB_SIZE_QUERY(get_aux_bytes_reshape, dtfft_get_aux_bytes_reshape)
GB_SIZE_QUERY(get_aux_size_transpose, dtfft_get_aux_size_transpose)
GB_SIZE_QUERY(get_aux_bytes_transpose, dtfft_get_aux_bytes_transpose)
GB_SIZE_QUERY(get_element_size, dtfft_get_element_size)
GB_SIZE_QUERY(get_alloc_bytes, dtfft_get_alloc_bytes)
#undef GB_SIZE_QUERY

Error Plan::get_local_sizes(std::vector<int32_t>& in_starts, std::vector<int32_t>& in_counts,
                            std::vector<int32_t>& out_starts, std::vector<int32_t>& out_counts,
                            size_t* alloc_size) const noexcept {
    int8_t nd = 0;
    const dtfft_error_t e = dtfft_get_dims(_plan, &nd, nullptr);
    if (e != DTFFT_SUCCESS) return E(e);
    in_starts.resize(nd);
    in_counts.resize(nd);
    out_starts.resize(nd);
    out_counts.resize(nd);
    return get_local_sizes(in_starts.data(), in_counts.data(), out_starts.data(), out_counts.data(), alloc_size);
}
Error Plan::get_local_sizes(int32_t* in_starts, int32_t* in_counts, int32_t* out_starts, int32_t* out_counts,
                            size_t* alloc_size) const noexcept {
    return E(dtfft_get_local_sizes(_plan, in_starts, in_counts, out_starts, out_counts, alloc_size));
}

Error Plan::get_executor(Executor* x) const noexcept {
    dtfft_executor_t c;
    const dtfft_error_t e = dtfft_get_executor(_plan, &c);
    if (e == DTFFT_SUCCESS) *x = static_cast<Executor>(c);
    return E(e);
}
Executor Plan::get_executor() const {
    return value_or_throw<Executor>([this](Executor* v) { return get_executor(v); });
}
Error Plan::get_precision(Precision* p) const noexcept {
    dtfft_precision_t c;
    const dtfft_error_t e = dtfft_get_precision(_plan, &c);
    if (e == DTFFT_SUCCESS) *p = static_cast<Precision>(c);
    return E(e);
}
Precision Plan::get_precision() const {
    return value_or_throw<Precision>([this](Precision* v) { return get_precision(v); });
}
Error Plan::get_dims(int8_t* ndims, const int32_t* dims[]) const noexcept { return E(dtfft_get_dims(_plan, ndims, dims)); }
std::vector<int32_t> Plan::get_dims() const {
    int8_t n = 0;
    const int32_t* d = nullptr;
    DTFFT_CXX_CALL(get_dims(&n, &d))
    return std::vector<int32_t>(d, d + n);
}
Error Plan::get_grid_dims(int8_t* ndims, const int32_t* grid_dims[]) const noexcept {
    return E(dtfft_get_grid_dims(_plan, ndims, grid_dims));
}
std::vector<int32_t> Plan::get_grid_dims() const {
    int8_t n = 0;
    const int32_t* d = nullptr;
    DTFFT_CXX_CALL(get_grid_dims(&n, &d))
    return std::vector<int32_t>(d, d + n);
}

Error Plan::get_backend(Backend& b) const noexcept {
    dtfft_backend_t c;
    const dtfft_error_t e = dtfft_get_backend(_plan, &c);
    b = static_cast<Backend>(c);
    return E(e);
}
Backend Plan::get_backend() const {
    Backend b;
    DTFFT_CXX_CALL(get_backend(b))
    return b;
}
Error Plan::get_reshape_backend(Backend& b) const noexcept {
    dtfft_backend_t c;
    const dtfft_error_t e = dtfft_get_reshape_backend(_plan, &c);
    b = static_cast<Backend>(c);
    return E(e);
}
Backend Plan::get_reshape_backend() const {
    Backend b;
    DTFFT_CXX_CALL(get_reshape_backend(b))
    return b;
}
Error Plan::get_stream(dtfft_stream_t* s) const noexcept { return E(dtfft_get_stream(_plan, s)); }
dtfft_stream_t Plan::get_stream() const {
    return value_or_throw<dtfft_stream_t>([this](dtfft_stream_t* v) { return get_stream(v); });
}
Error Plan::get_platform(Platform& p) const noexcept {
    dtfft_platform_t c;
    const dtfft_error_t e = dtfft_get_platform(_plan, &c);
    p = static_cast<Platform>(c);
    return E(e);
}
Platform Plan::get_platform() const {
    Platform p;
    DTFFT_CXX_CALL(get_platform(p))
    return p;
}

// ---- Plan: execution ----------------------------------------------------------
Error Plan::execute(void* in, void* out, Execute t, void* aux) const noexcept {
    return E(dtfft_execute(_plan, in, out, static_cast<dtfft_execute_t>(t), aux));
}
Error Plan::forward(void* in, void* out, void* aux) const noexcept { return execute(in, out, Execute::FORWARD, aux); }
Error Plan::backward(void* in, void* out, void* aux) const noexcept { return execute(in, out, Execute::BACKWARD, aux); }

Error Plan::transpose(void* in, void* out, Transpose t, void* aux) const noexcept {
    return E(dtfft_transpose(_plan, in, out, static_cast<dtfft_transpose_t>(t), aux));
}
Error Plan::transpose_start(void* in, void* out, Transpose t, void* aux, dtfft_request_t* r) const noexcept {
    return E(dtfft_transpose_start(_plan, in, out, static_cast<dtfft_transpose_t>(t), aux, r));
}
Error Plan::transpose_start(void* in, void* out, Transpose t, dtfft_request_t* r) const noexcept {
    return transpose_start(in, out, t, nullptr, r);
}
dtfft_request_t Plan::transpose_start(void* in, void* out, Transpose t, void* aux) const {
    dtfft_request_t r = nullptr;
    DTFFT_CXX_CALL(transpose_start(in, out, t, aux, &r))
    return r;
}
Error Plan::transpose_end(dtfft_request_t r) const noexcept { return E(dtfft_transpose_end(_plan, r)); }

Error Plan::reshape(void* in, void* out, Reshape t, void* aux) const noexcept {
    return E(dtfft_reshape(_plan, in, out, static_cast<dtfft_reshape_t>(t), aux));
}
Error Plan::reshape_start(void* in, void* out, Reshape t, void* aux, dtfft_request_t* r) const noexcept {
    return E(dtfft_reshape_start(_plan, in, out, static_cast<dtfft_reshape_t>(t), aux, r));
}
Error Plan::reshape_start(void* in, void* out, Reshape t, dtfft_request_t* r) const noexcept {
    return reshape_start(in, out, t, nullptr, r);
}
dtfft_request_t Plan::reshape_start(void* in, void* out, Reshape t, void* aux) const {
    dtfft_request_t r = nullptr;
    DTFFT_CXX_CALL(reshape_start(in, out, t, aux, &r))
    return r;
}
Error Plan::reshape_end(dtfft_request_t r) const noexcept { return E(dtfft_reshape_end(_plan, r)); }

// ---- Plan: memory and lifetime -----------------------------------------------------
Error Plan::mem_alloc(size_t alloc_bytes, void** ptr) const noexcept { return E(dtfft_mem_alloc(_plan, alloc_bytes, ptr)); }
void* Plan::mem_alloc(size_t alloc_bytes) const {
    void* p = nullptr;
    DTFFT_CXX_CALL(mem_alloc(alloc_bytes, &p))
    return p;
}
Error Plan::mem_free(void* ptr) const noexcept { return E(dtfft_mem_free(_plan, ptr)); }
Error Plan::destroy() noexcept { return E(dtfft_destroy(&_plan)); }

// ---- constructors -------------------------------------------------------------
namespace {
inline dtfft_precision_t cp(Precision p) { return static_cast<dtfft_precision_t>(p); }
inline dtfft_effort_t ce(Effort e) { return static_cast<dtfft_effort_t>(e); }
inline dtfft_executor_t cx(Executor x) { return static_cast<dtfft_executor_t>(x); }
inline const dtfft_r2r_kind_t* ck(const R2RKind* k) { return reinterpret_cast<const dtfft_r2r_kind_t*>(k); }
inline const R2RKind* kinds_or_null(const std::vector<R2RKind>& k) { return k.empty() ? nullptr : k.data(); }
}  // namespace

PlanC2C::PlanC2C(const std::vector<int32_t>& dims, MPI_Comm comm, Precision precision, Effort effort, Executor executor)
    : PlanC2C(static_cast<int8_t>(dims.size()), dims.data(), comm, precision, effort, executor) {}
PlanC2C::PlanC2C(const std::vector<int32_t>& dims, Precision precision, Effort effort)
    : PlanC2C(static_cast<int8_t>(dims.size()), dims.data(), MPI_COMM_WORLD, precision, effort) {}
PlanC2C::PlanC2C(int8_t ndims, const int32_t* dims, MPI_Comm comm, Precision precision, Effort effort,
                 Executor executor) {
    _plan = nullptr;
    DTFFT_CXX_CALL(E(dtfft_create_plan_c2c(ndims, dims, comm, cp(precision), ce(effort), cx(executor), &_plan)))
}
PlanC2C::PlanC2C(const Pencil& pencil, Precision precision, Effort effort)
    : PlanC2C(pencil, MPI_COMM_WORLD, precision, effort) {}
PlanC2C::PlanC2C(const Pencil& pencil, MPI_Comm comm, Precision precision, Effort effort, Executor executor) {
    _plan = nullptr;
    DTFFT_CXX_CALL(
        E(dtfft_create_plan_c2c_pencil(&pencil.c_struct(), comm, cp(precision), ce(effort), cx(executor), &_plan)))
}

PlanR2C::PlanR2C(const std::vector<int32_t>& dims, MPI_Comm comm, Precision precision, Effort effort, Executor executor)
    : PlanR2C(static_cast<int8_t>(dims.size()), dims.data(), comm, precision, effort, executor) {}
PlanR2C::PlanR2C(const std::vector<int32_t>& dims, Precision precision, Effort effort)
    : PlanR2C(static_cast<int8_t>(dims.size()), dims.data(), MPI_COMM_WORLD, precision, effort) {}
PlanR2C::PlanR2C(int8_t ndims, const int32_t* dims, MPI_Comm comm, Precision precision, Effort effort,
                 Executor executor) {
    _plan = nullptr;
    DTFFT_CXX_CALL(E(dtfft_create_plan_r2c(ndims, dims, comm, cp(precision), ce(effort), cx(executor), &_plan)))
}
PlanR2C::PlanR2C(const Pencil& pencil, Precision precision, Effort effort)
    : PlanR2C(pencil, MPI_COMM_WORLD, precision, effort) {}
PlanR2C::PlanR2C(const Pencil& pencil, MPI_Comm comm, Precision precision, Effort effort, Executor executor) {
    _plan = nullptr;
    DTFFT_CXX_CALL(
        E(dtfft_create_plan_r2c_pencil(&pencil.c_struct(), comm, cp(precision), ce(effort), cx(executor), &_plan)))
}

PlanR2R::PlanR2R(const std::vector<int32_t>& dims, const std::vector<R2RKind>& kinds, MPI_Comm comm,
                 Precision precision, Effort effort, Executor executor)
    : PlanR2R(static_cast<int8_t>(dims.size()), dims.data(), kinds_or_null(kinds), comm, precision, effort, executor) {}
PlanR2R::PlanR2R(const std::vector<int32_t>& dims, Precision precision, Effort effort)
    : PlanR2R(static_cast<int8_t>(dims.size()), dims.data(), nullptr, MPI_COMM_WORLD, precision, effort) {}
PlanR2R::PlanR2R(int8_t ndims, const int32_t* dims, const R2RKind* kinds, MPI_Comm comm, Precision precision,
                 Effort effort, Executor executor) {
    _plan = nullptr;
    DTFFT_CXX_CALL(
        E(dtfft_create_plan_r2r(ndims, dims, ck(kinds), comm, cp(precision), ce(effort), cx(executor), &_plan)))
}
PlanR2R::PlanR2R(const Pencil& pencil, Precision precision, Effort effort)
    : PlanR2R(pencil, static_cast<const R2RKind*>(nullptr), MPI_COMM_WORLD, precision, effort) {}
PlanR2R::PlanR2R(const Pencil& pencil, const std::vector<R2RKind>& kinds, MPI_Comm comm, Precision precision,
                 Effort effort, Executor executor)
    : PlanR2R(pencil, kinds_or_null(kinds), comm, precision, effort, executor) {}
PlanR2R::PlanR2R(const Pencil& pencil, const R2RKind* kinds, MPI_Comm comm, Precision precision, Effort effort,
                 Executor executor) {
    _plan = nullptr;
    DTFFT_CXX_CALL(E(dtfft_create_plan_r2r_pencil(&pencil.c_struct(), ck(kinds), comm, cp(precision), ce(effort),
                                                 cx(executor), &_plan)))
}

}  // namespace dtfft
