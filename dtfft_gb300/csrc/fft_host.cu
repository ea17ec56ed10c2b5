// Host side of the FFT executor: schedules, twiddle tables, launch shapes,
// and the fused FFT + transpose steps.  Kernels live in fft_kernels.cuh.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <sstream>

#include "fft_2f.cuh"
#include "fft_kernels.cuh"
#include "fft_tile.cuh"

namespace gb {

// Status words of the bounded waits, one per device, in pinned host memory
// that every device can write (portable + mapped; with unified addressing the
// host pointer is also the device pointer on every device).  A kernel whose
// wait gives up stores its code there; the host reads it without
// synchronising at the next entry point on that device (check_device_status).
static constexpr int kStatusDevices = 64;
static int* g_status = nullptr;
static dtfft_error_t g_status_err = DTFFT_SUCCESS;
static std::once_flag g_status_once;

dtfft_error_t status_setup() {
    std::call_once(g_status_once, [] {
        void* p = nullptr;
        if (cudaHostAlloc(&p, sizeof(int) * kStatusDevices, cudaHostAllocPortable | cudaHostAllocMapped) != cudaSuccess) {
            cudaGetLastError();
            g_status_err = DTFFT_ERROR_GPU_CALL_FAILED;
            return;
        }
        void* d = nullptr;
        if (cudaHostGetDevicePointer(&d, p, 0) != cudaSuccess || d != p) {
            cudaGetLastError();
            cudaFreeHost(p);
            g_status_err = DTFFT_ERROR_GPU_CALL_FAILED;
            return;
        }
        memset(p, 0, sizeof(int) * kStatusDevices);
        g_status = (int*)p;
    });
    return g_status_err;
}

static int current_device() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); dev = 0; }
    return (dev >= 0 && dev < kStatusDevices) ? dev : kStatusDevices - 1;
}

// Status word of the current device.  Plan, kernel and executor creation call
// status_setup() first, so a launch never allocates here.
static int* status_ptr() {
    if (!g_status && status_setup() != DTFFT_SUCCESS) return nullptr;
    return g_status + current_device();
}

int* gb_status_word() { return status_ptr(); }

// Wait limit of the tile kernels' consumer waits (tests shorten it).
int g_wait_limit = kWaitLimitDefault;

dtfft_error_t check_device_status() {
    if (!g_status) return DTFFT_SUCCESS;
    volatile int* w = g_status + current_device();
    const int v = *w;
    if (v == 0) return DTFFT_SUCCESS;
    *w = 0;
    fprintf(stderr, "dtFFT-gb300: an earlier kernel on this device gave up a bounded wait (code %d); "
                    "its output was incomplete\n", v);
    return DTFFT_ERROR_GPU_WAIT_TIMEOUT;
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
std::string Schedule::str() const {
    std::ostringstream o;
    for (size_t i = 0; i < radix.size(); ++i) o << (i ? "x" : "") << radix[i];
    return o.str();
}

bool make_schedule(int m, Schedule& s) {
    s.m = m;
    s.radix.clear();
    int r = m;
    while (r % 8 == 0) { s.radix.push_back(8); r /= 8; }
    if (r % 4 == 0) { s.radix.push_back(4); r /= 4; }
    if (r % 2 == 0) { s.radix.push_back(2); r /= 2; }
    const int small[] = {3, 5, 7};
    for (int p : small) while (r % p == 0) { s.radix.push_back(p); r /= p; }
    for (int p = 11; p <= 127 && r > 1; p += 2) {
        bool prime = true;
        for (int q = 3; q * q <= p; q += 2) if (p % q == 0) { prime = false; break; }
        if (!prime) continue;
        while (r % p == 0) { s.radix.push_back(p); r /= p; }
    }
    if (r != 1) return false;
    if (s.radix.size() > 26) return false;
    return true;
}

struct FftStep {
    bool cols = false;
    int dbl = 0;
    int mode = M_C2C;
    int sign = -1;
    // geometry
    i64 nsig = 0, idist = 0, odist = 0, plane = 0;
    int ld = 0, ncols = 0, n = 0, m = 0, per = 1, pitch = 0;
    const void* tw = nullptr;
    const void* ta = nullptr;
    const void* tb = nullptr;
    Schedule sched;
    size_t smem = 0;
    int E = 0;               // points per thread of the register kernel, 0 = shared-memory kernel
    int threads = 256;
    bool pipe = false;       // C2C rows: persistent TMA-pipelined kernel when buffers are 16-byte aligned
    size_t pipe_smem = 0;
    int pipe_ctas_per_sm = 0;
    bool reads_out = false;  // step reads the plan's output buffer (second pass)
    void* tc = nullptr;      // tensor-core form of this step (C2C FP32 rows), see fft_tc.cu
    void* blue = nullptr;    // Bluestein form (a prime factor above 127), see fft_bluestein.cu
    bool tile = false;       // C2C rows: warp-per-row tile kernel (fft_tile.cuh)
    int tile_S = 0, tile_nst = 0, tile_threads = 0, tile_nw = 0;
    size_t tile_smem = 0;
    const void* tw_dir = nullptr;   // W_m^(sign*e) for this step's direction
    void* f2 = nullptr;      // C2C float: two-factor kernel (fft_2f.cuh), f2_m1 x f2_m2, f2_per signals per CTA
    int f2_m1 = 0, f2_m2 = 0, f2_per = 0, f2_threads = 256;
    size_t f2_smem = 0;
    // pipelined form of the two-factor rows (fft2f_pipe_kernel): f2 is that kernel, with a ring of
    // f2_nst buffers and at most f2_ctas CTAs per SM; f2_plain (f2_plain_per signals per CTA, 128
    // threads) runs the rows when the input is not 16-byte aligned
    bool f2_pipe = false;
    int f2_nst = 2, f2_ctas = 0, f2_plain_per = 0;
    void* f2_plain = nullptr;
    size_t f2_plain_smem = 0;
    ~FftStep() { tc_destroy(tc); blue_destroy(blue); }
};

static int g_fft_form = -1;

int fft_form() {
    if (g_fft_form < 0) {
        const char* e = getenv("DTFFT_GB_FFT_FORM");
        g_fft_form = (e && atoi(e) == 1) ? 1 : 0;
    }
    return g_fft_form;
}

// Register-kernel schedule: points per thread E (compiled counts below),
// radices dividing E, fewest stages first, then fewest registers.
// `prec`: 0 float, 1 double (the register kernels compiled for that
// precision), -1 the counts the fused kernels are compiled for.
static bool make_reg_schedule(int m, bool cols, int& E_out, Schedule& sch, int& T_out, int max_T = 256,
                              int prec = -1) {
    static const std::vector<int> Es_fused = {8, 16, 24, 20, 28};
    static const std::vector<int> Es_f32 = {8, 16, 24, 20, 28, 7, 9, 10, 12, 14, 15, 18, 21, 25, 30, 35, 42};
    static const std::vector<int> Es_f64 = {8, 16, 24, 20, 28, 7, 9, 10, 12, 14, 15, 18, 21, 25};
    const std::vector<int>& Es = prec < 0 ? Es_fused : (prec == 0 ? Es_f32 : Es_f64);
    static const int rads[] = {16, 8, 7, 5, 4, 3, 2};
    int best_stages = 1 << 30, best_E = 0;
    Schedule best;
    for (int E : Es) {
        if (m % E != 0) continue;
        const int T = m / E;
        if (T < 1 || T > max_T) continue;
        if (cols && T > 64) continue;
        Schedule s;
        s.m = m;
        int r = m;
        while (r > 1) {
            int pick = 0;
            for (int q : rads)
                if (E % q == 0 && r % q == 0) { pick = q; break; }
            if (!pick) break;
            s.radix.push_back(pick);
            r /= pick;
        }
        if (r != 1) continue;
        const int st = (int)s.radix.size();
        if (st < best_stages || (st == best_stages && E < best_E)) { best_stages = st; best_E = E; best = s; }
    }
    if (!best_E) return false;
    E_out = best_E;
    T_out = m / best_E;
    sch = best;
    return true;
}

static int mode_for_r2r(int kind) {
    switch (kind) {
    case DTFFT_DCT_1: return M_DCT1;
    case DTFFT_DCT_2: return M_DCT2;
    case DTFFT_DCT_3: return M_DCT3;
    case DTFFT_DCT_4: return M_DCT4;
    case DTFFT_DST_1: return M_DST1;
    case DTFFT_DST_2: return M_DST2;
    case DTFFT_DST_3: return M_DST3;
    case DTFFT_DST_4: return M_DST4;
    }
    return -1;
}

static int inverse_kind(int kind) {  // src/dtfft_utils.F90:447-471
    switch (kind) {
    case DTFFT_DCT_2: return DTFFT_DCT_3;
    case DTFFT_DCT_3: return DTFFT_DCT_2;
    case DTFFT_DST_2: return DTFFT_DST_3;
    case DTFFT_DST_3: return DTFFT_DST_2;
    default: return kind;
    }
}

// Core length and core sign of a mode for a signal of logical length n.
static bool mode_geometry(int mode, int n, int plan_sign, int& m, int& sign) {
    sign = plan_sign;
    switch (mode) {
    case M_C2C: m = n; break;
    case M_R2C_HALF: m = n / 2; sign = -1; break;
    case M_R2C_FULL: m = n; sign = -1; break;
    case M_C2R_HALF: m = n / 2; sign = 1; break;
    case M_C2R_FULL: m = n; sign = 1; break;
    case M_DCT1: if (n < 2) return false; m = 2 * (n - 1); sign = -1; break;
    case M_DST1: m = 2 * (n + 1); sign = -1; break;
    case M_DCT2: case M_DST2: m = n; sign = -1; break;
    case M_DCT3: case M_DST3: m = n; sign = 1; break;
    case M_DCT4: case M_DST4: m = 2 * n; sign = -1; break;
    case M_DCT2H: case M_DST2H: m = n / 2; sign = -1; break;
    case M_DCT3H: case M_DST3H: m = n / 2; sign = 1; break;
    default: return false;
    }
    return m >= 1;
}

// Host table of exp(-2*pi*i*j*num/den) for j < count, built in double precision.
static std::vector<double> table_exp(int count, long long num, long long den) {
    std::vector<double> t(2 * (size_t)count);
    for (int j = 0; j < count; ++j) {
        // reduce j*num mod den exactly before converting to an angle
        long long q = ((long long)j * num) % den;
        double ang = -2.0 * M_PI * (double)q / (double)den;
        t[2 * j] = std::cos(ang);
        t[2 * j + 1] = std::sin(ang);
    }
    return t;
}

static dtfft_error_t upload_table(const std::vector<double>& t, int dbl, std::vector<void*>& owned, const void** out) {
    size_t n = t.size();
    void* d = nullptr;
    if (dbl) {
        GB_CUDA_TRY(cudaMalloc(&d, n * sizeof(double)));
        GB_CUDA_TRY(cudaMemcpy(d, t.data(), n * sizeof(double), cudaMemcpyHostToDevice));
    } else {
        std::vector<float> f(n);
        for (size_t i = 0; i < n; ++i) f[i] = (float)t[i];
        GB_CUDA_TRY(cudaMalloc(&d, n * sizeof(float)));
        GB_CUDA_TRY(cudaMemcpy(d, f.data(), n * sizeof(float), cudaMemcpyHostToDevice));
    }
    owned.push_back(d);
    *out = d;
    return DTFFT_SUCCESS;
}

static const size_t kSmemBudget = 96 * 1024;

// Table of W_m^(sign*e), e < m, for one direction (the tile kernels take the
// direction's own table instead of conjugating on the fly).
static dtfft_error_t upload_dir_table(int m, int sign, int dbl, std::vector<void*>& owned, const void** out) {
    std::vector<double> t = table_exp(m, 1, m);
    if (sign > 0)
        for (int j = 0; j < m; ++j) t[2 * (size_t)j + 1] = -t[2 * (size_t)j + 1];
    return upload_table(t, dbl, owned, out);
}

static size_t max_optin_smem();

// Launch shape of the warp-per-row tile kernel for rows of m points: rows per
// tile S (one 128-byte run per point when the tile is written transposed),
// ring depth, threads.  False when no variant is compiled for m or the ring
// cannot hold two tiles.
struct TileShape { int E = 0, S = 0, nst = 0, threads = 0; size_t smem = 0; };
static int sm_count();

// rows: rows the launch transforms (0 = unknown).  Tiles shrink (down to 2
// rows, 1 for complex128 rows without a transpose) while there would be
// fewer than two per SM, so small transforms still spread over every SM.
static bool tile_shape(int m, int dbl, bool xpose, TileShape& ts, i64 rows = 0) {
    const int E = dbl ? TilePtr<double>::points_per_thread(m) : TilePtr<float>::points_per_thread(m);
    if (!E || getenv("DTFFT_GB_NO_TILE")) return false;
    const size_t es = dbl ? 16 : 8;
    const size_t cap = max_optin_smem();
    const size_t hdr = xpose ? kTileHdrXpose : kTileHdrPlain;
    int S = dbl ? 8 : 16;
    if (const char* e = getenv("DTFFT_GB_TILE_S")) {   // measurements: rows per tile
        const int v = atoi(e);
        if (v >= 2 && v <= S && (v & (v - 1)) == 0) S = v;
    }
    while (S > 2 && hdr + 2 * (size_t)S * m * es > cap) S >>= 1;
    const int smin = (dbl && !xpose) ? 1 : 2;
    while (rows > 0 && S > smin && (rows + S - 1) / S < 2 * (i64)sm_count()) S >>= 1;
    const size_t tile = (size_t)S * m * es;
    const int nst = (int)std::min<size_t>(kTileMaxNst, (cap - hdr) / tile);
    if (nst < 2) return false;
    ts.E = E; ts.S = S; ts.nst = nst;
    ts.threads = dbl ? TilePtr<double>::default_threads(m, xpose) : TilePtr<float>::default_threads(m, xpose);
    if (!xpose) ts.threads = std::min(ts.threads, 32 * S);
    ts.smem = hdr + (size_t)nst * tile;
    return true;
}

// Fill geometry, tables and launch shape of one step.
static int pipe_occupancy(int dbl, int m, int E, bool fused, int threads, size_t smem);

// Kernel attributes are set when a plan is built, never on the launch path:
// execute then only enqueues kernels (and can be captured into a CUDA graph).
// A kernel's dynamic shared memory limit is shared by every plan that uses the
// kernel, so it only ever grows: a later plan with a smaller need must not
// lower the limit an earlier plan launches with.
static std::mutex g_attr_mu;
static std::map<const void*, size_t> g_attr_smem;

static size_t max_optin_smem() {
    static size_t v = 0;
    if (!v) {
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess || n <= 0) n = 48 * 1024;
        v = (size_t)n;
    }
    return v;
}

static dtfft_error_t set_smem_attrs(const void* fn, size_t smem) {
    if (!fn) return DTFFT_ERROR_FFT_SIZE_NOT_SUPPORTED;
    if (smem > max_optin_smem()) return DTFFT_ERROR_FFT_SIZE_NOT_SUPPORTED;   // the variant cannot launch
    std::lock_guard<std::mutex> lk(g_attr_mu);
    auto it = g_attr_smem.find(fn);
    if (it == g_attr_smem.end()) {
        // favour shared memory over L1 so several CTAs fit per SM
        GB_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout,
                                         (int)cudaSharedmemCarveoutMaxShared));
        it = g_attr_smem.emplace(fn, 48 * 1024).first;
    }
    if (smem > it->second) {
        GB_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        it->second = smem;
    }
    return DTFFT_SUCCESS;
}

static int sm_count();

static dtfft_error_t prepare_launch(const FftStep& S) {
    (void)sm_count();
    GB_TRY(status_setup());
    const void* fn;
    if (S.E) fn = S.dbl ? (const void*)KPtr<double>::reg(S.E, S.cols, S.mode == M_C2C)
                        : (const void*)KPtr<float>::reg(S.E, S.cols, S.mode == M_C2C);
    else fn = S.dbl ? (const void*)KPtr<double>::generic(S.cols) : (const void*)KPtr<float>::generic(S.cols);
    return set_smem_attrs(fn, S.smem);
}

static dtfft_error_t upload_mode_tables(FftStep& S, std::vector<void*>& owned);
static void f2_prefer(FftStep& S, std::vector<void*>& owned);

static dtfft_error_t prepare_step(FftStep& S, std::vector<void*>& owned) {
    // DCT/DST-II and -III of even length through an n/2-point complex FFT when
    // the register kernel has a schedule for n/2 (half the arithmetic)
    if ((S.mode == M_DCT2 || S.mode == M_DST2 || S.mode == M_DCT3 || S.mode == M_DST3) && S.n % 2 == 0 &&
        S.n >= 8 && !getenv("DTFFT_GB_NO_HALF_DCT") && !getenv("DTFFT_GB_NO_REG_FFT")) {
        int E0 = 0, T0 = 0;
        Schedule s0;
        if (make_reg_schedule(S.n / 2, S.cols, E0, s0, T0, 256, S.dbl))
            S.mode = S.mode == M_DCT2 ? M_DCT2H : S.mode == M_DST2 ? M_DST2H : S.mode == M_DCT3 ? M_DCT3H : M_DST3H;
    }
    int m, sign;
    if (!mode_geometry(S.mode, S.n, S.sign, m, sign)) return DTFFT_ERROR_FFT_SIZE_NOT_SUPPORTED;
    S.m = m;
    S.sign = sign;
    const size_t es = S.dbl ? 16 : 8;
    int E = 0, T = 0;
    if (!getenv("DTFFT_GB_NO_REG_FFT") && make_reg_schedule(m, S.cols, E, S.sched, T, 256, S.dbl)) {
        S.E = E;
        // S signals per CTA, blockDim = S*T (signals past the end are masked)
        S.per = std::max(1, 256 / T);
        S.threads = S.per * T;
        S.pitch = m + m / 16;
        S.smem = S.cols ? (size_t)m * S.per * es : (size_t)S.per * S.pitch * es;
        // contiguous C2C rows stream through the TMA pipeline (2 buffers in flight)
        if (!S.cols && S.mode == M_C2C && S.idist == m && S.odist == m && (m * es) % 16 == 0 &&
            !getenv("DTFFT_GB_NO_PIPE")) {
            S.pipe_smem = 128 + 2 * (size_t)S.per * m * es + S.smem;
            S.pipe_ctas_per_sm = pipe_occupancy(S.dbl, S.m, S.E, false, S.threads, S.pipe_smem);
            S.pipe = S.pipe_ctas_per_sm > 0;
        }
    } else if (!make_schedule(m, S.sched)) {
        // a prime factor above the direct butterflies: Bluestein's chirp-z form
        const bool r2r = S.mode >= M_DCT1 && S.mode <= M_DST4;
        const int kind = S.mode == M_C2C ? 0 : S.mode == M_R2C_FULL ? 1 : S.mode == M_C2R_FULL ? 2 : r2r ? 3 : -1;
        if (kind < 0) return DTFFT_ERROR_FFT_SIZE_NOT_SUPPORTED;
        if (r2r) GB_TRY(upload_mode_tables(S, owned));
        return blue_create(S.dbl, m, sign, kind, S.nsig, S.idist, S.odist, S.plane, S.ld, S.ncols, S.cols ? 1 : 0,
                           &S.blue, S.mode, S.n, S.ta, S.tb);
    }
    if (fft_form() == 1 && !S.cols && !S.dbl && S.mode == M_C2C && S.idist == m && S.odist == m && tc_supported(m))
        GB_TRY(tc_create(m, &S.tc));
    if (!S.cols && S.mode == M_C2C && S.idist == m && S.odist == m) {
        TileShape ts;
        if (tile_shape(m, S.dbl, false, ts, S.nsig)) {
            int nw = 0;
            if (const char* tw_env = getenv("DTFFT_GB_TILE_WARPS")) {   // experiments
                const int w = atoi(tw_env);
                if (w > 0 && (S.dbl ? TilePtr<double>::get(m, sign, false, w) : TilePtr<float>::get(m, sign, false, w)))
                    nw = w;
            }
            const void* fn = S.dbl ? TilePtr<double>::get(m, sign, false, nw) : TilePtr<float>::get(m, sign, false, nw);
            if (fn && set_smem_attrs(fn, ts.smem) == DTFFT_SUCCESS) {
                S.tile = true;
                S.tile_S = ts.S; S.tile_nst = ts.nst; S.tile_threads = nw ? 32 * nw : ts.threads; S.tile_smem = ts.smem;
                S.tile_nw = nw;
                GB_TRY(upload_dir_table(m, sign, S.dbl, owned, &S.tw_dir));
            }
        }
    }
    if (S.E) goto tables;
    {
    const size_t per_sig = 2 * (size_t)m * es;   // ping-pong buffers
    if (per_sig > 220 * 1024) return DTFFT_ERROR_FFT_SIZE_NOT_SUPPORTED;
    int per;
    if (S.cols) {
        per = S.dbl ? 8 : 16;
        while (per > 1 && per * per_sig > 200 * 1024) per >>= 1;
        per = std::min<i64>(per, S.ncols);
        S.pitch = per;
    } else {
        per = (int)std::max<size_t>(1, kSmemBudget / per_sig);
        // keep at least ~2 CTAs per SM worth of work when the batch is small
        i64 want = std::max<i64>(1, S.nsig / (152 * 4));
        per = (int)std::max<i64>(1, std::min<i64>(per, want));
        per = std::min(per, 64);
        S.pitch = m;
    }
    S.per = std::max(1, per);
    S.smem = (size_t)S.per * per_sig;
    }
tables:
    // tables
    std::vector<double> tw = table_exp(m, 1, m);
    GB_TRY(upload_table(tw, S.dbl, owned, &S.tw));
    GB_TRY(upload_mode_tables(S, owned));
    return prepare_launch(S);
}

// Pre/post-processing tables of the step's mode (S.ta, S.tb).
static dtfft_error_t upload_mode_tables(FftStep& S, std::vector<void*>& owned) {
    const int m = S.m;
    switch (S.mode) {
    case M_R2C_HALF: GB_TRY(upload_table(table_exp(m + 1, 1, S.n), S.dbl, owned, &S.ta)); break;
    case M_C2R_HALF: GB_TRY(upload_table(table_exp(m, 1, S.n), S.dbl, owned, &S.ta)); break;
    case M_DCT2: case M_DST2: case M_DCT3: case M_DST3:
        GB_TRY(upload_table(table_exp(S.n, 1, 4LL * S.n), S.dbl, owned, &S.ta)); break;
    case M_DCT2H: case M_DST2H:
        GB_TRY(upload_table(table_exp(m + 1, 1, S.n), S.dbl, owned, &S.ta));
        GB_TRY(upload_table(table_exp(S.n, 1, 4LL * S.n), S.dbl, owned, &S.tb));
        break;
    case M_DCT3H: case M_DST3H:
        GB_TRY(upload_table(table_exp(m, 1, S.n), S.dbl, owned, &S.ta));
        GB_TRY(upload_table(table_exp(S.n, 1, 4LL * S.n), S.dbl, owned, &S.tb));
        break;
    case M_DCT4: case M_DST4: {
        GB_TRY(upload_table(table_exp(S.n, 1, 4LL * S.n), S.dbl, owned, &S.ta));
        std::vector<double> t(2 * (size_t)S.n);
        for (int k = 0; k < S.n; ++k) {
            long long q = (2LL * k + 1) % (8LL * S.n);
            double ang = -2.0 * M_PI * (double)q / (8.0 * S.n);
            t[2 * k] = std::cos(ang); t[2 * k + 1] = std::sin(ang);
        }
        GB_TRY(upload_table(t, S.dbl, owned, &S.tb));
    } break;
    default: break;
    }
    return DTFFT_SUCCESS;
}

template <typename R, bool FUSED>
static void (*pipe_fn(int m, int E))(PArgs<R>) {
    return (void (*)(PArgs<R>))KPtr<R>::pipe(m, E, FUSED);
}

// CTAs of the pipelined kernel that fit one SM (0 when it cannot launch).
static int pipe_occupancy(int dbl, int m, int E, bool fused, int threads, size_t smem) {
    int n = 0;
    auto one = [&](auto fn) {
        if (!fn) return;
        if (set_smem_attrs((const void*)fn, smem) != DTFFT_SUCCESS) return;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, threads, smem) != cudaSuccess) n = 0;
    };
    if (dbl) { if (fused) one(pipe_fn<double, true>(m, E)); else one(pipe_fn<double, false>(m, E)); }
    else { if (fused) one(pipe_fn<float, true>(m, E)); else one(pipe_fn<float, false>(m, E)); }
    cudaGetLastError();
    return n;
}

static int sm_count() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 1;
    }
    return n;
}

template <typename R, bool FUSED>
static dtfft_error_t launch_pipe(const PArgs<R>& P, int E, int threads, size_t smem, int per_sm, cudaStream_t s) {
    void (*kfn)(PArgs<R>) = pipe_fn<R, FUSED>(P.m, E);
    if (!kfn || per_sm <= 0) return DTFFT_ERROR_FFT_SIZE_NOT_SUPPORTED;
    const i64 grid = std::min<i64>(P.ntiles, (i64)sm_count() * per_sm);
    const_cast<PArgs<R>&>(P).status = status_ptr();
    if (grid <= 0) return DTFFT_SUCCESS;
    kfn<<<(unsigned)grid, threads, smem, s>>>(P);
    return DTFFT_SUCCESS;
}

template <typename R, bool COLS>
static dtfft_error_t launch_step_t(const FftStep& S, const void* in, void* out, cudaStream_t s) {
    if (S.blue) return blue_execute(S.blue, in, out, s);
    if (S.f2 && S.f2_pipe && ((uintptr_t)in % 16) == 0) {
        F2PArgs<R> P;
        P.in = (const typename CT<R>::T*)in; P.out = (typename CT<R>::T*)out; P.tw = (const typename CT<R>::T*)S.tw;
        P.nsig = S.nsig; P.per = S.f2_per; P.ntiles = (S.nsig + S.f2_per - 1) / S.f2_per; P.nst = S.f2_nst;
        P.sign = S.sign; P.wait_limit = g_wait_limit; P.status = status_ptr();
        if (P.ntiles <= 0) return DTFFT_SUCCESS;
        const i64 grid = std::min<i64>(P.ntiles, (i64)sm_count() * S.f2_ctas);
        void (*kfn)(F2PArgs<R>) = (void (*)(F2PArgs<R>))S.f2;
        void* tok = prof_begin(s);
        kfn<<<(unsigned)grid, S.f2_threads, S.f2_smem, s>>>(P);
        if (tok) prof_end(tok, std::string("fft2f_pipe_c2c_m") + std::to_string(S.m) + "_f32", s);
        count_launch();
        GB_CUDA_TRY(cudaGetLastError());
        return DTFFT_SUCCESS;
    }
    if (S.f2) {
        const bool plain = S.f2_pipe;   // unaligned input of a pipelined step
        F2Args<R> F;
        F.in = in; F.out = out; F.tw = (const typename CT<R>::T*)S.tw; F.ta = (const typename CT<R>::T*)S.ta;
        F.n = S.n; F.nsig = S.nsig; F.idist = S.idist; F.odist = S.odist; F.plane = S.plane; F.ld = S.ld; F.ncols = S.ncols;
        F.sign = S.sign; F.per = plain ? S.f2_plain_per : S.f2_per;
        const i64 ctas = (S.nsig + F.per - 1) / F.per;
        if (ctas <= 0) return DTFFT_SUCCESS;
        if (ctas > 0x7fffffffLL) return DTFFT_ERROR_FFT_SIZE_NOT_SUPPORTED;
        void (*kfn)(F2Args<R>) = (void (*)(F2Args<R>))(plain ? S.f2_plain : S.f2);
        void* tok = prof_begin(s);
        kfn<<<(unsigned)ctas, plain ? 128 : S.f2_threads, plain ? S.f2_plain_smem : S.f2_smem, s>>>(F);
        if (tok) {
            static const char* mn[] = {"c2c", "r2c", "r2c", "c2r", "c2r"};
            prof_end(tok, std::string("fft2f_") + (COLS ? "cols_" : "rows_") + mn[S.mode] + "_m" + std::to_string(S.m) +
                              "_f32", s);
        }
        count_launch();
        GB_CUDA_TRY(cudaGetLastError());
        return DTFFT_SUCCESS;
    }
    if (S.tc) {
        void* tok = prof_begin(s);
        GB_TRY(tc_execute(S.tc, in, out, S.nsig, S.sign, status_ptr(), s));
        if (tok) prof_end(tok, std::string("ffttc_rows_c2c_m") + std::to_string(S.m) + "_f32", s);
        count_launch();
        GB_CUDA_TRY(cudaGetLastError());
        return DTFFT_SUCCESS;
    }
    Args<R> A;
    typedef typename CT<R>::T C;
    if (!COLS && S.tile && ((uintptr_t)in % 16) == 0 && ((uintptr_t)out % 16) == 0) {
        TArgs<R> P;
        P.in = (const C*)in; P.out = (C*)out; P.tw = (const C*)S.tw_dir;
        P.nsig = S.nsig; P.groups = nullptr; P.segs = nullptr; P.ngroups = 0;
        P.ntiles = (S.nsig + S.tile_S - 1) / S.tile_S;
        P.S = S.tile_S; P.nst = S.tile_nst; P.pair_ok = 0; P.wait_limit = g_wait_limit; P.status = status_ptr();
        P.wfast = 0;
        void (*kfn)(TArgs<R>) = (void (*)(TArgs<R>))TilePtr<R>::get(S.m, S.sign, false, S.tile_nw);
        if (!kfn) return DTFFT_ERROR_FFT_SIZE_NOT_SUPPORTED;
        const i64 grid = std::min<i64>(P.ntiles, (i64)sm_count());
        if (grid <= 0) return DTFFT_SUCCESS;
        void* tok = prof_begin(s);
        kfn<<<(unsigned)grid, S.tile_threads, S.tile_smem, s>>>(P);
        if (tok) prof_end(tok, std::string("ffttile_rows_c2c_m") + std::to_string(S.m) + (sizeof(R) == 8 ? "_f64" : "_f32"), s);
        count_launch();
        GB_CUDA_TRY(cudaGetLastError());
        return DTFFT_SUCCESS;
    }
    if (!COLS && S.pipe && S.pipe_ctas_per_sm > 0 && ((uintptr_t)in % 16) == 0 && ((uintptr_t)out % 16) == 0) {
        PArgs<R> P;
        P.in = (const C*)in; P.out = (C*)out;
        P.nsig = S.nsig; P.groups = nullptr; P.segs = nullptr; P.ngroups = 0;
        P.ntiles = (S.nsig + S.per - 1) / S.per;
        P.m = S.m; P.sign = S.sign; P.S = S.per; P.pitch = S.pitch; P.nst = 2; P.tw = (const C*)S.tw;
        P.st.ns = (int)S.sched.radix.size();
        for (int i = 0; i < P.st.ns; ++i) P.st.radix[i] = S.sched.radix[i];
        void* tok = prof_begin(s);
        GB_TRY((launch_pipe<R, false>(P, S.E, S.threads, S.pipe_smem, S.pipe_ctas_per_sm, s)));
        if (tok) prof_end(tok, std::string("fftpipe_rows_c2c_m") + std::to_string(S.m) + (sizeof(R) == 8 ? "_f64" : "_f32"), s);
        count_launch();
        GB_CUDA_TRY(cudaGetLastError());
        return DTFFT_SUCCESS;
    }
    A.in = (const char*)in; A.out = (char*)out;
    A.nsig = S.nsig; A.idist = S.idist; A.odist = S.odist; A.plane = S.plane;
    A.ld = S.ld; A.ncols = S.ncols; A.n = S.n; A.m = S.m; A.mode = S.mode; A.sign = S.sign;
    A.per_cta = S.per; A.pitch = S.pitch;
    A.tw = (const C*)S.tw; A.ta = (const C*)S.ta; A.tb = (const C*)S.tb;
    A.st.ns = (int)S.sched.radix.size();
    for (int i = 0; i < A.st.ns; ++i) A.st.radix[i] = S.sched.radix[i];
    const i64 ctas = (S.nsig + S.per - 1) / S.per;
    if (ctas <= 0) return DTFFT_SUCCESS;
    if (ctas > 0x7fffffffLL) return DTFFT_ERROR_FFT_SIZE_NOT_SUPPORTED;
    void* tok = prof_begin(s);
    if (S.E) {
        const bool c2c = S.mode == M_C2C;
        void (*kfn)(Args<R>) = (void (*)(Args<R>))KPtr<R>::reg(S.E, COLS, c2c);
        if (!kfn) return DTFFT_ERROR_FFT_SIZE_NOT_SUPPORTED;
        kfn<<<(unsigned)ctas, S.threads, S.smem, s>>>(A);
    } else {
        void (*gfn)(Args<R>) = (void (*)(Args<R>))KPtr<R>::generic(COLS);
        gfn<<<(unsigned)ctas, 256, S.smem, s>>>(A);
    }
    if (tok) {
        static const char* mn[] = {"c2c", "r2c", "r2c", "c2r", "c2r", "dct1", "dct2", "dct3", "dct4",
                                   "dst1", "dst2", "dst3", "dst4", "dct2h", "dst2h", "dct3h", "dst3h"};
        prof_end(tok, std::string(S.E ? "fftreg_" : "fft_") + (COLS ? "cols_" : "rows_") + mn[S.mode] + "_m" +
                          std::to_string(S.m) + (sizeof(R) == 8 ? "_f64" : "_f32"), s);
    }
    count_launch();
    GB_CUDA_TRY(cudaGetLastError());
    return DTFFT_SUCCESS;
}

static dtfft_error_t launch_step(const FftStep& S, const void* in, void* out, cudaStream_t s) {
    if (S.dbl) return S.cols ? launch_step_t<double, true>(S, in, out, s) : launch_step_t<double, false>(S, in, out, s);
    return S.cols ? launch_step_t<float, true>(S, in, out, s) : launch_step_t<float, false>(S, in, out, s);
}

dtfft_error_t FftPlan::create(const FftDesc& d, FftPlan** out) {
    *out = nullptr;
    if (d.rank != 1 && d.rank != 2) return DTFFT_ERROR_INVALID_USAGE;
    if (d.n_fast < 1 || d.n_slow < 1 || d.batch < 0) return DTFFT_ERROR_INVALID_DIMENSION_SIZE;
    FftPlan* p = new FftPlan();
    p->d_ = d;
    dtfft_error_t e = p->build(FFT_FWD, p->fwd_);
    if (e == DTFFT_SUCCESS) e = p->build(FFT_BWD, p->bwd_);
    if (e != DTFFT_SUCCESS) { delete p; return e; }
    p->launches_ = (int)p->fwd_.size();
    *out = p;
    return DTFFT_SUCCESS;
}

FftPlan::~FftPlan() {
    for (auto* s : fwd_) delete s;
    for (auto* s : bwd_) delete s;
    for (void* t : tables_) cudaFree(t);
}

// Steps of one direction:
//   rank 1: one row step (any mode)
//   rank 2: row step along n_fast, then an in-place column step along n_slow
//           (C2R runs the column step first, on the input, then the row step)
dtfft_error_t FftPlan::build(int sign, std::vector<FftStep*>& steps) {
    const FftDesc& d = d_;
    const int nf = d.n_fast, ns = d.n_slow;
    const i64 planes = d.batch;
    // row step
    FftStep* row = new FftStep();
    row->dbl = d.dbl; row->cols = false; row->sign = sign; row->n = nf;
    row->nsig = planes * (d.rank == 2 ? ns : 1);
    int row_ld_out = nf;  // complex row length after the row step (for the column step)
    i64 in_row = d.rank == 2 ? 0 : d.idist, out_row = d.rank == 2 ? 0 : d.odist;
    switch (d.type) {
    case FFT_C2C:
        row->mode = M_C2C;
        if (d.rank == 2) { in_row = nf; out_row = nf; }
        break;
    case FFT_R2C:
        if (sign == FFT_FWD) row->mode = (nf % 2 == 0) ? M_R2C_HALF : M_R2C_FULL;
        else row->mode = (nf % 2 == 0) ? M_C2R_HALF : M_C2R_FULL;
        row_ld_out = nf / 2 + 1;
        if (d.rank == 2) {
            if (sign == FFT_FWD) { in_row = nf; out_row = nf / 2 + 1; }
            else { in_row = nf / 2 + 1; out_row = nf; }
        }
        break;
    case FFT_R2R: {
        int kind = sign == FFT_FWD ? d.kind_fast : inverse_kind(d.kind_fast);
        row->mode = mode_for_r2r(kind);
        if (row->mode < 0) { delete row; return DTFFT_ERROR_INVALID_R2R_KINDS; }
        if (d.rank == 2) { in_row = nf; out_row = nf; }
    } break;
    default: delete row; return DTFFT_ERROR_INVALID_USAGE;
    }
    // rank 1: idist/odist describe the forward (real -> complex) direction;
    // the C2R step reads complex rows odist apart and writes real rows idist apart
    if (d.rank == 1 && d.type == FFT_R2C && sign == FFT_BWD) std::swap(in_row, out_row);
    row->idist = in_row; row->odist = out_row;
    dtfft_error_t e = prepare_step(*row, tables_);
    if (e != DTFFT_SUCCESS) { delete row; return e; }
    f2_prefer(*row, tables_);

    FftStep* col = nullptr;
    if (d.rank == 2) {
        col = new FftStep();
        col->dbl = d.dbl; col->cols = true; col->sign = sign; col->n = ns;
        col->ncols = row_ld_out; col->ld = row_ld_out;
        col->plane = (i64)ns * row_ld_out;
        col->nsig = planes * row_ld_out;
        if (d.type == FFT_R2R) {
            int kind = sign == FFT_FWD ? d.kind_slow : inverse_kind(d.kind_slow);
            col->mode = mode_for_r2r(kind);
            if (col->mode < 0) { delete row; delete col; return DTFFT_ERROR_INVALID_R2R_KINDS; }
        } else {
            col->mode = M_C2C;
        }
        e = prepare_step(*col, tables_);
        if (e != DTFFT_SUCCESS) { delete row; delete col; return e; }
        f2_prefer(*col, tables_);
    }
    if (d.rank == 2 && d.type == FFT_R2C && sign == FFT_BWD) {
        col->reads_out = false;
        steps.push_back(col);   // in place on the (destroyable) complex input
        steps.push_back(row);
    } else {
        steps.push_back(row);
        if (col) { col->reads_out = true; steps.push_back(col); }
    }
    return DTFFT_SUCCESS;
}

dtfft_error_t FftPlan::execute(const void* in, void* out, int sign, cudaStream_t s) {
    if (d_.batch == 0) return DTFFT_SUCCESS;
    const std::vector<FftStep*>& steps = sign == FFT_FWD ? fwd_ : bwd_;
    if (d_.rank == 1) return launch_step(*steps[0], in, out, s);
    if (d_.type == FFT_R2C && sign == FFT_BWD) {
        GB_TRY(launch_step(*steps[0], in, const_cast<void*>(in), s));
        return launch_step(*steps[1], in, out, s);
    }
    GB_TRY(launch_step(*steps[0], in, out, s));
    return launch_step(*steps[1], out, out, s);
}

// ---------------------------------------------------------------------------
// Measured choice of every FFT step's kernel and schedule (EXHAUSTIVE plans)
// ---------------------------------------------------------------------------
// Replaces the reference's NVRTC block optimizer for the FFT side
// (src/dtfft_nvrtc_block_optimizer.F90:502-751 scores candidates analytically,
// src/dtfft_kernel_device.F90:259-411 times them under EXHAUSTIVE): for each
// step the candidates are
//   tile   the warp-per-row tile kernel (C2C rows of a compiled length) with
//          S rows per tile and a ring of nst tiles,
//   reg    the register kernel for every compiled points-per-thread count E
//          and several radix orders, with 256 / T or 128 / T signals per CTA,
//   pipe   the same register schedules on the bulk-copy pipelined kernel,
//   smem   the shared-memory kernel,
// each timed with CUDA events on scratch buffers of the step's footprint; the
// fastest is kept.  Choices are cached per (GPU, library version, step
// geometry) in the process and, with DTFFT_GB_TUNE_CACHE, in that file.
struct StepCand {
    enum Kind { TILE, PIPE, REG, SMEM, F2, F2P } kind = SMEM;
    int E = 0, per = 1, S = 0, nst = 0;
    std::vector<int> radix;
    std::string name() const {
        std::ostringstream o;
        switch (kind) {
        case TILE: o << "tile:S" << S << ":nst" << nst; break;
        case SMEM: o << "smem"; break;
        case F2: o << "f2:t" << S << ":per" << per; break;
        case F2P: o << "f2p:t" << S << ":per" << per << ":nst" << nst; break;
        default: {
            o << (kind == PIPE ? "pipe:E" : "reg:E") << E << ":";
            for (size_t i = 0; i < radix.size(); ++i) o << (i ? "x" : "") << radix[i];
            o << ":per" << per;
        }
        }
        return o.str();
    }
    static bool parse(const std::string& t, StepCand& c) {
        c = StepCand();
        if (t == "smem") { c.kind = SMEM; return true; }
        if (t.compare(0, 4, "f2p:") == 0) {
            c.kind = F2P;
            return sscanf(t.c_str(), "f2p:t%d:per%d:nst%d", &c.S, &c.per, &c.nst) == 3 && c.per > 0 && c.per % 2 == 0 &&
                   (c.S == 128 || c.S == 256) && c.nst >= 2 && c.nst <= 4;
        }
        if (t.compare(0, 3, "f2:") == 0) {
            c.kind = F2;
            return sscanf(t.c_str(), "f2:t%d:per%d", &c.S, &c.per) == 2 && c.per > 0 &&
                   (c.S == 32 || c.S == 64 || c.S == 128 || c.S == 256);
        }
        if (t.compare(0, 5, "tile:") == 0) {
            c.kind = TILE;
            return sscanf(t.c_str(), "tile:S%d:nst%d", &c.S, &c.nst) == 2;
        }
        const bool pipe = t.compare(0, 5, "pipe:") == 0;
        if (!pipe && t.compare(0, 4, "reg:") != 0) return false;
        c.kind = pipe ? PIPE : REG;
        const size_t a = t.find(":E"), b = t.find(':', a + 2), d = t.find(":per");
        if (a == std::string::npos || b == std::string::npos || d == std::string::npos) return false;
        c.E = atoi(t.c_str() + a + 2);
        c.per = atoi(t.c_str() + d + 4);
        std::string rs = t.substr(b + 1, d - b - 1);
        for (size_t i = 0; i <= rs.size();) {
            size_t j = rs.find('x', i);
            if (j == std::string::npos) j = rs.size();
            c.radix.push_back(atoi(rs.substr(i, j - i).c_str()));
            i = j + 1;
        }
        return c.E > 0 && c.per > 0;
    }
};

// DCT/DST-II and -III through an n/2-point complex FFT: only the register
// kernels implement these modes.
static bool half_mode(int mode) { return mode == M_DCT2H || mode == M_DST2H || mode == M_DCT3H || mode == M_DST3H; }

// Greedy radix schedule of m for points-per-thread E with a radix preference.
static bool greedy_schedule(int m, int E, const std::vector<int>& pref, std::vector<int>& out) {
    out.clear();
    int r = m;
    while (r > 1) {
        int pick = 0;
        for (int q : pref)
            if (E % q == 0 && r % q == 0) { pick = q; break; }
        if (!pick) return false;
        out.push_back(pick);
        r /= pick;
    }
    return !out.empty() || m == 1;
}

// Set a step up for one candidate; false when the candidate cannot run.
static bool apply_cand(FftStep& S, const StepCand& c, std::vector<void*>& owned) {
    const size_t es = S.dbl ? 16 : 8;
    const int m = S.m;
    const bool c2c_rows = !S.cols && S.mode == M_C2C && S.idist == m && S.odist == m;
    S.tile = false;
    S.pipe = false;
    S.f2 = nullptr;
    S.f2_pipe = false;
    S.f2_plain = nullptr;
    switch (c.kind) {
    case StepCand::F2P: {
        int a = 0, b = 0, pa = 0, pb = 0;
        if (S.dbl || !c2c_rows || c.per < 2 || c.per % 2 || c.nst < 2 || c.nst > 4) return false;
        void* fn = f2_pipe_kernel_f32(m, &a, &b);
        void* plain = f2_kernel_f32(m, false, M_C2C, &pa, &pb);
        if (!fn || !plain) return false;
        const size_t smem = f2p_smem(a, b, c.per, c.nst, es);
        const int threads = c.S == 128 ? 128 : 256;
        if (smem > max_optin_smem() || set_smem_attrs(fn, smem) != DTFFT_SUCCESS) { cudaGetLastError(); return false; }
        int occ = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, threads, smem) != cudaSuccess || occ < 1) {
            cudaGetLastError();
            return false;
        }
        const int pper = std::max(1, (128 + std::min(pa, pb) - 1) / std::min(pa, pb) / 2);
        const size_t psmem = f2_smem(pa, pb, false, pper, es, M_C2C);
        if (set_smem_attrs(plain, psmem) != DTFFT_SUCCESS) { cudaGetLastError(); return false; }
        S.f2 = fn; S.f2_m1 = a; S.f2_m2 = b; S.f2_per = c.per; S.f2_smem = smem; S.f2_threads = threads;
        S.f2_pipe = true; S.f2_nst = c.nst; S.f2_ctas = occ;
        S.f2_plain = plain; S.f2_plain_per = pper; S.f2_plain_smem = psmem;
        return true;
    }
    case StepCand::F2: {
        int a = 0, b = 0;
        void* fn = (S.dbl || S.mode > M_C2R_FULL) ? nullptr : f2_kernel_f32(m, S.cols, S.mode, &a, &b);
        if (!fn || c.per < 1) return false;
        const size_t smem = f2_smem(a, b, S.cols, c.per, es, S.mode);
        if (smem > max_optin_smem() || set_smem_attrs(fn, smem) != DTFFT_SUCCESS) { cudaGetLastError(); return false; }
        S.f2 = fn; S.f2_m1 = a; S.f2_m2 = b; S.f2_per = c.per; S.f2_smem = smem;
        S.f2_threads = (c.S == 32 || c.S == 64 || c.S == 128) ? c.S : 256;
        return true;
    }
    case StepCand::TILE: {
        if (!c2c_rows) return false;
        const void* fn = S.dbl ? TilePtr<double>::get(m, S.sign, false) : TilePtr<float>::get(m, S.sign, false);
        if (!fn) return false;
        const size_t smem = kTileHdrPlain + (size_t)c.nst * c.S * m * es;
        if (c.nst < 2 || c.nst > kTileMaxNst || smem > max_optin_smem()) return false;
        if (set_smem_attrs(fn, smem) != DTFFT_SUCCESS) { cudaGetLastError(); return false; }
        if (!S.tw_dir && upload_dir_table(m, S.sign, S.dbl, owned, &S.tw_dir) != DTFFT_SUCCESS) return false;
        const int dthreads = S.dbl ? TilePtr<double>::default_threads(m, false) : TilePtr<float>::default_threads(m, false);
        S.tile = true;
        S.tile_S = c.S; S.tile_nst = c.nst; S.tile_nw = 0;
        S.tile_threads = std::min(dthreads, 32 * c.S);
        S.tile_smem = smem;
        return true;
    }
    case StepCand::REG:
    case StepCand::PIPE: {
        const bool c2c = S.mode == M_C2C;
        const void* fn = S.dbl ? KPtr<double>::reg(c.E, S.cols, c2c) : KPtr<float>::reg(c.E, S.cols, c2c);
        if (!fn || m % c.E) return false;
        int prod = 1;
        for (int r : c.radix) { if (c.E % r) return false; prod *= r; }
        if (prod != m) return false;
        const int T = m / c.E;
        if (c.per < 1 || c.per * T > 1024) return false;
        S.E = c.E;
        S.sched.m = m;
        S.sched.radix = c.radix;
        S.per = c.per;
        S.threads = c.per * T;
        S.pitch = m + m / 16;
        S.smem = S.cols ? (size_t)m * c.per * es : (size_t)c.per * S.pitch * es;
        if (S.smem > max_optin_smem() || set_smem_attrs(fn, S.smem) != DTFFT_SUCCESS) { cudaGetLastError(); return false; }
        if (c.kind == StepCand::PIPE) {
            if (!c2c_rows || (m * es) % 16) return false;
            S.pipe_smem = 128 + 2 * (size_t)c.per * m * es + S.smem;
            if (S.pipe_smem > max_optin_smem()) return false;
            S.pipe_ctas_per_sm = pipe_occupancy(S.dbl, m, c.E, false, S.threads, S.pipe_smem);
            if (S.pipe_ctas_per_sm <= 0) return false;
            S.pipe = true;
        }
        return true;
    }
    case StepCand::SMEM: {
        Schedule sc;
        if (half_mode(S.mode) || !make_schedule(m, sc)) return false;
        const size_t per_sig = 2 * (size_t)m * es;
        if (per_sig > 220 * 1024) return false;
        S.E = 0;
        S.sched = sc;
        int per;
        if (S.cols) {
            per = S.dbl ? 8 : 16;
            while (per > 1 && per * per_sig > 200 * 1024) per >>= 1;
            per = (int)std::min<i64>(per, S.ncols);
            S.pitch = per;
        } else {
            per = (int)std::max<size_t>(1, kSmemBudget / per_sig);
            i64 want = std::max<i64>(1, S.nsig / (152 * 4));
            per = (int)std::max<i64>(1, std::min<i64>(per, want));
            per = std::min(per, 64);
            S.pitch = m;
        }
        S.per = std::max(1, per);
        S.smem = (size_t)S.per * per_sig;
        const void* fn = S.dbl ? KPtr<double>::generic(S.cols) : KPtr<float>::generic(S.cols);
        if (set_smem_attrs(fn, S.smem) != DTFFT_SUCCESS) { cudaGetLastError(); return false; }
        return true;
    }
    }
    return false;
}

// C2C, R2C and C2R float steps without a tile kernel take the two-factor
// kernel when one is compiled for their core length (measured faster than the
// register, pipelined and shared-memory kernels on most such lengths;
// EXHAUSTIVE plans time them all).  DTFFT_GB_F2=0: never; DTFFT_GB_F2=1: also
// over the tile kernels.
static void f2_prefer(FftStep& S, std::vector<void*>& owned) {
    const char* e = getenv("DTFFT_GB_F2");
    const bool never = e && strcmp(e, "0") == 0, always = e && strcmp(e, "1") == 0;
    if (never || S.tc || S.blue || S.dbl || S.mode > M_C2R_FULL || (S.tile && !always)) return;
    int a = 0, b = 0;
    if (!f2_kernel_f32(S.m, S.cols, S.mode, &a, &b)) return;
    StepCand c;
    c.kind = StepCand::F2;
    // 128-thread CTAs of few signals (half of what fills the threads in the phase of the smaller
    // factor) measured fastest on rows: more CTAs per SM overlap their load and transform phases
    c.S = 128;
    if (const char* v = getenv("DTFFT_GB_F2_THREADS")) {   // measurements
        const int t = atoi(v);
        c.S = (t == 32 || t == 64 || t == 256) ? t : 128;
    }
    c.per = S.cols ? 32 : std::max(1, (c.S + std::min(a, b) - 1) / std::min(a, b) / 2);
    if (const char* v = getenv("DTFFT_GB_F2_PER")) c.per = std::max(1, atoi(v));
    // contiguous C2C rows: the pipelined form, 128 threads, a ring of two tiles of about
    // 1024 points (4-16 rows), measured 10-15 % faster than the unpipelined kernel
    // (DTFFT_GB_F2P=0: the unpipelined kernel; "threads,per,nst": that shape, for measurements)
    const bool c2c_rows = !S.cols && S.mode == M_C2C && S.idist == S.m && S.odist == S.m;
    StepCand cp;
    const char* pv = getenv("DTFFT_GB_F2P");
    if (c2c_rows && !(pv && strcmp(pv, "0") == 0) && f2_pipe_kernel_f32(S.m, nullptr, nullptr)) {
        cp.kind = StepCand::F2P; cp.S = 128; cp.nst = 2;
        cp.per = 2 * std::max(2, std::min(8, (512 + S.m / 2) / S.m));
        int nt = 0, per = 0, nst = 0;
        if (pv && sscanf(pv, "%d,%d,%d", &nt, &per, &nst) == 3) { cp.S = nt; cp.per = per; cp.nst = nst; }
    }
    for (const StepCand& k : {cp, c}) {
        if (k.kind != StepCand::F2P && k.kind != StepCand::F2) continue;
        FftStep t = S;
        t.tc = nullptr; t.blue = nullptr;
        const bool ok = apply_cand(t, k, owned);
        if (ok) S = t;
        t.tc = nullptr; t.blue = nullptr;
        if (ok) return;
    }
}

static std::vector<StepCand> step_candidates(const FftStep& S) {
    std::vector<StepCand> out;
    const int m = S.m;
    const size_t es = S.dbl ? 16 : 8;
    const bool c2c_rows = !S.cols && S.mode == M_C2C && S.idist == m && S.odist == m;
    if (c2c_rows && (S.dbl ? TilePtr<double>::get(m, S.sign, false) : TilePtr<float>::get(m, S.sign, false))) {
        for (int sr : {16, 8, 4, 2}) {
            if (sr > (S.dbl ? 8 : 16)) continue;
            const int maxn = (int)std::min<size_t>(kTileMaxNst, (max_optin_smem() - kTileHdrPlain) / ((size_t)sr * m * es));
            for (int nst : {2, 3, 4, maxn}) {
                if (nst < 2 || nst > maxn) continue;
                StepCand c;
                c.kind = StepCand::TILE; c.S = sr; c.nst = nst;
                bool dup = false;
                for (const StepCand& o : out) dup = dup || (o.kind == c.kind && o.S == c.S && o.nst == c.nst);
                if (!dup) out.push_back(c);
            }
        }
    }
    static const std::vector<int> Es_f32 = {8, 16, 24, 20, 28, 7, 9, 10, 12, 14, 15, 18, 21, 25, 30, 35, 42};
    static const std::vector<int> Es_f64 = {8, 16, 24, 20, 28, 7, 9, 10, 12, 14, 15, 18, 21, 25};
    static const std::vector<std::vector<int>> prefs = {
        {16, 8, 7, 5, 4, 3, 2}, {8, 16, 7, 5, 4, 3, 2}, {7, 5, 3, 16, 8, 4, 2}, {4, 8, 16, 7, 5, 3, 2}};
    for (int E : S.dbl ? Es_f64 : Es_f32) {
        if (m % E) continue;
        const int T = m / E;
        if (T > 256 || (S.cols && T > 64)) continue;
        std::vector<std::vector<int>> scheds;
        for (const auto& pf : prefs) {
            std::vector<int> r;
            if (!greedy_schedule(m, E, pf, r)) continue;
            bool dup = false;
            for (const auto& o : scheds) dup = dup || o == r;
            if (!dup) scheds.push_back(r);
        }
        for (const auto& r : scheds) {
            for (int per : {256 / T, 128 / T}) {
                if (per < 1) continue;
                StepCand c;
                c.kind = StepCand::REG; c.E = E; c.radix = r; c.per = per;
                out.push_back(c);
                if (c2c_rows && (m * es) % 16 == 0) { c.kind = StepCand::PIPE; out.push_back(c); }
                if (256 / T == 128 / T) break;
            }
        }
    }
    Schedule sc;
    if (make_schedule(m, sc) && !half_mode(S.mode)) out.push_back(StepCand());   // smem
    int a = 0, b = 0;
    if (!S.dbl && S.mode <= M_C2R_FULL && f2_kernel_f32(m, S.cols, S.mode, &a, &b)) {
        // CTAs of 64, 128 or 256 threads; rows: a quarter, half and all of the signals that
        // fill the threads in the phase of the smaller factor; columns: runs of 16, 32 or 64
        // adjacent columns
        for (int nt : {64, 128, 256}) {
            const int base = (nt + std::min(a, b) - 1) / std::min(a, b);
            const std::vector<int> pers = S.cols ? std::vector<int>{16, 32, 64}
                                                 : std::vector<int>{std::max(1, base / 4), std::max(1, base / 2), base};
            for (int per : pers) {
                if (f2_smem(a, b, S.cols, per, es, S.mode) > 100 * 1024) continue;
                StepCand c;
                c.kind = StepCand::F2; c.per = per; c.S = nt;
                bool dup = false;
                for (const StepCand& o : out) dup = dup || (o.kind == c.kind && o.per == c.per && o.S == c.S);
                if (!dup) out.push_back(c);
            }
        }
        // pipelined rows: 128 or 256 threads, tiles of 4, 8 or 16 rows, rings of 2 or 3 tiles
        if (c2c_rows && f2_pipe_kernel_f32(m, nullptr, nullptr)) {
            for (int nt : {128, 256})
                for (int per : {4, 8, 16})
                    for (int nst : {2, 3}) {
                        if (f2p_smem(a, b, per, nst, es) > 200 * 1024) continue;
                        StepCand c;
                        c.kind = StepCand::F2P; c.S = nt; c.per = per; c.nst = nst;
                        out.push_back(c);
                    }
        }
    }
    return out;
}

static std::string library_gpu_name() {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return "unknown";
    std::string s = prop.name;
    for (char& c : s) if (c == ' ' || c == '|' || c == '\t') c = '_';
    return s;
}

static std::string step_key(const FftStep& S) {
    std::ostringstream o;
    o << library_gpu_name() << "|v" << DTFFT_VERSION_CODE << "|" << S.dbl << "|" << S.mode << "|" << (S.cols ? 1 : 0)
      << "|" << S.n << "|" << S.m << "|" << S.nsig << "|" << S.idist << "|" << S.odist << "|" << S.plane << "|" << S.ld
      << "|" << S.ncols;
    return o.str();
}

struct TuneRecord {
    std::string step, best, second;
    float best_ms = 0, second_ms = 0;
    int candidates = 0;
};

static std::mutex g_step_tune_mu;
static std::map<std::string, std::string> g_step_tune;   // key -> candidate name
static bool g_step_tune_loaded = false;
static std::vector<TuneRecord> g_tune_records;

static void step_tune_load() {
    if (g_step_tune_loaded) return;
    g_step_tune_loaded = true;
    const char* path = getenv("DTFFT_GB_TUNE_CACHE");
    if (!path) return;
    FILE* f = fopen(path, "r");
    if (!f) return;
    char tag[16], key[512], val[256];
    while (fscanf(f, "%15s %511s %255s", tag, key, val) == 3) {
        if (strcmp(tag, "fft1") == 0) g_step_tune[key] = val;
        else { int ch; while ((ch = fgetc(f)) != '\n' && ch != EOF) {} }
    }
    fclose(f);
}

static void step_tune_store(const std::string& key, const std::string& val) {
    const char* path = getenv("DTFFT_GB_TUNE_CACHE");
    if (!path) return;
    if (FILE* f = fopen(path, "a")) {
        fprintf(f, "fft1 %s %s\n", key.c_str(), val.c_str());
        fclose(f);
    }
}

// Bytes a step touches from the start of its input and output buffers.
static size_t step_bytes(const FftStep& S) {
    const size_t es = S.dbl ? 16 : 8;
    i64 elems;
    if (S.cols) elems = (S.nsig / std::max(S.ncols, 1) + 1) * S.plane + S.ld;
    else elems = S.nsig * std::max<i64>(std::max(S.idist, S.odist), S.m) + 2 * (i64)S.m + 2;
    return (size_t)elems * es;
}

dtfft_error_t FftPlan::autotune(cudaStream_t s, int warmup, int iters, bool log) {
    std::lock_guard<std::mutex> lk(g_step_tune_mu);
    step_tune_load();
    for (std::vector<FftStep*>* dir : {&fwd_, &bwd_}) {
        for (FftStep* S : *dir) {
            if (S->tc || S->blue) continue;
            const std::string key = step_key(*S);
            StepCand chosen;
            auto it = g_step_tune.find(key);
            if (it != g_step_tune.end() && StepCand::parse(it->second, chosen)) {
                FftStep t = *S;
                t.tc = nullptr; t.blue = nullptr;
                if (apply_cand(t, chosen, tables_)) { *S = t; t.tc = nullptr; t.blue = nullptr; }
                continue;
            }
            const size_t bytes = step_bytes(*S);
            if (bytes > (size_t)4 << 30) continue;   // keep the default for very large steps
            void *a = nullptr, *b = nullptr;
            if (cudaMalloc(&a, bytes) != cudaSuccess || cudaMalloc(&b, bytes) != cudaSuccess) {
                cudaGetLastError();
                if (a) cudaFree(a);
                continue;
            }
            cudaMemsetAsync(a, 0, bytes, s);
            cudaMemsetAsync(b, 0, bytes, s);
            cudaEvent_t e0, e1;
            cudaEventCreate(&e0);
            cudaEventCreate(&e1);
            const std::vector<StepCand> cands = step_candidates(*S);
            const FftStep orig = *S;
            TuneRecord rec;
            rec.step = std::string(S->cols ? "cols" : "rows") + "_m" + std::to_string(S->m) + "_mode" +
                       std::to_string(S->mode) + (S->dbl ? "_f64" : "_f32") + "_n" + std::to_string(S->nsig);
            float best = 1e30f, second = 1e30f;
            StepCand best_c, second_c;
            bool any = false;
            for (const StepCand& c : cands) {
                FftStep t = orig;
                t.tc = nullptr; t.blue = nullptr;
                if (!apply_cand(t, c, tables_)) { t.tc = nullptr; t.blue = nullptr; continue; }
                bool ok = true;
                for (int i = 0; i < warmup && ok; ++i) ok = launch_step(t, a, b, s) == DTFFT_SUCCESS;
                cudaEventRecord(e0, s);
                for (int i = 0; i < iters && ok; ++i) ok = launch_step(t, a, b, s) == DTFFT_SUCCESS;
                cudaEventRecord(e1, s);
                const bool synced = cudaEventSynchronize(e1) == cudaSuccess;
                t.tc = nullptr; t.blue = nullptr;
                if (!ok || !synced) { cudaGetLastError(); continue; }
                float ms = 0;
                cudaEventElapsedTime(&ms, e0, e1);
                ms /= (float)std::max(iters, 1);
                ++rec.candidates;
                if (log) printf("dtFFT-gb300: fft step %s %s: %.4f ms\n", rec.step.c_str(), c.name().c_str(), ms);
                if (ms < best) { second = best; second_c = best_c; best = ms; best_c = c; any = true; }
                else if (ms < second) { second = ms; second_c = c; }
            }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            cudaStreamSynchronize(s);
            cudaFree(a);
            cudaFree(b);
            cudaGetLastError();
            if (!any) continue;
            FftStep t = orig;
            t.tc = nullptr; t.blue = nullptr;
            if (apply_cand(t, best_c, tables_)) { *S = t; }
            t.tc = nullptr; t.blue = nullptr;
            rec.best = best_c.name(); rec.best_ms = best;
            if (second < 1e29f) { rec.second = second_c.name(); rec.second_ms = second; }
            g_tune_records.push_back(rec);
            g_step_tune[key] = rec.best;
            step_tune_store(key, rec.best);
        }
    }
    return DTFFT_SUCCESS;
}

// ---------------------------------------------------------------------------
// FusedFT: batched C2C along the source's aligned axis + the box-list transpose
// ---------------------------------------------------------------------------
// Tensor-store write-out of a fused tile pass (fft_tile_xpose_tma_kernel):
// the pass's source groups and destination segments, its launch shape, and
// the tensor maps of the last few (input, output) buffer pairs (a map holds the
// buffer's address, so it is encoded on the host the first time a pair is
// seen; a pure host computation, also legal while a stream is being captured).
struct XTma {
    std::vector<FGroup> groups;
    std::vector<FSeg> segs;
    std::vector<int> seg_group;    // group of each segment
    int S = 0;                     // rows per tile: a point's line is S * sizeof(complex) bytes
    int lb = 0;                    // line bytes: 128 or 64 (the tensor maps' swizzle span)
    int ncw = 0;                   // compute warps
    const void* dgroups = nullptr; // device groups tiled by S (nullptr: the pass's own groups)
    i64 tiles = 0;                 // tiles of the pass at S rows
    int nst = 0;
    size_t smem = 0;
    int box_i = 256;               // points per tensor store: 256, 128, 64 or 32
    std::mutex mu;
    int m = 0;                     // points per row
    std::vector<std::pair<std::pair<const void*, const void*>, TmaXMaps*>> maps;   // per (input, output), most recent last
    ~XTma() { for (auto& e : maps) delete e.second; }
};

// Every store box of the pass fits the tensor-store kernel: segments start on
// an 8-point boundary (the 128-byte swizzle of the staged lines repeats every
// 8 lines, the 64-byte one every 8 lines of 64 bytes), no box reads past the
// tile's M lines, destination base and strides are 16-byte multiples, and the
// maps fit the kernel parameter.
static bool xtma_fits(int m, int es, const std::vector<FSeg>& segs, int box_i = 256) {
    if (segs.empty() || (int)segs.size() > kTmaXMaxSegs) return false;
    for (const FSeg& sg : segs) {
        const int len = sg.i1 - sg.i0;
        if (len < 1 || sg.i0 % 8) return false;
        const int box = std::min(len, box_i);
        for (int i = sg.i0; i < sg.i1; i += box_i)
            if (i + box > m) return false;
        if ((sg.dst_off * es) % 16 || (sg.di * es) % 16 || (sg.dw * es) % 16) return false;
        if (sg.di * es >= (1LL << 40) || sg.dw * es >= (1LL << 40) || sg.di < 1 || sg.dw < 0) return false;
    }
    return true;
}

// Tensor maps of every destination segment of the pass for output `out`:
// (u in 8-byte words, i, w) of the segment's block, boxes of one line (u, 128
// or 64 bytes) by up to 256 points, swizzled over the line's span.  With
// input `in` (non-null), also the load maps of the source groups whose rows
// are not adjacent: (row words in runs of 256, run, u, w), one box = a tile of
// S whole rows (one tensor load per tile instead of S row copies); `loads`
// stays 0 when a group does not fit (every tile then takes bulk copies).
static dtfft_error_t xtma_encode(const XTma& x, int es, const void* in, void* out, TmaXMaps* mp) {
    typedef CUresult (*EncodeFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    EncodeFn enc = (EncodeFn)tma_encode_tiled_fn();
    if (!enc) return DTFFT_ERROR_GPU_CALL_FAILED;
    memset(mp, 0, sizeof(TmaXMaps));
    const int w8 = es / 8;
    for (size_t k = 0; k < x.segs.size(); ++k) {
        const FSeg& sg = x.segs[k];
        const FGroup& g = x.groups[x.seg_group[k]];
        const int len = sg.i1 - sg.i0;
        cuuint64_t gdim[3] = {(cuuint64_t)g.nu * w8, (cuuint64_t)len, (cuuint64_t)std::max(g.nw, 1)};
        cuuint64_t gstr[2] = {(cuuint64_t)(sg.di * es), (cuuint64_t)(std::max<i64>(sg.dw, 1) * es)};
        if (g.nw <= 1) gstr[1] = gstr[0] * (cuuint64_t)len;   // a single w plane: any stride does
        cuuint32_t box[3] = {(cuuint32_t)(x.lb / 8), (cuuint32_t)std::min(len, x.box_i), 1};
        cuuint32_t estr[3] = {1, 1, 1};
        void* base = (char*)out + sg.dst_off * es;
        const CUresult r = enc(&mp->map[k], CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, base, gdim, gstr, box, estr,
                               CU_TENSOR_MAP_INTERLEAVE_NONE,
                               x.lb == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                               CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return DTFFT_ERROR_GPU_CALL_FAILED;
    }
    const char* le = getenv("DTFFT_GB_XTMA_TILE_LOADS");   // measurements: 0 = bulk copies only
    const i64 words = (i64)x.m * es / 8;
    bool strided = false;
    for (const FGroup& g : x.groups) strided = strided || g.su != x.m;
    if (in && strided && !(le && le[0] == '0') && (int)x.groups.size() <= kTmaXMaxGroups && words % 256 == 0 &&
        words / 256 <= 256) {
        bool ok = true;
        for (size_t gi = 0; gi < x.groups.size() && ok; ++gi) {
            const FGroup& g = x.groups[gi];
            if (g.su == x.m) continue;   // adjacent rows: one bulk copy per tile
            cuuint64_t gdim[4] = {256, (cuuint64_t)(words / 256), (cuuint64_t)g.nu, (cuuint64_t)std::max(g.nw, 1)};
            cuuint64_t gstr[3] = {256 * 8, (cuuint64_t)(g.su * es), (cuuint64_t)(std::max<i64>(g.sw, 1) * es)};
            if (g.nw <= 1) gstr[2] = gstr[1] * (cuuint64_t)g.nu;
            cuuint32_t box[4] = {256, (cuuint32_t)(words / 256), (cuuint32_t)x.S, 1};
            cuuint32_t estr[4] = {1, 1, 1, 1};
            const void* base = (const char*)in + g.src_off * es;
            ok = ((uintptr_t)base % 16) == 0 && gstr[1] % 16 == 0 && gstr[2] % 16 == 0 && gstr[1] < (1ULL << 40) &&
                 gstr[2] < (1ULL << 40) &&
                 enc(&mp->lmap[gi], CU_TENSOR_MAP_DATA_TYPE_UINT64, 4, const_cast<void*>(base), gdim, gstr, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
        }
        mp->loads = ok ? 1 : 0;
    }
    return DTFFT_SUCCESS;
}

dtfft_error_t FusedFT::create(const BoxList& bl, int m, int dbl, bool tile_only, FusedFT** out) {
    *out = nullptr;
    if (bl.copy || bl.host.empty()) return DTFFT_ERROR_INVALID_USAGE;
    if (bl.elem != (dbl ? 16 : 8)) return DTFFT_ERROR_INVALID_USAGE;
    const size_t es = dbl ? 16 : 8;
    // bulk copies need every source row 16-byte aligned
    bool aligned = (m * es) % 16 == 0;
    for (const Box& x : bl.host)
        aligned = aligned && ((x.src_off - x.a0) * (i64)es) % 16 == 0 && (x.sb * (i64)es) % 16 == 0 &&
                  (x.sc * (i64)es) % 16 == 0;
    // warp-per-row tile kernel when one is compiled for m, else the register kernels
    TileShape ts;
    i64 box_rows = 0;   // rows of the pass: every box holds nb x nc rows of one source rank
    {
        std::vector<std::pair<i64, i64>> seen;
        for (const Box& x : bl.host) {
            const std::pair<i64, i64> key(x.src_off - x.a0, (i64)x.nb * x.nc);
            if (std::find(seen.begin(), seen.end(), key) == seen.end()) { seen.push_back(key); box_rows += key.second; }
        }
    }
    const bool tile = aligned && tile_shape(m, dbl, true, ts, box_rows);
    // otherwise the two-factor kernel fused with the transpose (float) when one
    // is compiled for m, else the register kernels
    int f2a = 0, f2b = 0;
    void* f2fn = nullptr;
    {
        const char* e = getenv("DTFFT_GB_F2");
        if (!tile && !dbl && !(e && strcmp(e, "0") == 0)) f2fn = f2_xpose_kernel_f32(m, &f2a, &f2b);
    }
    if (tile_only && !tile && !f2fn) return DTFFT_ERROR_FFT_SIZE_NOT_SUPPORTED;
    int E = 0, T = 0;
    Schedule sch;
    int S = 1;
    if (tile) {
        S = ts.S;
    } else if (f2fn) {
        // rows per tile (runs of S adjacent destination points per output):
        // measured 3-8 % faster with 16 below 320 points, 8 above
        S = m < 320 ? 16 : 8;
        if (const char* e = getenv("DTFFT_GB_F2X_S")) S = std::min(32, std::max(1, atoi(e)));   // measurements
    } else {
        if (!make_reg_schedule(m, false, E, sch, T, 64) && !make_reg_schedule(m, false, E, sch, T, 256))
            return DTFFT_ERROR_FFT_SIZE_NOT_SUPPORTED;
        // rows per CTA: a power of two, at most 16 and (S*T) within the launch bound
        while (S * 2 <= 16 && S * 2 * T <= (dbl ? 256 : 512)) S *= 2;
    }
    std::vector<FGroup> groups;
    std::vector<FSeg> segs;
    i64 ctas = 0;
    size_t b = 0;
    const std::vector<Box>& bx = bl.host;
    while (b < bx.size()) {
        const Box& f = bx[b];
        FGroup g;
        g.src_off = f.src_off - f.a0;
        g.su = f.sb; g.sw = f.sc; g.nu = f.nb; g.nw = f.nc;
        g.seg_first = (int)segs.size();
        std::vector<FSeg> gs;
        size_t e = b;
        while (e < bx.size() && bx[e].src_off - bx[e].a0 == g.src_off && bx[e].nb == f.nb && bx[e].nc == f.nc &&
               bx[e].sb == f.sb && bx[e].sc == f.sc) {
            FSeg sgm;
            sgm.i0 = bx[e].a0; sgm.i1 = bx[e].a0 + bx[e].na;
            sgm.dst_off = bx[e].dst_off; sgm.di = bx[e].da_or_db; sgm.dw = bx[e].dc;
            gs.push_back(sgm);
            ++e;
        }
        std::sort(gs.begin(), gs.end(), [](const FSeg& x, const FSeg& y) { return x.i0 < y.i0; });
        int cov = 0;
        for (const FSeg& sgm : gs) { if (sgm.i0 != cov) return DTFFT_ERROR_INVALID_USAGE; cov = sgm.i1; }
        if (cov != m) return DTFFT_ERROR_INVALID_USAGE;   // rows must hold the whole transform axis
        for (const FSeg& sgm : gs)   // the write-out indexes a segment with 32-bit offsets
            if ((i64)(sgm.i1 - sgm.i0) * sgm.di + 16 >= 0x7fffffffLL) return DTFFT_ERROR_INVALID_USAGE;
        g.nseg = (int)gs.size();
        segs.insert(segs.end(), gs.begin(), gs.end());
        g.tiles_u = (g.nu + S - 1) / S;
        g.cta_begin = ctas;
        ctas += (i64)g.tiles_u * g.nw;
        groups.push_back(g);
        b = e;
    }
    if (ctas > 0x7fffffffLL) return DTFFT_ERROR_FFT_SIZE_NOT_SUPPORTED;
    FusedFT* p = new FusedFT();
    p->m_ = m; p->dbl_ = dbl; p->E_ = E; p->T_ = T; p->S_ = S; p->sched_ = sch;
    p->ngroups_ = (int)groups.size();
    p->ctas_ = ctas;
    dtfft_error_t err = DTFFT_SUCCESS;
    if (tile) {
        p->tile_ = true;
        if (const char* e = getenv("DTFFT_GB_TILE_WFAST")) p->wfast_ = atoi(e) == 1;   // measurements
        p->tile_nst_ = ts.nst;
        p->tile_threads_ = ts.threads;
        p->smem_ = ts.smem;
        // two rows per 16-byte store when every destination offset and stride is even
        int pair = dbl ? 0 : 1;
        for (const FSeg& sgm : segs) pair = pair && (sgm.dst_off % 2 == 0) && (sgm.di % 2 == 0) && (sgm.dw % 2 == 0);
        p->pair_ok_ = pair;
        // warp split override of the fused pass (experiments): DTFFT_GB_XPOSE_WARPS=<compute>,<store>
        if (const char* xw = getenv("DTFFT_GB_XPOSE_WARPS")) {
            int c = 0, w = 0;
            if (sscanf(xw, "%d,%d", &c, &w) == 2 && (dbl ? TilePtr<double>::get(m, -1, true, c, w)
                                                           : TilePtr<float>::get(m, -1, true, c, w))) {
                p->ncw_ = c; p->nsw_ = w;
                p->tile_threads_ = 32 * (c + w);
            }
        }
        err = upload_dir_table(m, -1, dbl, p->owned_, &p->tw_);
        if (err == DTFFT_SUCCESS) err = upload_dir_table(m, 1, dbl, p->owned_, &p->tw_bwd_);
        for (int sg = -1; sg <= 1 && err == DTFFT_SUCCESS; sg += 2) {
            const void* fn = dbl ? TilePtr<double>::get(m, sg, true, p->ncw_, p->nsw_)
                                 : TilePtr<float>::get(m, sg, true, p->ncw_, p->nsw_);
            err = set_smem_attrs(fn, ts.smem);
        }
        // the tensor-store write-out when a kernel is compiled for m, the
        // tiles come out as whole 128- or 64-byte lines and every segment fits
        // it (the default then); its tiles may hold fewer rows than the
        // store-warp kernel's, over their own copy of the groups
        int xs = 0, xw = 0;
        const void* fk = dbl ? TilePtr<double>::get_tma(m, -1, &xs, &xw) : TilePtr<float>::get_tma(m, -1, &xs, &xw);
        const void* bk = dbl ? TilePtr<double>::get_tma(m, 1) : TilePtr<float>::get_tma(m, 1);
        // (the widest store box that keeps every box inside the tile's M lines)
        int box = 256;
        while (box > 32 && !xtma_fits(m, (int)es, segs, box)) box >>= 1;
        if (err == DTFFT_SUCCESS && fk && bk && xs <= ts.S && (xs * (int)es == 128 || xs * (int)es == 64) &&
            tma_encode_tiled_fn() && xtma_fits(m, (int)es, segs, box)) {
            XTma* x = new XTma();
            x->box_i = box;
            x->m = m;
            x->S = xs;
            x->lb = xs * (int)es;
            x->ncw = xw;
            x->groups = groups;
            x->segs = segs;
            x->tiles = ctas;
            if (xs != ts.S) {
                x->tiles = 0;
                for (FGroup& g : x->groups) {
                    g.tiles_u = (g.nu + xs - 1) / xs;
                    g.cta_begin = x->tiles;
                    x->tiles += (i64)g.tiles_u * g.nw;
                }
            }
            for (size_t gi = 0; gi < groups.size(); ++gi)
                for (int k = 0; k < groups[gi].nseg; ++k) x->seg_group.push_back((int)gi);
            const size_t line_bytes = (size_t)m * x->lb;
            x->nst = (int)std::min<size_t>(kTileMaxNst, (max_optin_smem() - 2 * kTileHdrXTma) / line_bytes);
            x->smem = 2 * kTileHdrXTma + (size_t)x->nst * line_bytes;
            // the driver validates the maps' shapes and strides when they are
            // encoded: try once on an aligned stand-in address (host only)
            TmaXMaps probe;
            const bool encodable = xtma_encode(*x, (int)es, nullptr, (void*)(uintptr_t)4096, &probe) == DTFFT_SUCCESS;
            bool ok = encodable && x->nst >= 2 && x->tiles <= 0x7fffffffLL &&
                      set_smem_attrs(fk, x->smem) == DTFFT_SUCCESS && set_smem_attrs(bk, x->smem) == DTFFT_SUCCESS;
            if (ok && xs != ts.S) {
                void* dg = nullptr;
                ok = cudaMalloc(&dg, sizeof(FGroup) * x->groups.size()) == cudaSuccess &&
                     cudaMemcpy(dg, x->groups.data(), sizeof(FGroup) * x->groups.size(), cudaMemcpyHostToDevice) ==
                         cudaSuccess;
                if (dg) p->owned_.push_back(dg);
                x->dgroups = dg;
            }
            if (ok) {
                p->xtma_ = x;
                p->use_xtma_ = true;
            } else {
                delete x;
            }
            cudaGetLastError();
        }
    } else if (!f2fn) {
        const int pitch = m + m / 16;
        p->pitch_ = pitch;
        p->smem_ = std::max((size_t)S * pitch, (size_t)m * (S + 1)) * es;
        // TMA-pipelined variant: every row start must be 16-byte aligned
        if (aligned && !getenv("DTFFT_GB_NO_PIPE")) {
            p->pipe_smem_ = 128 + 2 * (size_t)S * m * es + p->smem_;
            p->pipe_per_sm_ = pipe_occupancy(dbl, m, E, true, S * T, p->pipe_smem_);
        }
        err = upload_table(table_exp(m, 1, m), dbl, p->owned_, &p->tw_);
    } else if (f2fn) {
        p->f2_ = f2fn;
        p->f2_threads_ = 128;
        if (const char* e = getenv("DTFFT_GB_F2X_THREADS")) {   // measurements
            const int t = atoi(e);
            if (t == 32 || t == 64 || t == 256) p->f2_threads_ = t;
        }
        p->smem_ = f2x_smem(f2a, f2b, S, es);
        err = set_smem_attrs(f2fn, p->smem_);
        if (err == DTFFT_SUCCESS) err = upload_table(table_exp(m, 1, m), dbl, p->owned_, &p->tw_);
    }
    if (err == DTFFT_SUCCESS) {
        void* dg = nullptr; void* ds = nullptr;
        if (cudaMalloc(&dg, sizeof(FGroup) * groups.size()) != cudaSuccess ||
            cudaMalloc(&ds, sizeof(FSeg) * segs.size()) != cudaSuccess) {
            err = DTFFT_ERROR_GPU_CALL_FAILED;
        } else {
            cudaMemcpy(dg, groups.data(), sizeof(FGroup) * groups.size(), cudaMemcpyHostToDevice);
            cudaMemcpy(ds, segs.data(), sizeof(FSeg) * segs.size(), cudaMemcpyHostToDevice);
        }
        if (dg) p->owned_.push_back(dg);
        if (ds) p->owned_.push_back(ds);
        p->groups_ = dg; p->segs_ = ds;
    }
    if (err == DTFFT_SUCCESS) {
        (void)sm_count();
        err = status_setup();
    }
    if (err == DTFFT_SUCCESS) {
        if (!tile && !f2fn)
            err = set_smem_attrs(dbl ? (const void*)KPtr<double>::xpose(E) : (const void*)KPtr<float>::xpose(E),
                                 p->smem_);
    }
    if (err != DTFFT_SUCCESS) { delete p; return err; }
    *out = p;
    return DTFFT_SUCCESS;
}

FusedFT::~FusedFT() {
    for (void* t : owned_) cudaFree(t);
    delete xtma_;
}

template <typename R>
static dtfft_error_t launch_fused_t(const FusedFT& F, int m, int E, int T, int S, int pitch, const Schedule& sch,
                                   const void* tw, const void* groups, const void* segs, int ngroups, i64 ctas,
                                   size_t smem, const void* in, void* out, int sign, cudaStream_t s) {
    typedef typename CT<R>::T C;
    FArgs<R> A;
    A.in = (const C*)in; A.out = (C*)out;
    A.groups = (const FGroup*)groups; A.segs = (const FSeg*)segs; A.ngroups = ngroups;
    A.m = m; A.sign = sign; A.S = S; A.pitch = pitch; A.tw = (const C*)tw;
    A.st.ns = (int)sch.radix.size();
    for (int i = 0; i < A.st.ns; ++i) A.st.radix[i] = sch.radix[i];
    void (*kfn)(FArgs<R>) = (void (*)(FArgs<R>))KPtr<R>::xpose(E);
    if (!kfn) return DTFFT_ERROR_FFT_SIZE_NOT_SUPPORTED;
    void* tok = prof_begin(s);
    kfn<<<(unsigned)ctas, S * T, smem, s>>>(A);
    if (tok) prof_end(tok, std::string("fftxpose_m") + std::to_string(m) + (sizeof(R) == 8 ? "_f64" : "_f32"), s);
    (void)F;
    count_launch();
    GB_CUDA_TRY(cudaGetLastError());
    return DTFFT_SUCCESS;
}

template <typename R>
static dtfft_error_t launch_fused_pipe(int m, int E, int T, int S, int pitch, const Schedule& sch, const void* tw,
                                      const void* groups, const void* segs, int ngroups, i64 tiles, size_t smem,
                                      int per_sm, const void* in, void* out, int sign, cudaStream_t s) {
    typedef typename CT<R>::T C;
    PArgs<R> P;
    P.in = (const C*)in; P.out = (C*)out;
    P.nsig = 0; P.groups = (const FGroup*)groups; P.segs = (const FSeg*)segs; P.ngroups = ngroups;
    P.ntiles = tiles; P.m = m; P.sign = sign; P.S = S; P.pitch = pitch; P.nst = 2; P.tw = (const C*)tw;
    P.st.ns = (int)sch.radix.size();
    for (int i = 0; i < P.st.ns; ++i) P.st.radix[i] = sch.radix[i];
    void* tok = prof_begin(s);
    GB_TRY((launch_pipe<R, true>(P, E, S * T, smem, per_sm, s)));
    if (tok) prof_end(tok, std::string("fftpipe_xpose_m") + std::to_string(m) + (sizeof(R) == 8 ? "_f64" : "_f32"), s);
    count_launch();
    GB_CUDA_TRY(cudaGetLastError());
    return DTFFT_SUCCESS;
}

template <typename R>
static dtfft_error_t launch_fused_tile_tma(int m, XTma& x, const void* tw, const void* groups, const void* segs,
                                          int ngroups, i64 tiles, const void* in, void* out, int sign, int wfast,
                                          cudaStream_t s) {
    typedef typename CT<R>::T C;
    TXArgs<R> X;
    TArgs<R>& P = X.a;
    X.box_i = x.box_i;
    P.in = (const C*)in; P.out = (C*)out; P.tw = (const C*)tw;
    P.nsig = 0; P.groups = (const FGroup*)groups; P.segs = (const FSeg*)segs; P.ngroups = ngroups;
    if (x.dgroups) { P.groups = (const FGroup*)x.dgroups; tiles = x.tiles; }
    P.ntiles = tiles; P.S = x.S; P.nst = x.nst; P.pair_ok = 0; P.wait_limit = g_wait_limit;
    P.status = status_ptr();
    P.wfast = wfast;
    {
        std::lock_guard<std::mutex> lk(x.mu);
        TmaXMaps* mp = nullptr;
        for (auto& e : x.maps)
            if (e.first.first == in && e.first.second == out) mp = e.second;
        if (!mp) {
            mp = new TmaXMaps();
            const dtfft_error_t r = xtma_encode(x, (int)sizeof(C), in, out, mp);
            if (r != DTFFT_SUCCESS) { delete mp; return r; }
            if (x.maps.size() >= 4) { delete x.maps.front().second; x.maps.erase(x.maps.begin()); }
            x.maps.emplace_back(std::make_pair(in, (const void*)out), mp);
        }
        memcpy(&X.m, mp, sizeof(TmaXMaps));
    }
    void (*kfn)(TXArgs<R>) = (void (*)(TXArgs<R>))TilePtr<R>::get_tma(m, sign);
    if (!kfn) return DTFFT_ERROR_FFT_SIZE_NOT_SUPPORTED;
    const i64 grid = std::min<i64>(tiles, (i64)sm_count());
    const int threads = 32 * (x.ncw + 1);
    void* tok = prof_begin(s);
    kfn<<<(unsigned)grid, threads, x.smem, s>>>(X);
    if (tok) prof_end(tok, std::string("ffttile_xtma_m") + std::to_string(m) + (sizeof(R) == 8 ? "_f64" : "_f32"), s);
    count_launch();
    GB_CUDA_TRY(cudaGetLastError());
    return DTFFT_SUCCESS;
}

template <typename R>
static dtfft_error_t launch_fused_tile(int m, int S, int nst, int threads, int ncw, int nsw, size_t smem, int pair_ok,
                                      const void* tw, const void* groups, const void* segs, int ngroups, i64 tiles,
                                      const void* in, void* out, int sign, int wfast, cudaStream_t s) {
    typedef typename CT<R>::T C;
    TArgs<R> P;
    P.in = (const C*)in; P.out = (C*)out; P.tw = (const C*)tw;
    P.nsig = 0; P.groups = (const FGroup*)groups; P.segs = (const FSeg*)segs; P.ngroups = ngroups;
    P.ntiles = tiles; P.S = S; P.nst = nst; P.pair_ok = pair_ok; P.wait_limit = g_wait_limit;
    P.status = status_ptr();
    P.wfast = wfast;
    void (*kfn)(TArgs<R>) = (void (*)(TArgs<R>))TilePtr<R>::get(m, sign, true, ncw, nsw);
    if (!kfn) return DTFFT_ERROR_FFT_SIZE_NOT_SUPPORTED;
    const i64 grid = std::min<i64>(tiles, (i64)sm_count());
    void* tok = prof_begin(s);
    kfn<<<(unsigned)grid, threads, smem, s>>>(P);
    if (tok) prof_end(tok, std::string("ffttile_xpose_m") + std::to_string(m) + (sizeof(R) == 8 ? "_f64" : "_f32"), s);
    count_launch();
    const cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) {
        cudaFuncAttributes fa;
        if (cudaFuncGetAttributes(&fa, (const void*)kfn) == cudaSuccess)
            fprintf(stderr, "dtFFT-gb300: fused pass m=%d: grid %lld x %d threads, %zu B dynamic smem; kernel: max %d "
                            "threads, %d registers, max dynamic smem %d B, static smem %zu B\n",
                    m, (long long)grid, threads, smem, fa.maxThreadsPerBlock, fa.numRegs,
                    fa.maxDynamicSharedSizeBytes, fa.sharedSizeBytes);
        GB_CUDA_TRY(le);
    }
    return DTFFT_SUCCESS;
}

// ---------------------------------------------------------------------------
// Measured warp split of the fused tile pass (part of the EXHAUSTIVE autotune
// that replaces src/dtfft_nvrtc_block_optimizer.F90's kernel choice)
// ---------------------------------------------------------------------------
static std::mutex g_ft_tune_mu;
static std::map<std::string, std::pair<int, int>> g_ft_tune;

dtfft_error_t FusedFT::autotune(i64 max_elems, cudaStream_t s, int warmup, int iters, bool log) {
    if (!tile_ || ctas_ == 0) return DTFFT_SUCCESS;
    int dev = 0;
    cudaGetDevice(&dev);
    std::ostringstream key;
    key << dev << "|" << m_ << "|" << dbl_ << "|" << S_ << "|" << ngroups_ << "|" << ctas_ << "|" << smem_;
    std::lock_guard<std::mutex> lk(g_ft_tune_mu);
    auto apply = [&](int c, int w) {
        if (c < 0) {   // the tensor-store write-out, stores of 256 >> (-1 - c) points
            if (!xtma_) return DTFFT_ERROR_FFT_SIZE_NOT_SUPPORTED;
            const int box = 256 >> (-1 - c);
            if (!xtma_fits(m_, dbl_ ? 16 : 8, xtma_->segs, box)) return DTFFT_ERROR_FFT_SIZE_NOT_SUPPORTED;
            std::lock_guard<std::mutex> lk2(xtma_->mu);
            if (xtma_->box_i != box) {   // the cached maps hold the old box
                for (auto& e : xtma_->maps) delete e.second;
                xtma_->maps.clear();
                xtma_->box_i = box;
            }
            use_xtma_ = true;
            return DTFFT_SUCCESS;
        }
        use_xtma_ = false;
        ncw_ = c; nsw_ = w;
        const void* f = dbl_ ? TilePtr<double>::get(m_, -1, true, c, w) : TilePtr<float>::get(m_, -1, true, c, w);
        int threads = 0;
        if (c == 0) threads = dbl_ ? TilePtr<double>::default_threads(m_, true) : TilePtr<float>::default_threads(m_, true);
        else threads = 32 * (c + w);
        tile_threads_ = threads;
        for (int sg = -1; sg <= 1; sg += 2) {
            const void* fn = dbl_ ? TilePtr<double>::get(m_, sg, true, c, w) : TilePtr<float>::get(m_, sg, true, c, w);
            GB_TRY(set_smem_attrs(fn, smem_));
        }
        return f ? DTFFT_SUCCESS : DTFFT_ERROR_FFT_SIZE_NOT_SUPPORTED;
    };
    auto it = g_ft_tune.find(key.str());
    if (it != g_ft_tune.end()) return apply(it->second.first, it->second.second);
    const size_t bytes = (size_t)max_elems * (dbl_ ? 16 : 8);
    void *a = nullptr, *b = nullptr;
    if (cudaMalloc(&a, bytes) != cudaSuccess || cudaMalloc(&b, bytes) != cudaSuccess) {
        cudaGetLastError();
        if (a) cudaFree(a);
        return DTFFT_SUCCESS;   // keep the default split when scratch is not available
    }
    cudaMemsetAsync(a, 0, bytes, s);
    static const int cands[][2] = {{-1, -1}, {-2, -1}, {-3, -1}, {-4, -1}, {0, 0}, {3, 5}, {4, 4},
                                   {2, 6}, {4, 8}, {6, 6}, {8, 4}};
    int best_c = 0, best_w = 0;
    float best_ms = 1e30f, second_ms = 1e30f;
    std::string best_name, second_name;
    int timed = 0;
    auto cand_name = [](int c, int w) {
        if (c < 0) return std::string("tensor_store:") + std::to_string(256 >> (-1 - c));
        if (c == 0) return std::string("store_warps:default");
        return std::string("store_warps:") + std::to_string(c) + "+" + std::to_string(w);
    };
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (const auto& c : cands) {
        const bool have = c[0] == 0 || (c[0] < 0 && xtma_) ||
                          (c[0] > 0 && (dbl_ ? TilePtr<double>::get(m_, -1, true, c[0], c[1])
                                             : TilePtr<float>::get(m_, -1, true, c[0], c[1])) != nullptr);
        if (!have || apply(c[0], c[1]) != DTFFT_SUCCESS) continue;
        bool ok = true;
        for (int i = 0; i < warmup && ok; ++i) ok = execute(a, b, -1, s) == DTFFT_SUCCESS;
        cudaEventRecord(e0, s);
        for (int i = 0; i < iters && ok; ++i) ok = execute(a, b, -1, s) == DTFFT_SUCCESS;
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        if (!ok) { cudaGetLastError(); continue; }
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        ms /= (float)std::max(iters, 1);
        if (log) {
            if (c[0] < 0)
                printf("dtFFT-gb300: fused pass m=%d tensor-store write-out, %d-point stores: %.4f ms\n", m_,
                       256 >> (-1 - c[0]), ms);
            else printf("dtFFT-gb300: fused pass m=%d warps %d+%d: %.4f ms\n", m_, c[0], c[1], ms);
        }
        ++timed;
        if (ms < best_ms) {
            second_ms = best_ms; second_name = best_name;
            best_ms = ms; best_c = c[0]; best_w = c[1]; best_name = cand_name(c[0], c[1]);
        } else if (ms < second_ms) {
            second_ms = ms; second_name = cand_name(c[0], c[1]);
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamSynchronize(s);
    cudaFree(a);
    cudaFree(b);
    cudaGetLastError();
    g_ft_tune[key.str()] = std::make_pair(best_c, best_w);
    if (timed > 0) {
        TuneRecord rec;
        rec.step = std::string("fused_xpose_m") + std::to_string(m_) + (dbl_ ? "_f64" : "_f32") + "_tiles" +
                   std::to_string(ctas_);
        rec.best = best_name; rec.best_ms = best_ms;
        if (second_ms < 1e29f) { rec.second = second_name; rec.second_ms = second_ms; }
        rec.candidates = timed;
        std::lock_guard<std::mutex> lk3(g_step_tune_mu);
        g_tune_records.push_back(rec);
    }
    return apply(best_c, best_w);
}

dtfft_error_t FusedFT::execute(const void* in, void* out, int sign, cudaStream_t s) {
    if (ctas_ == 0) return DTFFT_SUCCESS;
    if (f2_) {
        F2XArgs<float> A;
        A.in = (const float2*)in; A.out = (float2*)out; A.tw = (const float2*)tw_;
        A.groups = (const FGroup*)groups_; A.segs = (const FSeg*)segs_; A.ngroups = ngroups_;
        A.S = S_; A.sign = sign;
        void (*kfn)(F2XArgs<float>) = (void (*)(F2XArgs<float>))f2_;
        void* tok = prof_begin(s);
        kfn<<<(unsigned)ctas_, f2_threads_, smem_, s>>>(A);
        if (tok) prof_end(tok, std::string("fft2f_xpose_m") + std::to_string(m_) + "_f32", s);
        count_launch();
        GB_CUDA_TRY(cudaGetLastError());
        return DTFFT_SUCCESS;
    }
    if (tile_) {
        if (((uintptr_t)in % 16) != 0 || ((uintptr_t)out % 16) != 0) return DTFFT_ERROR_INVALID_USAGE;
        const void* tw = sign > 0 ? tw_bwd_ : tw_;
        if (use_xtma_ && xtma_) {
            if (dbl_)
                return launch_fused_tile_tma<double>(m_, *xtma_, tw, groups_, segs_, ngroups_, ctas_, in, out, sign,
                                                     wfast_, s);
            return launch_fused_tile_tma<float>(m_, *xtma_, tw, groups_, segs_, ngroups_, ctas_, in, out, sign, wfast_, s);
        }
        if (dbl_)
            return launch_fused_tile<double>(m_, S_, tile_nst_, tile_threads_, ncw_, nsw_, smem_, pair_ok_, tw, groups_,
                                             segs_, ngroups_, ctas_, in, out, sign, wfast_, s);
        return launch_fused_tile<float>(m_, S_, tile_nst_, tile_threads_, ncw_, nsw_, smem_, pair_ok_, tw, groups_,
                                        segs_, ngroups_, ctas_, in, out, sign, wfast_, s);
    }
    if (pipe_per_sm_ > 0 && ((uintptr_t)in % 16) == 0 && ((uintptr_t)out % 16) == 0) {
        if (dbl_)
            return launch_fused_pipe<double>(m_, E_, T_, S_, pitch_, sched_, tw_, groups_, segs_, ngroups_, ctas_,
                                             pipe_smem_, pipe_per_sm_, in, out, sign, s);
        return launch_fused_pipe<float>(m_, E_, T_, S_, pitch_, sched_, tw_, groups_, segs_, ngroups_, ctas_,
                                        pipe_smem_, pipe_per_sm_, in, out, sign, s);
    }
    if (dbl_)
        return launch_fused_t<double>(*this, m_, E_, T_, S_, pitch_, sched_, tw_, groups_, segs_, ngroups_, ctas_,
                                      smem_, in, out, sign, s);
    return launch_fused_t<float>(*this, m_, E_, T_, S_, pitch_, sched_, tw_, groups_, segs_, ngroups_, ctas_, smem_,
                                 in, out, sign, s);
}

}  // namespace gb

extern "C" int32_t dtfft_gb_device_status(int32_t reset) {
    if (gb::status_setup() != DTFFT_SUCCESS) return -1;
    if (cudaDeviceSynchronize() != cudaSuccess) { cudaGetLastError(); return -1; }
    volatile int* w = gb::g_status + gb::current_device();
    const int v = *w;
    if (reset) *w = 0;
    return v;
}

extern "C" int32_t dtfft_gb_tune_records(char* buf, size_t cap, size_t* len) {
    std::lock_guard<std::mutex> lk(gb::g_step_tune_mu);
    std::ostringstream o;
    o << "[";
    for (size_t i = 0; i < gb::g_tune_records.size(); ++i) {
        const gb::TuneRecord& r = gb::g_tune_records[i];
        o << (i ? "," : "") << "{\"step\":\"" << r.step << "\",\"chosen\":\"" << r.best << "\",\"chosen_ms\":" << r.best_ms
          << ",\"runner_up\":\"" << r.second << "\",\"runner_up_ms\":" << r.second_ms
          << ",\"candidates\":" << r.candidates << "}";
    }
    o << "]";
    const std::string t = o.str();
    if (len) *len = t.size() + 1;
    if (!buf) return DTFFT_SUCCESS;
    if (cap < t.size() + 1) return DTFFT_ERROR_INVALID_USAGE;
    memcpy(buf, t.c_str(), t.size() + 1);
    return DTFFT_SUCCESS;
}

extern "C" int32_t dtfft_gb_set_wait_limit(int32_t iterations) {
    if (iterations < 0) return DTFFT_ERROR_INVALID_USAGE;
    gb::g_wait_limit = iterations;
    return DTFFT_SUCCESS;
}

extern "C" int32_t dtfft_gb_set_fft_form(int32_t form) {
    if (form != 0 && form != 1) return DTFFT_ERROR_INVALID_USAGE;
    gb::g_fft_form = form;
    return DTFFT_SUCCESS;
}

extern "C" int32_t dtfft_gb_get_fft_form(void) { return gb::fft_form(); }
