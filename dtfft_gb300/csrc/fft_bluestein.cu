// Bluestein (chirp-z) form of a batched transform whose length has a prime
// factor above the largest direct butterfly (127): the reference's executors
// (cuFFT, VkFFT, FFTW) take every length, so the drop-in must as well.
//
// With jk = (j^2 + k^2 - (k-j)^2) / 2 the length-m DFT
//   X[k] = sum_j x[j] exp(s 2 pi i j k / m)
// becomes X[k] = w[k] * sum_j (x[j] w[j]) conj(w[k-j]),  w[j] = exp(s pi i j^2 / m),
// a convolution evaluated as a circular one of length L (a power of two,
// L >= 2m - 1) with two L-point FFTs of this library:
//   chirp-in:  a[j] = x[j] w[j] (j < m), 0 (m <= j < L)
//   A = FFT_L(a);  A *= FFT_L(c) / L  (c[d] = conj(w[d]) at d and L - d)
//   a = IFFT_L(A); chirp-out: X[k] = w[k] a[k]
// Rows go through in chunks so the L-point scratch stays bounded.  Real
// input (R2C of odd length) and Hermitian input (C2R of odd length) are
// expanded in chirp-in, and only the transform's own outputs are written in
// chirp-out.  An R2R kind (DCT/DST-I..IV) is a length-m complex FFT between
// a pre- and a post-processing step; chirp-in builds the core sequence from
// the signal's reals and chirp-out reads each output's core-spectrum point
// (r2r_pre / r2r_post in fft_kernels.cuh, shared with the shared-memory
// kernel).
#include <cmath>
#include <complex>
#include <vector>

#include "fft.cuh"
#include "fft_kernels.cuh"

namespace gb {

struct BlueGeom {
    i64 idist, odist;   // rows: signal s at s*idist (input) / s*odist (output)
    i64 plane;          // columns: signal s = column s % ncols of plane s / ncols
    int ld, ncols;
    int cols;
    int mode, n;        // R2R (kind 3): the core mode and the kind's length
    const void* ta;     // R2R pre/post tables
    const void* tb;
};

template <typename R>
__device__ __forceinline__ i64 blue_at(const BlueGeom& g, i64 s, int k, bool in) {
    if (g.cols) return (s / g.ncols) * g.plane + (s % g.ncols) + (i64)k * g.ld;
    return s * (in ? g.idist : g.odist) + k;
}

// kind: 0 C2C, 1 real input (R2C, odd n), 2 Hermitian half input (C2R, odd n),
// 3 R2R (the core sequence of mode g.mode)
template <typename R>
__global__ void blue_chirp_in(const void* in, typename CT<R>::T* a, const typename CT<R>::T* w, BlueGeom g,
                              i64 s0, int nrows, int m, int L, int kind) {
    typedef typename CT<R>::T C;
    const i64 total = (i64)nrows * L;
    for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (i64)gridDim.x * blockDim.x) {
        const int r = (int)(e / L), j = (int)(e - (i64)r * L);
        C v; v.x = 0; v.y = 0;
        if (j < m) {
            const i64 s = s0 + r;
            C x;
            if (kind == 3) {
                const R* inR = reinterpret_cast<const R*>(in);
                x = r2r_pre<R>(g.mode, g.n, m, j, [&](int i) { return inR[blue_at<R>(g, s, i, true)]; },
                               reinterpret_cast<const C*>(g.ta));
            } else if (kind == 1) {
                x.x = reinterpret_cast<const R*>(in)[blue_at<R>(g, s, j, true)];
                x.y = 0;
            } else if (kind == 2) {
                const C* inC = reinterpret_cast<const C*>(in);
                if (j <= m / 2) { x = inC[blue_at<R>(g, s, j, true)]; if (j == 0) x.y = 0; }
                else x = cconj(inC[blue_at<R>(g, s, m - j, true)]);
            } else {
                x = reinterpret_cast<const C*>(in)[blue_at<R>(g, s, j, true)];
            }
            v = cmul(x, w[j]);
        }
        a[e] = v;
    }
}

template <typename R>
__global__ void blue_mul(typename CT<R>::T* a, const typename CT<R>::T* cf, int nrows, int L) {
    const i64 total = (i64)nrows * L;
    for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (i64)gridDim.x * blockDim.x)
        a[e] = cmul(a[e], cf[e % L]);
}

template <typename R>
__global__ void blue_chirp_out(const typename CT<R>::T* a, void* out, const typename CT<R>::T* w, BlueGeom g,
                               i64 s0, int nrows, int m, int L, int kind) {
    typedef typename CT<R>::T C;
    const int nk = kind == 1 ? m / 2 + 1 : kind == 3 ? g.n : m;
    const i64 total = (i64)nrows * nk;
    for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (i64)gridDim.x * blockDim.x) {
        const int r = (int)(e / nk), k = (int)(e - (i64)r * nk);
        const i64 o = blue_at<R>(g, s0 + r, k, false);
        if (kind == 3) {
            const int p = r2r_post_src(g.mode, g.n, k);
            const C X = cmul(a[(i64)r * L + p], w[p]);
            reinterpret_cast<R*>(out)[o] =
                r2r_post<R>(g.mode, g.n, k, X, reinterpret_cast<const C*>(g.ta), reinterpret_cast<const C*>(g.tb));
            continue;
        }
        const C X = cmul(a[(i64)r * L + k], w[k]);
        if (kind == 2) reinterpret_cast<R*>(out)[o] = X.x;
        else reinterpret_cast<C*>(out)[o] = X;
    }
}

// host FFT in double (radix 2, in place) for the filter spectrum
static void host_fft(std::vector<std::complex<double>>& x, int sign) {
    const size_t n = x.size();
    for (size_t i = 1, j = 0; i < n; ++i) {
        size_t bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) std::swap(x[i], x[j]);
    }
    for (size_t len = 2; len <= n; len <<= 1) {
        const double ang = sign * 2.0 * M_PI / (double)len;
        for (size_t i = 0; i < n; i += len)
            for (size_t k = 0; k < len / 2; ++k) {
                const std::complex<double> wk(std::cos(ang * (double)k), std::sin(ang * (double)k));
                const std::complex<double> u = x[i + k], v = x[i + k + len / 2] * wk;
                x[i + k] = u + v;
                x[i + k + len / 2] = u - v;
            }
    }
}

struct Bluestein {
    int dbl = 0, m = 0, L = 0, kind = 0, chunk = 1;
    i64 nsig = 0;
    BlueGeom g{};
    FftPlan* fftL = nullptr;     // L-point C2C rows, `chunk` of them
    void* scratch = nullptr;     // chunk x L elements
    void* w = nullptr;           // w[j], j < m
    void* cf = nullptr;          // FFT_L(c) / L
    ~Bluestein() {
        delete fftL;
        if (scratch) cudaFree(scratch);
        if (w) cudaFree(w);
        if (cf) cudaFree(cf);
    }
};

template <typename T>
static dtfft_error_t upload_c(const std::vector<std::complex<double>>& v, void** out) {
    std::vector<T> h(2 * v.size());
    for (size_t i = 0; i < v.size(); ++i) { h[2 * i] = (T)v[i].real(); h[2 * i + 1] = (T)v[i].imag(); }
    GB_CUDA_TRY(cudaMalloc(out, h.size() * sizeof(T)));
    GB_CUDA_TRY(cudaMemcpy(*out, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
    return DTFFT_SUCCESS;
}

dtfft_error_t blue_create(int dbl, int m, int sign, int kind, i64 nsig, i64 idist, i64 odist, i64 plane, int ld,
                          int ncols, int cols, void** out, int r2r_mode, int r2r_n, const void* ta, const void* tb) {
    *out = nullptr;
    if (m < 2 || nsig < 0 || kind < 0 || kind > 3) return DTFFT_ERROR_FFT_SIZE_NOT_SUPPORTED;
    Bluestein* b = new Bluestein();
    b->dbl = dbl; b->m = m; b->kind = kind; b->nsig = nsig;
    b->g.idist = idist; b->g.odist = odist; b->g.plane = plane; b->g.ld = ld; b->g.ncols = ncols; b->g.cols = cols;
    b->g.mode = r2r_mode; b->g.n = r2r_n; b->g.ta = ta; b->g.tb = tb;
    int L = 1;
    while (L < 2 * m - 1) L <<= 1;
    b->L = L;
    const size_t es = dbl ? 16 : 8;
    const i64 budget = std::max<i64>(1, (i64)((64u << 20) / ((size_t)L * es)));   // 64 MiB of scratch
    b->chunk = (int)std::max<i64>(1, std::min<i64>(nsig, budget));
    std::vector<std::complex<double>> w(m), c(L, 0.0);
    for (int j = 0; j < m; ++j) {
        const long long q = ((long long)j * j) % (2LL * m);            // exact reduction of j^2 mod 2m
        const double ang = sign * M_PI * (double)q / (double)m;
        w[j] = std::complex<double>(std::cos(ang), std::sin(ang));
    }
    c[0] = std::conj(w[0]);
    for (int d = 1; d < m; ++d) c[d] = c[L - d] = std::conj(w[d]);
    host_fft(c, -1);
    for (auto& v : c) v /= (double)L;
    dtfft_error_t e = dbl ? upload_c<double>(w, &b->w) : upload_c<float>(w, &b->w);
    if (e == DTFFT_SUCCESS) e = dbl ? upload_c<double>(c, &b->cf) : upload_c<float>(c, &b->cf);
    if (e == DTFFT_SUCCESS && cudaMalloc(&b->scratch, (size_t)b->chunk * L * es) != cudaSuccess) {
        cudaGetLastError();
        e = DTFFT_ERROR_GPU_CALL_FAILED;
    }
    if (e == DTFFT_SUCCESS) {
        FftDesc d;
        d.type = FFT_C2C; d.dbl = dbl; d.rank = 1; d.n_fast = L; d.batch = b->chunk; d.idist = d.odist = L;
        e = FftPlan::create(d, &b->fftL);
    }
    if (e != DTFFT_SUCCESS) { delete b; return e; }
    *out = b;
    return DTFFT_SUCCESS;
}

void blue_destroy(void* p) { delete static_cast<Bluestein*>(p); }

template <typename R>
static dtfft_error_t blue_run(Bluestein& b, const void* in, void* out, cudaStream_t s) {
    typedef typename CT<R>::T C;
    C* a = (C*)b.scratch;
    for (i64 s0 = 0; s0 < b.nsig; s0 += b.chunk) {
        const int nr = (int)std::min<i64>(b.chunk, b.nsig - s0);
        const i64 tot = (i64)nr * b.L;
        const int grid = (int)std::min<i64>((tot + 255) / 256, 152 * 16);
        blue_chirp_in<R><<<grid, 256, 0, s>>>(in, a, (const C*)b.w, b.g, s0, nr, b.m, b.L, b.kind);
        count_launch();
        GB_CUDA_TRY(cudaGetLastError());
        // the L-point plan covers `chunk` rows; a shorter last chunk transforms
        // a few rows of stale scratch that nothing reads
        GB_TRY(b.fftL->execute(a, a, FFT_FWD, s));
        blue_mul<R><<<grid, 256, 0, s>>>(a, (const C*)b.cf, nr, b.L);
        count_launch();
        GB_CUDA_TRY(cudaGetLastError());
        GB_TRY(b.fftL->execute(a, a, FFT_BWD, s));
        blue_chirp_out<R><<<grid, 256, 0, s>>>(a, out, (const C*)b.w, b.g, s0, nr, b.m, b.L, b.kind);
        count_launch();
        GB_CUDA_TRY(cudaGetLastError());
    }
    return DTFFT_SUCCESS;
}

dtfft_error_t blue_execute(void* p, const void* in, void* out, cudaStream_t s) {
    Bluestein* b = static_cast<Bluestein*>(p);
    if (b->nsig == 0) return DTFFT_SUCCESS;
    void* tok = prof_begin(s);
    dtfft_error_t e = b->dbl ? blue_run<double>(*b, in, out, s) : blue_run<float>(*b, in, out, s);
    if (tok) prof_end(tok, std::string("bluestein_m") + std::to_string(b->m) + (b->dbl ? "_f64" : "_f32"), s);
    return e;
}

}  // namespace gb
