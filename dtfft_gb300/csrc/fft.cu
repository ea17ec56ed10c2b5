// Stockham FFT kernels for the GB300 execute path.
//
// One CTA loads whole signals (contiguous rows, or TC adjacent columns of a
// plane) into shared memory, runs every radix stage there and writes the
// result back: each transform costs one read and one write of its data in
// HBM.  Stages follow the Stockham autosort formulation (each stage reads
// x[j + r*m/R], applies twiddles W_{Ns*R}^{r*(j mod Ns)}, a radix-R DFT in
// registers, and writes y[(j - j mod Ns)*R + j mod Ns + r*Ns]), so no bit
// reversal pass is needed.  Radices 2, 3, 4, 5, 7, 8 have closed-form
// butterflies; any other prime factor up to 127 uses a direct O(R^2) butterfly.
//
// Real transforms reuse the complex core:
//   R2C / C2R, even n  : half-length complex FFT with the standard split /
//                        merge post-twiddle W_n^k
//   R2C / C2R, odd n   : full-length complex FFT of the real sequence
//   DCT-II / DCT-III   : Makhoul's n-point reordering
//   DCT-IV             : 2n-point FFT with pre-twiddle W_4n^j, post W_8n^(2k+1)
//   DCT-I / DST-I      : even / odd symmetric extension to 2(n-1) / 2(n+1)
//   DST-II/III/IV      : the matching DCT with (-1)^j signs and reversal
// Conventions are FFTW's (unnormalised, sign -1 forward), which the reference
// executors use (src/interfaces/fft/fftw/dtfft_executor_fftw_m.F90:91-226).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <sstream>

#include "fft.cuh"

namespace gb {

// ---------------------------------------------------------------------------
// Complex helpers
// ---------------------------------------------------------------------------
template <typename R> struct CT;
template <> struct CT<float> { typedef float2 T; };
template <> struct CT<double> { typedef double2 T; };

template <typename C> __device__ __forceinline__ C cadd(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
    C r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
template <typename C> __device__ __forceinline__ C cconj(C a) { a.y = -a.y; return a; }
// multiply by i*s (s = +1 or -1)
template <typename C> __device__ __forceinline__ C cmul_is(C a, int s) {
    C r; if (s > 0) { r.x = -a.y; r.y = a.x; } else { r.x = a.y; r.y = -a.x; } return r;
}
template <typename C, typename R> __device__ __forceinline__ C cscale(C a, R s) { a.x *= s; a.y *= s; return a; }

// ---------------------------------------------------------------------------
// Radix butterflies in registers: v[q] <- sum_r v[r] * exp(s*2*pi*i*r*q/R)
// ---------------------------------------------------------------------------
template <typename R, typename C>
__device__ __forceinline__ void dft2(C& a, C& b) { C t = a; a = cadd(t, b); b = csub(t, b); }

template <typename R, typename C>
__device__ __forceinline__ void dft3(C* v, int s) {
    const R h = (R)0.86602540378443864676;  // sin(2pi/3)
    C t1 = cadd(v[1], v[2]);
    C t2 = csub(v[0], cscale(t1, (R)0.5));
    C t3 = cmul_is(cscale(csub(v[1], v[2]), h), s);
    v[0] = cadd(v[0], t1);
    v[1] = cadd(t2, t3);
    v[2] = csub(t2, t3);
}

template <typename R, typename C>
__device__ __forceinline__ void dft4(C* v, int s) {
    C a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
    C c = cadd(v[1], v[3]), d = cmul_is(csub(v[1], v[3]), s);
    v[0] = cadd(a, c); v[2] = csub(a, c);
    v[1] = cadd(b, d); v[3] = csub(b, d);
}

template <typename R, typename C>
__device__ __forceinline__ void dft5(C* v, int s) {
    const R c1 = (R)0.30901699437494742410, c2 = (R)-0.80901699437494742410;   // cos(2pi/5), cos(4pi/5)
    const R s1 = (R)0.95105651629515357212, s2 = (R)0.58778525229247312917;    // sin(2pi/5), sin(4pi/5)
    C t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
    C t3 = csub(v[1], v[4]), t4 = csub(v[2], v[3]);
    C m1 = cadd(v[0], cadd(cscale(t1, c1), cscale(t2, c2)));
    C m2 = cadd(v[0], cadd(cscale(t1, c2), cscale(t2, c1)));
    C n1 = cmul_is(cadd(cscale(t3, s1), cscale(t4, s2)), s);
    C n2 = cmul_is(csub(cscale(t3, s2), cscale(t4, s1)), s);
    v[0] = cadd(v[0], cadd(t1, t2));
    v[1] = cadd(m1, n1); v[4] = csub(m1, n1);
    v[2] = cadd(m2, n2); v[3] = csub(m2, n2);
}

template <typename R, typename C>
__device__ __forceinline__ void dft7(C* v, int s) {
    const R cs[3] = {(R)0.62348980185873353053, (R)-0.22252093395631440429, (R)-0.90096886790241912624};
    const R sn[3] = {(R)0.78183148246802980871, (R)0.97492791218182360702, (R)0.43388373911755812048};
    C p[3], q[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) { p[j] = cadd(v[1 + j], v[6 - j]); q[j] = csub(v[1 + j], v[6 - j]); }
    C y0 = cadd(v[0], cadd(p[0], cadd(p[1], p[2])));
#pragma unroll
    for (int k = 1; k <= 3; ++k) {
        C mr = v[0], ni; ni.x = 0; ni.y = 0;
#pragma unroll
        for (int j = 1; j <= 3; ++j) {
            const int e = (j * k) % 7;           // cos/sin of 2*pi*e/7
            const int ee = e <= 3 ? e : 7 - e;
            const R sg = e <= 3 ? (R)1 : (R)-1;
            mr = cadd(mr, cscale(p[j - 1], cs[ee - 1]));
            ni = cadd(ni, cscale(q[j - 1], sg * sn[ee - 1]));
        }
        C t = cmul_is(ni, s);
        v[k] = cadd(mr, t);
        v[7 - k] = csub(mr, t);
    }
    v[0] = y0;
}

template <typename R, typename C>
__device__ __forceinline__ void dft8(C* v, int s) {
    C e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
    dft4<R>(e, s); dft4<R>(o, s);
    const R r2 = (R)0.70710678118654752440;
    // W8^1 = (1 + i s)/sqrt2, W8^2 = i s, W8^3 = (-1 + i s)/sqrt2
    C w1 = cscale(cadd(o[1], cmul_is(o[1], s)), r2);
    C w2 = cmul_is(o[2], s);
    C w3 = cscale(csub(cmul_is(o[3], s), o[3]), r2);
    v[0] = cadd(e[0], o[0]); v[4] = csub(e[0], o[0]);
    v[1] = cadd(e[1], w1);   v[5] = csub(e[1], w1);
    v[2] = cadd(e[2], w2);   v[6] = csub(e[2], w2);
    v[3] = cadd(e[3], w3);   v[7] = csub(e[3], w3);
}

// ---------------------------------------------------------------------------
// Kernel arguments
// ---------------------------------------------------------------------------
enum Mode {
    M_C2C = 0, M_R2C_HALF, M_R2C_FULL, M_C2R_HALF, M_C2R_FULL,
    M_DCT1, M_DCT2, M_DCT3, M_DCT4, M_DST1, M_DST2, M_DST3, M_DST4
};

struct Stages { int ns; int radix[26]; };

template <typename R>
struct Args {
    typedef typename CT<R>::T C;
    const char* in; char* out;
    i64 nsig;               // signals in total
    // rows: signal i starts at i*idist (input) / i*odist (output), unit element stride
    // cols: signal i = column (i % ncols) of plane (i / ncols); element k at k*ld
    i64 idist, odist;
    i64 plane;              // cols: plane stride (elements)
    int ld, ncols;          // cols
    int n;                  // logical length (reals for R2C/R2R, complex for C2C)
    int m;                  // complex core length
    int mode;
    int sign;               // core FFT sign
    int per_cta;            // signals per CTA
    int pitch;              // smem elements between signals (rows) / columns stride (cols)
    const C* tw;            // W_m^k, k < m (sign -1)
    const C* ta;            // mode table A
    const C* tb;            // mode table B
    Stages st;
};

// smem index of element k of local signal s
template <bool COLS>
__device__ __forceinline__ int sidx(int s, int k, int pitch, int per) { return COLS ? k * per + s : s * pitch + k; }

// ---------------------------------------------------------------------------
// Stockham stages on shared memory
// ---------------------------------------------------------------------------
template <typename R, bool COLS>
__device__ typename CT<R>::T* run_stages(typename CT<R>::T* a, typename CT<R>::T* b, int nloc,
                                          const Args<R>& A) {
    typedef typename CT<R>::T C;
    const int m = A.m, s = A.sign, per = A.per_cta, pitch = A.pitch;
    int Ns = 1;
    C* src = a; C* dst = b;
    for (int st = 0; st < A.st.ns; ++st) {
        const int Rr = A.st.radix[st];
        const int nb = m / Rr;
        const int total = nloc * nb;
        const int tstep = m / (Ns * Rr);
        for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
            int sg, j;
            if (COLS) { sg = idx % nloc; j = idx / nloc; } else { j = idx % nb; sg = idx / nb; }
            const int k = j % Ns;
            const int base = (j - k) * Rr + k;
            const int e1 = tstep * k;
#define GB_LOAD(RR)                                                                 \
    C v[RR];                                                                        \
    _Pragma("unroll") for (int r = 0; r < RR; ++r) {                                \
        v[r] = src[sidx<COLS>(sg, j + r * nb, pitch, per)];                         \
        if (r > 0 && k != 0) {                                                      \
            C w = A.tw[e1 * r];                                                     \
            if (s > 0) w.y = -w.y;                                                  \
            v[r] = cmul(v[r], w);                                                   \
        }                                                                           \
    }
#define GB_STORE(RR)                                                                \
    _Pragma("unroll") for (int r = 0; r < RR; ++r) dst[sidx<COLS>(sg, base + r * Ns, pitch, per)] = v[r];
            switch (Rr) {
            case 2: { GB_LOAD(2) dft2<R>(v[0], v[1]); GB_STORE(2) } break;
            case 3: { GB_LOAD(3) dft3<R>(v, s); GB_STORE(3) } break;
            case 4: { GB_LOAD(4) dft4<R>(v, s); GB_STORE(4) } break;
            case 5: { GB_LOAD(5) dft5<R>(v, s); GB_STORE(5) } break;
            case 7: { GB_LOAD(7) dft7<R>(v, s); GB_STORE(7) } break;
            case 8: { GB_LOAD(8) dft8<R>(v, s); GB_STORE(8) } break;
            default: {
                // direct butterfly for other primes: y_q = sum_r (v_r * tw) * W_R^(r q)
                for (int q = 0; q < Rr; ++q) {
                    C acc; acc.x = 0; acc.y = 0;
                    for (int r = 0; r < Rr; ++r) {
                        C x = src[sidx<COLS>(sg, j + r * nb, pitch, per)];
                        int e = e1 * r + ((r * q) % Rr) * nb;
                        if (e >= m) e -= m;
                        C w = A.tw[e];
                        if (s > 0) w.y = -w.y;
                        acc = cadd(acc, cmul(x, w));
                    }
                    dst[sidx<COLS>(sg, base + q * Ns, pitch, per)] = acc;
                }
            } break;
            }
#undef GB_LOAD
#undef GB_STORE
        }
        __syncthreads();
        C* t = src; src = dst; dst = t;
        Ns *= Rr;
    }
    return src;
}

// ---------------------------------------------------------------------------
// Load: global signal -> complex core sequence in smem (per mode)
// ---------------------------------------------------------------------------
template <typename R, bool COLS>
__device__ __forceinline__ i64 gin(const Args<R>& A, i64 sig, int k) {
    if (COLS) return (sig / A.ncols) * A.plane + (sig % A.ncols) + (i64)k * A.ld;
    return sig * A.idist + k;
}
template <typename R, bool COLS>
__device__ __forceinline__ i64 gout(const Args<R>& A, i64 sig, int k) {
    if (COLS) return (sig / A.ncols) * A.plane + (sig % A.ncols) + (i64)k * A.ld;
    return sig * A.odist + k;
}

template <typename R, bool COLS>
__global__ void __launch_bounds__(256) fft_kernel(Args<R> A) {
    typedef typename CT<R>::T C;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int per = A.per_cta;
    const int bufsz = COLS ? A.m * per : per * A.pitch;
    C* bufA = reinterpret_cast<C*>(smem_raw);
    C* bufB = bufA + bufsz;
    const i64 sig0 = (i64)blockIdx.x * per;
    const int nloc = (int)min((i64)per, A.nsig - sig0);
    if (nloc <= 0) return;
    const int n = A.n, m = A.m, pitch = A.pitch;
    const C* inC = reinterpret_cast<const C*>(A.in);
    const R* inR = reinterpret_cast<const R*>(A.in);
    C* outC = reinterpret_cast<C*>(A.out);
    R* outR = reinterpret_cast<R*>(A.out);

    // --- load / pre-process: thread idx -> (signal, k) with the contiguous
    //     global index fastest across the warp ---
    const int lenL = (A.mode == M_C2R_HALF || A.mode == M_C2R_FULL) ? (m) : m;
    const int totalL = nloc * lenL;
    for (int idx = threadIdx.x; idx < totalL; idx += blockDim.x) {
        int sl, k;
        if (COLS) { sl = idx % nloc; k = idx / nloc; } else { k = idx % lenL; sl = idx / lenL; }
        const i64 sg = sig0 + sl;
        C v; v.x = 0; v.y = 0;
        switch (A.mode) {
        case M_C2C: v = inC[gin<R, COLS>(A, sg, k)]; break;
        case M_R2C_HALF: { i64 g = gin<R, COLS>(A, sg, 2 * k); v.x = inR[g]; v.y = inR[g + 1]; } break;
        case M_R2C_FULL: v.x = inR[gin<R, COLS>(A, sg, k)]; break;
        case M_C2R_HALF: {
            // k < m = n/2: Z[k] = E[k] + i*O[k]
            C xk = inC[gin<R, COLS>(A, sg, k)];
            C xm = inC[gin<R, COLS>(A, sg, m - k)];
            if (k == 0) { xk.y = 0; xm.y = 0; }
            C cxm = cconj(xm);
            C e = cadd(xk, cxm);
            C o = cmul(csub(xk, cxm), cconj(A.ta[k]));
            v = cadd(e, cmul_is(o, 1));
        } break;
        case M_C2R_FULL: {
            if (k <= n / 2) { v = inC[gin<R, COLS>(A, sg, k)]; if (k == 0) v.y = 0; }
            else v = cconj(inC[gin<R, COLS>(A, sg, n - k)]);
        } break;
        case M_DCT1: {  // m = 2(n-1): even extension
            int j = k < n ? k : m - k;
            v.x = inR[gin<R, COLS>(A, sg, j)];
        } break;
        case M_DST1: {  // m = 2(n+1): [0, x, 0, -rev x]
            if (k >= 1 && k <= n) v.x = inR[gin<R, COLS>(A, sg, k - 1)];
            else if (k >= n + 2) v.x = -inR[gin<R, COLS>(A, sg, m - k - 1)];
        } break;
        case M_DCT2: case M_DST2: {  // m = n, Makhoul order: v[k] = x[2k] or x[2(n-1-k)+1]
            int j = (2 * k < n) ? 2 * k : 2 * (n - 1 - k) + 1;
            R x = inR[gin<R, COLS>(A, sg, j)];
            if (A.mode == M_DST2 && (j & 1)) x = -x;
            v.x = x;
        } break;
        case M_DCT3: case M_DST3: {  // m = n: V[k] = (X[k] - i X[n-k]) * conj(W_4n^k)
            R a, b = 0;
            if (A.mode == M_DCT3) {
                a = inR[gin<R, COLS>(A, sg, k)];
                if (k > 0) b = inR[gin<R, COLS>(A, sg, n - k)];
            } else {   // DST-III: X'[j] = x[n-1-j]
                a = inR[gin<R, COLS>(A, sg, n - 1 - k)];
                if (k > 0) b = inR[gin<R, COLS>(A, sg, k - 1)];
            }
            C t; t.x = a; t.y = -b;
            v = cmul(t, cconj(A.ta[k]));
        } break;
        case M_DCT4: case M_DST4: {  // m = 2n: x[j] * W_4n^j, zero padded
            if (k < n) {
                R x = inR[gin<R, COLS>(A, sg, A.mode == M_DCT4 ? k : n - 1 - k)];
                C t; t.x = x; t.y = 0;
                v = cmul(t, A.ta[k]);
            }
        } break;
        }
        bufA[sidx<COLS>(sl, k, pitch, per)] = v;
    }
    __syncthreads();

    C* res = run_stages<R, COLS>(bufA, bufB, nloc, A);

    // --- store / post-process ---
    int lenS;
    switch (A.mode) {
    case M_R2C_HALF: lenS = m + 1; break;
    case M_R2C_FULL: lenS = n / 2 + 1; break;
    case M_C2R_HALF: lenS = n; break;
    case M_C2C: lenS = m; break;
    default: lenS = n; break;
    }
    const int totalS = nloc * lenS;
    for (int idx = threadIdx.x; idx < totalS; idx += blockDim.x) {
        int sl, k;
        if (COLS) { sl = idx % nloc; k = idx / nloc; } else { k = idx % lenS; sl = idx / lenS; }
        const i64 sg = sig0 + sl;
        switch (A.mode) {
        case M_C2C: outC[gout<R, COLS>(A, sg, k)] = res[sidx<COLS>(sl, k, pitch, per)]; break;
        case M_R2C_HALF: {
            C zk = res[sidx<COLS>(sl, k == m ? 0 : k, pitch, per)];
            C zm = cconj(res[sidx<COLS>(sl, k == 0 ? 0 : m - k, pitch, per)]);
            C e = cscale(cadd(zk, zm), (R)0.5);
            C o = cscale(csub(zk, zm), (R)0.5);
            // X[k] = e + W_n^k * o / i
            C t = cmul(A.ta[k], o);
            outC[gout<R, COLS>(A, sg, k)] = cadd(e, cmul_is(t, -1));
        } break;
        case M_R2C_FULL: outC[gout<R, COLS>(A, sg, k)] = res[sidx<COLS>(sl, k, pitch, per)]; break;
        case M_C2R_HALF: {
            C z = res[sidx<COLS>(sl, k >> 1, pitch, per)];
            outR[gout<R, COLS>(A, sg, k)] = (k & 1) ? z.y : z.x;
        } break;
        case M_C2R_FULL: outR[gout<R, COLS>(A, sg, k)] = res[sidx<COLS>(sl, k, pitch, per)].x; break;
        case M_DCT1: outR[gout<R, COLS>(A, sg, k)] = res[sidx<COLS>(sl, k, pitch, per)].x; break;
        case M_DST1: outR[gout<R, COLS>(A, sg, k)] = -res[sidx<COLS>(sl, k + 1, pitch, per)].y; break;
        case M_DCT2: case M_DST2: {
            // y[k] = 2 Re(W_4n^k F[k]); DST-II writes it reversed
            C f = res[sidx<COLS>(sl, k, pitch, per)];
            C w = A.ta[k];
            R y = (R)2 * (w.x * f.x - w.y * f.y);
            outR[gout<R, COLS>(A, sg, A.mode == M_DCT2 ? k : n - 1 - k)] = y;
        } break;
        case M_DCT3: case M_DST3: {
            // y[2j] = Re v[j], y[2j+1] = Re v[n-1-j]  (index k of the output)
            int j = (k & 1) ? (n - 1 - (k >> 1)) : (k >> 1);
            R y = res[sidx<COLS>(sl, j, pitch, per)].x;
            if (A.mode == M_DST3 && (k & 1)) y = -y;
            outR[gout<R, COLS>(A, sg, k)] = y;
        } break;
        case M_DCT4: case M_DST4: {
            C f = res[sidx<COLS>(sl, k, pitch, per)];
            C w = A.tb[k];
            R y = (R)2 * (w.x * f.x - w.y * f.y);
            if (A.mode == M_DST4 && (k & 1)) y = -y;
            outR[gout<R, COLS>(A, sg, k)] = y;
        } break;
        }
    }
}

// ===========================================================================
// Register-resident Stockham kernel (fast path)
//
// A signal of m points is owned by T = m / E threads; thread t keeps the E
// points t + T*q (q < E) in registers.  With that ownership every radix-R
// stage is local: butterfly j = t + b*T (b < E/R) reads points j + r*m/R =
// t + T*(b + r*E/R), which the thread already holds.  Only the Stockham output
// permutation between stages goes through shared memory (one write, one read
// per point and stage boundary, padded i + i/16 against bank conflicts).  The
// last stage's outputs land on points t + T*q again, so the first stage loads
// and the last stage stores straight from / to HBM with the warp's lanes on
// consecutive addresses.  Real-transform pre/post work is folded into those
// global loads and stores; only R2C with even n exchanges once more.
// ===========================================================================

// W16^e = exp(s * 2*pi*i*e/16), e in [0, 9]
template <typename R, typename C>
__device__ __forceinline__ C w16(int e, int s) {
    const R cs[10] = {(R)1, (R)0.92387953251128675613, (R)0.70710678118654752440, (R)0.38268343236508977173, (R)0,
                      (R)-0.38268343236508977173, (R)-0.70710678118654752440, (R)-0.92387953251128675613, (R)-1,
                      (R)-0.92387953251128675613};
    const R sn[10] = {(R)0, (R)0.38268343236508977173, (R)0.70710678118654752440, (R)0.92387953251128675613, (R)1,
                      (R)0.92387953251128675613, (R)0.70710678118654752440, (R)0.38268343236508977173, (R)0,
                      (R)-0.38268343236508977173};
    C w; w.x = cs[e]; w.y = s > 0 ? sn[e] : -sn[e];
    return w;
}

template <typename R, typename C>
__device__ __forceinline__ void dft16(C* v, int s) {
    C a[4][4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
#pragma unroll
        for (int r = 0; r < 4; ++r) a[q][r] = v[q + 4 * r];
        dft4<R>(a[q], s);
#pragma unroll
        for (int k1 = 1; k1 < 4; ++k1)
            if (q) a[q][k1] = cmul(a[q][k1], w16<R, C>(q * k1, s));
    }
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
        C b[4] = {a[0][k1], a[1][k1], a[2][k1], a[3][k1]};
        dft4<R>(b, s);
#pragma unroll
        for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = b[k2];
    }
}

template <typename R, int RAD, typename C>
__device__ __forceinline__ void dft_any(C* w, int s) {
    if constexpr (RAD == 2) dft2<R>(w[0], w[1]);
    else if constexpr (RAD == 3) dft3<R>(w, s);
    else if constexpr (RAD == 4) dft4<R>(w, s);
    else if constexpr (RAD == 5) dft5<R>(w, s);
    else if constexpr (RAD == 7) dft7<R>(w, s);
    else if constexpr (RAD == 8) dft8<R>(w, s);
    else if constexpr (RAD == 16) dft16<R>(w, s);
}

__device__ __forceinline__ int rpad(int i) { return i + (i >> 4); }

// smem slot of point i of local signal sl
template <bool COLS>
__device__ __forceinline__ int rslot(int sl, int i, int spitch, int S) {
    return COLS ? i * S + sl : sl * spitch + rpad(i);
}

// One radix-RAD stage on the registers of thread t; with EX the outputs are
// written to their Stockham positions in smem (the exchange).
template <typename R, int E, int RAD, bool COLS, bool EX>
__device__ __forceinline__ void reg_stage(typename CT<R>::T (&v)[E], int t, int T, int Ns, int m,
                                          const typename CT<R>::T* __restrict__ tw, int s,
                                          typename CT<R>::T* sm, int sl, int spitch, int S) {
    typedef typename CT<R>::T C;
    constexpr int B = E / RAD;
    const int tstep = m / (Ns * RAD);
#pragma unroll
    for (int b = 0; b < B; ++b) {
        const int j = t + b * T;
        const int k = j % Ns;
        C w[RAD];
#pragma unroll
        for (int r = 0; r < RAD; ++r) w[r] = v[b + r * B];
        if (k != 0) {
            const int e1 = tstep * k;
#pragma unroll
            for (int r = 1; r < RAD; ++r) {
                C tv = __ldg(&tw[e1 * r]);
                if (s > 0) tv.y = -tv.y;
                w[r] = cmul(w[r], tv);
            }
        }
        dft_any<R, RAD>(w, s);
        if constexpr (EX) {
            const int base = (j - k) * RAD + k;
#pragma unroll
            for (int r = 0; r < RAD; ++r) sm[rslot<COLS>(sl, base + r * Ns, spitch, S)] = w[r];
        } else {
#pragma unroll
            for (int r = 0; r < RAD; ++r) v[b + r * B] = w[r];
        }
    }
}

template <typename R, int E, bool COLS, bool EX>
__device__ __forceinline__ bool reg_stage_any(int rad, typename CT<R>::T (&v)[E], int t, int T, int Ns, int m,
                                              const typename CT<R>::T* tw, int s, typename CT<R>::T* sm, int sl,
                                              int spitch, int S) {
    switch (rad) {
    case 2: if constexpr (E % 2 == 0) { reg_stage<R, E, 2, COLS, EX>(v, t, T, Ns, m, tw, s, sm, sl, spitch, S); return true; } break;
    case 3: if constexpr (E % 3 == 0) { reg_stage<R, E, 3, COLS, EX>(v, t, T, Ns, m, tw, s, sm, sl, spitch, S); return true; } break;
    case 4: if constexpr (E % 4 == 0) { reg_stage<R, E, 4, COLS, EX>(v, t, T, Ns, m, tw, s, sm, sl, spitch, S); return true; } break;
    case 5: if constexpr (E % 5 == 0) { reg_stage<R, E, 5, COLS, EX>(v, t, T, Ns, m, tw, s, sm, sl, spitch, S); return true; } break;
    case 7: if constexpr (E % 7 == 0) { reg_stage<R, E, 7, COLS, EX>(v, t, T, Ns, m, tw, s, sm, sl, spitch, S); return true; } break;
    case 8: if constexpr (E % 8 == 0) { reg_stage<R, E, 8, COLS, EX>(v, t, T, Ns, m, tw, s, sm, sl, spitch, S); return true; } break;
    case 16: if constexpr (E % 16 == 0) { reg_stage<R, E, 16, COLS, EX>(v, t, T, Ns, m, tw, s, sm, sl, spitch, S); return true; } break;
    }
    return false;
}

template <typename R, int E, bool COLS, bool C2C_ONLY>
__global__ void __launch_bounds__(256) fft_reg_kernel(Args<R> A) {
    typedef typename CT<R>::T C;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* sm = reinterpret_cast<C*>(smem_raw);
    const int S = A.per_cta;          // signals per CTA
    const int T = A.m / E;            // threads per signal
    int sl, t;
    if (COLS) { sl = threadIdx.x % S; t = threadIdx.x / S; }
    else { sl = threadIdx.x / T; t = threadIdx.x % T; }
    const i64 sig = (i64)blockIdx.x * S + sl;
    const bool live = sig < A.nsig;
    const int n = A.n, m = A.m, s = A.sign, spitch = A.pitch;
    const int mode = C2C_ONLY ? (int)M_C2C : A.mode;
    const C* inC = reinterpret_cast<const C*>(A.in);
    const R* inR = reinterpret_cast<const R*>(A.in);
    C* outC = reinterpret_cast<C*>(A.out);
    R* outR = reinterpret_cast<R*>(A.out);

    // ---- load core input points i = t + T*q ----
    C v[E];
#pragma unroll
    for (int q = 0; q < E; ++q) {
        const int i = t + T * q;
        C x; x.x = 0; x.y = 0;
        if (live) {
            switch (mode) {
            case M_C2C: x = inC[gin<R, COLS>(A, sig, i)]; break;
            case M_R2C_HALF: x = *reinterpret_cast<const C*>(inR + gin<R, COLS>(A, sig, 2 * i)); break;
            case M_R2C_FULL: x.x = inR[gin<R, COLS>(A, sig, i)]; break;
            case M_C2R_HALF: {
                C xk = inC[gin<R, COLS>(A, sig, i)];
                C xm = inC[gin<R, COLS>(A, sig, m - i)];
                if (i == 0) { xk.y = 0; xm.y = 0; }
                C cxm = cconj(xm);
                C o = cmul(csub(xk, cxm), cconj(__ldg(&A.ta[i])));
                x = cadd(cadd(xk, cxm), cmul_is(o, 1));
            } break;
            case M_C2R_FULL:
                if (i <= n / 2) { x = inC[gin<R, COLS>(A, sig, i)]; if (i == 0) x.y = 0; }
                else x = cconj(inC[gin<R, COLS>(A, sig, n - i)]);
                break;
            case M_DCT1: x.x = inR[gin<R, COLS>(A, sig, i < n ? i : m - i)]; break;
            case M_DST1:
                if (i >= 1 && i <= n) x.x = inR[gin<R, COLS>(A, sig, i - 1)];
                else if (i >= n + 2) x.x = -inR[gin<R, COLS>(A, sig, m - i - 1)];
                break;
            case M_DCT2: case M_DST2: {
                const int j = (2 * i < n) ? 2 * i : 2 * (n - 1 - i) + 1;
                R y = inR[gin<R, COLS>(A, sig, j)];
                if (mode == M_DST2 && (j & 1)) y = -y;
                x.x = y;
            } break;
            case M_DCT3: case M_DST3: {
                R a, b = 0;
                if (mode == M_DCT3) { a = inR[gin<R, COLS>(A, sig, i)]; if (i > 0) b = inR[gin<R, COLS>(A, sig, n - i)]; }
                else { a = inR[gin<R, COLS>(A, sig, n - 1 - i)]; if (i > 0) b = inR[gin<R, COLS>(A, sig, i - 1)]; }
                C tt; tt.x = a; tt.y = -b;
                x = cmul(tt, cconj(__ldg(&A.ta[i])));
            } break;
            case M_DCT4: case M_DST4:
                if (i < n) {
                    C tt; tt.x = inR[gin<R, COLS>(A, sig, mode == M_DCT4 ? i : n - 1 - i)]; tt.y = 0;
                    x = cmul(tt, __ldg(&A.ta[i]));
                }
                break;
            }
        }
        v[q] = x;
    }
    // every point of the CTA is read before any is written (in-place safety)
    __syncthreads();

    // ---- stages ----
    int Ns = 1;
    const int ns = A.st.ns;
    for (int st = 0; st < ns - 1; ++st) {
        const int rad = A.st.radix[st];
        reg_stage_any<R, E, COLS, true>(rad, v, t, T, Ns, m, A.tw, s, sm, sl, spitch, S);
        __syncthreads();
#pragma unroll
        for (int q = 0; q < E; ++q) v[q] = sm[rslot<COLS>(sl, t + T * q, spitch, S)];
        __syncthreads();
        Ns *= rad;
    }
    if (ns > 0) reg_stage_any<R, E, COLS, false>(A.st.radix[ns - 1], v, t, T, Ns, m, A.tw, s, sm, sl, spitch, S);

    // ---- store core output points i = t + T*q ----
    if (mode == M_R2C_HALF) {
        // X[k] needs Z[k] and Z[m-k]: one more exchange
#pragma unroll
        for (int q = 0; q < E; ++q) sm[rslot<COLS>(sl, t + T * q, spitch, S)] = v[q];
        __syncthreads();
        if (live) {
            for (int k = t; k <= m; k += T) {
                C zk = sm[rslot<COLS>(sl, k == m ? 0 : k, spitch, S)];
                C zm = cconj(sm[rslot<COLS>(sl, k == 0 ? 0 : m - k, spitch, S)]);
                C e = cscale(cadd(zk, zm), (R)0.5);
                C o = cscale(csub(zk, zm), (R)0.5);
                C tt = cmul(__ldg(&A.ta[k]), o);
                outC[gout<R, COLS>(A, sig, k)] = cadd(e, cmul_is(tt, -1));
            }
        }
        return;
    }
    if (!live) return;
#pragma unroll
    for (int q = 0; q < E; ++q) {
        const int i = t + T * q;
        const C f = v[q];
        switch (mode) {
        case M_C2C: outC[gout<R, COLS>(A, sig, i)] = f; break;
        case M_R2C_FULL: if (i <= n / 2) outC[gout<R, COLS>(A, sig, i)] = f; break;
        case M_C2R_HALF: *reinterpret_cast<C*>(outR + gout<R, COLS>(A, sig, 2 * i)) = f; break;
        case M_C2R_FULL: outR[gout<R, COLS>(A, sig, i)] = f.x; break;
        case M_DCT1: if (i < n) outR[gout<R, COLS>(A, sig, i)] = f.x; break;
        case M_DST1: if (i >= 1 && i <= n) outR[gout<R, COLS>(A, sig, i - 1)] = -f.y; break;
        case M_DCT2: case M_DST2: {
            C w = __ldg(&A.ta[i]);
            R y = (R)2 * (w.x * f.x - w.y * f.y);
            outR[gout<R, COLS>(A, sig, mode == M_DCT2 ? i : n - 1 - i)] = y;
        } break;
        case M_DCT3: case M_DST3: {
            if (2 * i < n) outR[gout<R, COLS>(A, sig, 2 * i)] = f.x;
            const int k2 = 2 * (n - 1 - i) + 1;
            if (k2 < n) outR[gout<R, COLS>(A, sig, k2)] = mode == M_DST3 ? -f.x : f.x;
        } break;
        case M_DCT4: case M_DST4: {
            if (i >= n) break;
            C w = __ldg(&A.tb[i]);
            R y = (R)2 * (w.x * f.x - w.y * f.y);
            if (mode == M_DST4 && (i & 1)) y = -y;
            outR[gout<R, COLS>(A, sig, i)] = y;
        } break;
        }
    }
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
    bool reads_out = false;  // step reads the plan's output buffer (second pass)
};

// Register-kernel schedule: points per thread E (compiled: 8, 16, 24, 20, 28),
// radices dividing E, fewest stages first, then fewest registers.
static bool make_reg_schedule(int m, bool cols, int& E_out, Schedule& sch, int& T_out) {
    static const int Es[] = {8, 16, 24, 20, 28};
    static const int rads[] = {16, 8, 7, 5, 4, 3, 2};
    int best_stages = 1 << 30, best_E = 0;
    Schedule best;
    for (int E : Es) {
        if (m % E != 0) continue;
        const int T = m / E;
        if (T < 1 || T > 256) continue;
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

// Fill geometry, tables and launch shape of one step.
static dtfft_error_t prepare_step(FftStep& S, std::vector<void*>& owned) {
    int m, sign;
    if (!mode_geometry(S.mode, S.n, S.sign, m, sign)) return DTFFT_ERROR_FFT_SIZE_NOT_SUPPORTED;
    S.m = m;
    S.sign = sign;
    const size_t es = S.dbl ? 16 : 8;
    int E = 0, T = 0;
    if (!getenv("DTFFT_GB_NO_REG_FFT") && make_reg_schedule(m, S.cols, E, S.sched, T)) {
        S.E = E;
        // S signals per CTA, blockDim = S*T (signals past the end are masked)
        S.per = std::max(1, 256 / T);
        S.threads = S.per * T;
        S.pitch = m + m / 16;
        S.smem = S.cols ? (size_t)m * S.per * es : (size_t)S.per * S.pitch * es;
    } else if (!make_schedule(m, S.sched)) {
        return DTFFT_ERROR_FFT_SIZE_NOT_SUPPORTED;
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
    switch (S.mode) {
    case M_R2C_HALF: GB_TRY(upload_table(table_exp(m + 1, 1, S.n), S.dbl, owned, &S.ta)); break;
    case M_C2R_HALF: GB_TRY(upload_table(table_exp(m, 1, S.n), S.dbl, owned, &S.ta)); break;
    case M_DCT2: case M_DST2: case M_DCT3: case M_DST3:
        GB_TRY(upload_table(table_exp(S.n, 1, 4LL * S.n), S.dbl, owned, &S.ta)); break;
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

template <typename R, bool COLS>
static dtfft_error_t launch_step_t(const FftStep& S, const void* in, void* out, cudaStream_t s) {
    Args<R> A;
    typedef typename CT<R>::T C;
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
        void (*kfn)(Args<R>) = nullptr;
        const bool c2c = S.mode == M_C2C;
        switch (S.E) {
        case 8: kfn = c2c ? fft_reg_kernel<R, 8, COLS, true> : fft_reg_kernel<R, 8, COLS, false>; break;
        case 16: kfn = c2c ? fft_reg_kernel<R, 16, COLS, true> : fft_reg_kernel<R, 16, COLS, false>; break;
        case 24: kfn = c2c ? fft_reg_kernel<R, 24, COLS, true> : fft_reg_kernel<R, 24, COLS, false>; break;
        case 20: kfn = c2c ? fft_reg_kernel<R, 20, COLS, true> : fft_reg_kernel<R, 20, COLS, false>; break;
        case 28: kfn = c2c ? fft_reg_kernel<R, 28, COLS, true> : fft_reg_kernel<R, 28, COLS, false>; break;
        default: return DTFFT_ERROR_FFT_SIZE_NOT_SUPPORTED;
        }
        if (S.smem > 48 * 1024)
            GB_CUDA_TRY(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S.smem));
        kfn<<<(unsigned)ctas, S.threads, S.smem, s>>>(A);
    } else {
        if (S.smem > 48 * 1024)
            GB_CUDA_TRY(cudaFuncSetAttribute(fft_kernel<R, COLS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S.smem));
        fft_kernel<R, COLS><<<(unsigned)ctas, 256, S.smem, s>>>(A);
    }
    if (tok) {
        static const char* mn[] = {"c2c", "r2c", "r2c", "c2r", "c2r", "dct1", "dct2", "dct3", "dct4",
                                   "dst1", "dst2", "dst3", "dst4"};
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

}  // namespace gb
