// Device code of the FFT kernels (templates only; instantiated per precision in
// fft_inst_*.cu so the build compiles them in parallel).
#pragma once

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

#include <cstdint>

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
    M_DCT1, M_DCT2, M_DCT3, M_DCT4, M_DST1, M_DST2, M_DST3, M_DST4,
    // even n, register kernel only: DCT/DST-II and -III through an n/2-point
    // complex FFT (the real Makhoul sequence packed two points per complex)
    M_DCT2H, M_DST2H, M_DCT3H, M_DST3H
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

// ---------------------------------------------------------------------------
// R2R kinds as a length-m complex FFT (modes M_DCT1 .. M_DST4): point k of the
// core sequence from the signal's n reals, and output k of the kind from one
// point of the core spectrum.  Shared by the shared-memory kernel and the
// Bluestein form (fft_bluestein.cu).
// ---------------------------------------------------------------------------
// x(j): real j of the signal; ta: W_4n^k (DCT/DST-II/-III/-IV)
template <typename R, typename X>
__device__ __forceinline__ typename CT<R>::T r2r_pre(int mode, int n, int m, int k, X x,
                                                     const typename CT<R>::T* ta) {
    typedef typename CT<R>::T C;
    C v; v.x = 0; v.y = 0;
    switch (mode) {
    case M_DCT1:    // m = 2(n-1): even extension
        v.x = x(k < n ? k : m - k);
        break;
    case M_DST1:    // m = 2(n+1): [0, x, 0, -rev x]
        if (k >= 1 && k <= n) v.x = x(k - 1);
        else if (k >= n + 2) v.x = -x(m - k - 1);
        break;
    case M_DCT2: case M_DST2: {   // m = n, Makhoul order: v[k] = x[2k] or x[2(n-1-k)+1]
        const int j = (2 * k < n) ? 2 * k : 2 * (n - 1 - k) + 1;
        R t = x(j);
        if (mode == M_DST2 && (j & 1)) t = -t;
        v.x = t;
    } break;
    case M_DCT3: case M_DST3: {   // m = n: V[k] = (X[k] - i X[n-k]) * conj(W_4n^k)
        R a, b = 0;
        if (mode == M_DCT3) {
            a = x(k);
            if (k > 0) b = x(n - k);
        } else {                  // DST-III: X'[j] = x[n-1-j]
            a = x(n - 1 - k);
            if (k > 0) b = x(k - 1);
        }
        C t; t.x = a; t.y = -b;
        v = cmul(t, cconj(ta[k]));
    } break;
    case M_DCT4: case M_DST4:     // m = 2n: x[j] * W_4n^j, zero padded
        if (k < n) {
            C t; t.x = x(mode == M_DCT4 ? k : n - 1 - k); t.y = 0;
            v = cmul(t, ta[k]);
        }
        break;
    }
    return v;
}

// The core-spectrum point output k of the kind is made from.
__device__ __forceinline__ int r2r_post_src(int mode, int n, int k) {
    switch (mode) {
    case M_DST1: return k + 1;
    case M_DST2: return n - 1 - k;                                   // DST-II is DCT-II's order reversed
    case M_DCT3: case M_DST3: return (k & 1) ? (n - 1 - (k >> 1)) : (k >> 1);
    default: return k;
    }
}

// Output k of the kind from f = core spectrum point r2r_post_src(mode, n, k);
// tb: W_8n^(2k+1) (DCT/DST-IV).
template <typename R>
__device__ __forceinline__ R r2r_post(int mode, int n, int k, typename CT<R>::T f, const typename CT<R>::T* ta,
                                      const typename CT<R>::T* tb) {
    switch (mode) {
    case M_DCT1: return f.x;
    case M_DST1: return -f.y;
    case M_DCT2: case M_DST2: {   // y = 2 Re(W_4n^p F[p])
        const int p = mode == M_DCT2 ? k : n - 1 - k;
        const typename CT<R>::T w = ta[p];
        return (R)2 * (w.x * f.x - w.y * f.y);
    }
    case M_DCT3: return f.x;
    case M_DST3: return (k & 1) ? -f.x : f.x;
    case M_DCT4: case M_DST4: {
        const typename CT<R>::T w = tb[k];
        const R y = (R)2 * (w.x * f.x - w.y * f.y);
        return (mode == M_DST4 && (k & 1)) ? -y : y;
    }
    }
    return 0;
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
        default:
            v = r2r_pre<R>(A.mode, n, m, k, [&](int j) { return inR[gin<R, COLS>(A, sg, j)]; }, A.ta);
            break;
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
        default:
            outR[gout<R, COLS>(A, sg, k)] =
                r2r_post<R>(A.mode, n, k, res[sidx<COLS>(sl, r2r_post_src(A.mode, n, k), pitch, per)], A.ta, A.tb);
            break;
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

// Makhoul's order of an n-point DCT-II input: v[p] = x[mk_perm(p)]
__device__ __forceinline__ int mk_perm(int p, int n) { return (2 * p < n) ? 2 * p : 2 * (n - 1 - p) + 1; }

// V[k] = (y[k] - i y[n-k]) conj(W_4n^k) of a DCT-III input (DST-III: y read
// reversed, y[n-1-k] and y[k-1]); V[0] and V[n/2] are real
template <typename R, bool COLS>
__device__ __forceinline__ typename CT<R>::T dct3_v(const Args<R>& A, const R* inR, i64 sig, int k, int n, bool dst) {
    typedef typename CT<R>::T C;
    R a, b = 0;
    if (!dst) { a = inR[gin<R, COLS>(A, sig, k)]; if (k > 0) b = inR[gin<R, COLS>(A, sig, n - k)]; }
    else { a = inR[gin<R, COLS>(A, sig, n - 1 - k)]; if (k > 0) b = inR[gin<R, COLS>(A, sig, k - 1)]; }
    C tt; tt.x = a; tt.y = -b;
    return cmul(tt, cconj(__ldg(&A.tb[k])));
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
            case M_DCT2H: case M_DST2H: {   // z[i] = (v[2i], v[2i+1]), DST: odd-indexed x negated
                const int j0 = mk_perm(2 * i, n), j1 = mk_perm(2 * i + 1, n);
                R a0 = inR[gin<R, COLS>(A, sig, j0)], a1 = inR[gin<R, COLS>(A, sig, j1)];
                if (mode == M_DST2H) { if (j0 & 1) a0 = -a0; if (j1 & 1) a1 = -a1; }
                x.x = a0; x.y = a1;
            } break;
            case M_DCT3H: case M_DST3H: {   // half spectrum of the real Makhoul sequence, as C2R
                C vk = dct3_v<R, COLS>(A, inR, sig, i, n, mode == M_DST3H);
                C vm = dct3_v<R, COLS>(A, inR, sig, m - i, n, mode == M_DST3H);
                if (i == 0) { vk.y = 0; vm.y = 0; }
                C cvm = cconj(vm);
                C o = cmul(csub(vk, cvm), cconj(__ldg(&A.ta[i])));
                x = cadd(cadd(vk, cvm), cmul_is(o, 1));
            } break;
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
    if (mode == M_DCT2H || mode == M_DST2H) {
        // V[k] (k <= m) of the real Makhoul sequence from Z[k], Z[m-k]; then
        // y[k] = 2 Re(W_4n^k V[k]) and y[n-k] = 2 Re(W_4n^(n-k) conj(V[k]))
#pragma unroll
        for (int q = 0; q < E; ++q) sm[rslot<COLS>(sl, t + T * q, spitch, S)] = v[q];
        __syncthreads();
        if (live) {
            const bool dst = mode == M_DST2H;
            for (int k = t; k <= m; k += T) {
                C zk = sm[rslot<COLS>(sl, k == m ? 0 : k, spitch, S)];
                C zm = cconj(sm[rslot<COLS>(sl, k == 0 ? 0 : m - k, spitch, S)]);
                C e = cscale(cadd(zk, zm), (R)0.5);
                C o = cscale(csub(zk, zm), (R)0.5);
                C V = cadd(e, cmul_is(cmul(__ldg(&A.ta[k]), o), -1));
                C w = __ldg(&A.tb[k]);
                outR[gout<R, COLS>(A, sig, dst ? n - 1 - k : k)] = (R)2 * (w.x * V.x - w.y * V.y);
                if (k > 0 && k < m) {
                    C w2 = __ldg(&A.tb[n - k]);
                    outR[gout<R, COLS>(A, sig, dst ? k - 1 : n - k)] = (R)2 * (w2.x * V.x + w2.y * V.y);
                }
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
        case M_DCT3H: case M_DST3H: {   // z[i] = (v[2i], v[2i+1]) to Makhoul's positions
            const int j0 = mk_perm(2 * i, n), j1 = mk_perm(2 * i + 1, n);
            R a0 = f.x, a1 = f.y;
            if (mode == M_DST3H) { if (j0 & 1) a0 = -a0; if (j1 & 1) a1 = -a1; }
            outR[gout<R, COLS>(A, sig, j0)] = a0;
            outR[gout<R, COLS>(A, sig, j1)] = a1;
        } break;
        }
    }
}

// ===========================================================================
// Fused FFT + transpose (C2C)
//
// One pass replaces "FFT along the aligned axis" followed by "transpose to the
// next pencil layout" of the reference's schedule (e.g. fft(1) then X->Y in
// execute_generic, src/dtfft_plan.F90:1088-1090).  A CTA takes S rows of one
// source rank block that are consecutive along the destination's contiguous
// axis (u), transforms them in registers, stages the spectra in shared memory
// as [point i][row] and writes, for every point i, the S values as one
// contiguous run of the destination.  Point i belongs to the destination rank
// whose segment [i0, i1) contains it; segments carry that rank's base offset
// and strides, so the virtual-rank exchange costs nothing extra.
// ===========================================================================
struct FGroup {           // one source rank block
    i64 src_off;          // element (i = 0, u = 0, w = 0) of the block
    i64 su, sw;           // source strides of u and w (rows are contiguous)
    int nu, nw;
    int seg_first, nseg;
    int tiles_u;
    i64 cta_begin;
};
struct FSeg {             // points [i0, i1) of a group go to one destination rank
    int i0, i1;
    i64 dst_off;          // destination element of (i0, u = 0, w = 0); u has stride 1
    i64 di, dw;
};

template <typename R>
struct FArgs {
    typedef typename CT<R>::T C;
    const C* in;
    C* out;
    const FGroup* groups;
    const FSeg* segs;
    int ngroups;
    int m, sign, S, pitch;
    const C* tw;
    Stages st;
};

template <typename R, int E>
__global__ void __launch_bounds__(sizeof(R) == 8 ? 256 : 512) fft_xpose_kernel(FArgs<R> A) {
    typedef typename CT<R>::T C;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* sm = reinterpret_cast<C*>(smem_raw);
    const int S = A.S, m = A.m, s = A.sign;
    const int T = m / E;
    const int sl = threadIdx.x / T, t = threadIdx.x % T;
    // group of this CTA
    const i64 cta = blockIdx.x;
    int lo = 0, hi = A.ngroups - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (A.groups[mid].cta_begin <= cta) lo = mid; else hi = mid - 1;
    }
    const FGroup g = A.groups[lo];
    const int tile = (int)(cta - g.cta_begin);
    const int u0 = (tile % g.tiles_u) * S;
    const int w = tile / g.tiles_u;
    const int u = u0 + sl;
    const bool live = u < g.nu;
    const C* src = A.in + g.src_off + (i64)u * g.su + (i64)w * g.sw;

    C v[E];
#pragma unroll
    for (int q = 0; q < E; ++q) {
        if (live) v[q] = src[t + T * q];
        else { v[q].x = 0; v[q].y = 0; }
    }
    int Ns = 1;
    const int ns = A.st.ns;
    for (int st = 0; st < ns - 1; ++st) {
        const int rad = A.st.radix[st];
        reg_stage_any<R, E, false, true>(rad, v, t, T, Ns, m, A.tw, s, sm, sl, A.pitch, S);
        __syncthreads();
#pragma unroll
        for (int q = 0; q < E; ++q) v[q] = sm[rslot<false>(sl, t + T * q, A.pitch, S)];
        __syncthreads();
        Ns *= rad;
    }
    if (ns > 0) reg_stage_any<R, E, false, false>(A.st.radix[ns - 1], v, t, T, Ns, m, A.tw, s, sm, sl, A.pitch, S);
    if (ns == 1) __syncthreads();   // no exchange ran: all loads precede the staging writes
    // stage spectra as [i][row] (row stride S+1 keeps the column writes conflict-free)
    const int SP = S + 1;
#pragma unroll
    for (int q = 0; q < E; ++q) sm[(t + T * q) * SP + sl] = v[q];
    __syncthreads();
    const int nu_here = min(S, g.nu - u0);
    for (int k = 0; k < g.nseg; ++k) {
        const FSeg sg = A.segs[g.seg_first + k];
        const int cnt = (sg.i1 - sg.i0) * S;
        C* dst = A.out + sg.dst_off + (i64)w * sg.dw + u0;
        for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
            const int ii = e / S, r = e - ii * S;
            if (r < nu_here) dst[(i64)ii * sg.di + r] = sm[(sg.i0 + ii) * SP + r];
        }
    }
}

// ===========================================================================
// Pipelined persistent FFT kernels (TMA bulk copies + mbarriers)
//
// Persistent CTAs walk a list of tiles (S signals each).  One thread streams
// the rows of upcoming tiles from HBM into a ring of NST shared-memory buffers
// with cp.async.bulk (the Blackwell bulk-copy engine), completion tracked by a
// transaction-count mbarrier per buffer.  The CTA transforms tile k while
// tiles k+1 .. k+NST-1 are in flight, so HBM stays busy through the compute
// and exchange phases.  Each thread reads its points t+T*q from the landed
// buffer, runs the register stages, and stores straight to HBM (plain rows) or
// through the [point][row] staging to each destination rank (fused transpose).
//
// Every mbarrier wait is bounded: on timeout the kernel records an error code
// in g_gb_status, waits (bounded) for its own copies still in flight and
// returns, leaving the context usable.
// ===========================================================================

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_load(void* dst_smem, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst_smem)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ uint32_t mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok;
}
// bounded wait: false after ~2^22 polls (each poll may suspend the thread briefly)
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
    for (int it = 0; it < kWaitLimitDefault; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
// consumer wait with a launch-time limit (kWaitLimitDefault unless a test shortens it)
__device__ __forceinline__ bool mbar_wait_limit(uint64_t* bar, uint32_t parity, int limit) {
    for (int it = 0; it < limit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

template <typename R>
struct PArgs {
    typedef typename CT<R>::T C;
    const C* in;
    C* out;
    // plain rows: signal r at r*m, tile k = rows [k*S, k*S + S)
    i64 nsig;
    // fused: tiles are (group, u-tile, w)
    const FGroup* groups;
    const FSeg* segs;
    int ngroups;
    i64 ntiles;
    int m, sign, S, pitch, nst;
    const C* tw;
    Stages st;
    int* status;            // device status word (bounded-wait timeouts)
};

// Rows of tile `tile`: first source row, row stride, count (fused or plain).
template <typename R, bool FUSED>
__device__ __forceinline__ void tile_rows(const PArgs<R>& A, i64 tile, i64& row0, i64& rstride, int& nrows, int& gi,
                                          int& u0, int& w) {
    if (FUSED) {
        int lo = 0, hi = A.ngroups - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (A.groups[mid].cta_begin <= tile) lo = mid; else hi = mid - 1;
        }
        const FGroup& g = A.groups[lo];
        const int tl = (int)(tile - g.cta_begin);
        u0 = (tl % g.tiles_u) * A.S;
        w = tl / g.tiles_u;
        nrows = min(A.S, g.nu - u0);
        row0 = g.src_off + (i64)u0 * g.su + (i64)w * g.sw;
        rstride = g.su;
        gi = lo;
    } else {
        row0 = tile * A.S * (i64)A.m;
        nrows = (int)min((i64)A.S, A.nsig - tile * A.S);
        rstride = A.m;
        gi = 0; u0 = 0; w = 0;
    }
}

template <typename R, bool FUSED>
__device__ __forceinline__ void issue_tile(const PArgs<R>& A, i64 tile, typename CT<R>::T* buf, uint64_t* bar) {
    typedef typename CT<R>::T C;
    i64 row0, rs;
    int nrows, gi, u0, w;
    tile_rows<R, FUSED>(A, tile, row0, rs, nrows, gi, u0, w);
    const uint32_t row_bytes = (uint32_t)(A.m * sizeof(C));
    mbar_expect_tx(bar, row_bytes * (uint32_t)nrows);
    if (rs == A.m) {
        bulk_load(buf, A.in + row0, row_bytes * (uint32_t)nrows, bar);
    } else {
        for (int r = 0; r < nrows; ++r) bulk_load(buf + (i64)r * A.m, A.in + row0 + (i64)r * rs, row_bytes, bar);
    }
}

// ---- stage schedules: runtime (any supported length) or compile time (hot lengths) ----
template <int E_>
struct RtSch {
    static constexpr int E = E_;
    static constexpr bool CT = false;
};
template <int E_, int... Rs>
struct CtSch {
    static constexpr int E = E_;
    static constexpr bool CT = true;
    static constexpr int M = (Rs * ... * 1);
    static constexpr int T = M / E_;
};

// One compile-time radix stage: T, M, RAD and Ns are constants, so the
// butterfly index, the twiddle exponent and the exchange address reduce to
// per-thread bases plus immediate offsets.
template <typename R, int E, int T, int M, int RAD, int Ns, bool EX>
__device__ __forceinline__ void ct_stage(typename CT<R>::T (&v)[E], int t, const typename CT<R>::T* __restrict__ tw,
                                         int s, typename CT<R>::T* xrow) {
    typedef typename CT<R>::T C;
    constexpr int B = E / RAD;
    constexpr int tstep = M / (Ns * RAD);
#pragma unroll
    for (int b = 0; b < B; ++b) {
        const int j = t + b * T;
        const int k = (T % Ns == 0) ? (t % Ns) : (j % Ns);
        C w[RAD];
#pragma unroll
        for (int r = 0; r < RAD; ++r) w[r] = v[b + r * B];
        if constexpr (Ns > 1) {
            const int e1 = tstep * k;   // W^0 = 1 sits at tw[0]: no branch on k
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
            for (int r = 0; r < RAD; ++r) xrow[rpad(base + r * Ns)] = w[r];
        } else {
#pragma unroll
            for (int r = 0; r < RAD; ++r) v[b + r * B] = w[r];
        }
    }
}

template <typename R, int E, int T, int M, int Ns, int RAD, int... Rest>
__device__ __forceinline__ void ct_stages(typename CT<R>::T (&v)[E], int t, const typename CT<R>::T* tw, int s,
                                          typename CT<R>::T* xrow) {
    if constexpr (sizeof...(Rest) == 0) {
        ct_stage<R, E, T, M, RAD, Ns, false>(v, t, tw, s, xrow);
    } else {
        ct_stage<R, E, T, M, RAD, Ns, true>(v, t, tw, s, xrow);
        __syncthreads();
#pragma unroll
        for (int q = 0; q < E; ++q) v[q] = xrow[rpad(t + T * q)];
        __syncthreads();
        ct_stages<R, E, T, M, Ns * RAD, Rest...>(v, t, tw, s, xrow);
    }
}

template <typename R, int E, int... Rs>
__device__ __forceinline__ void run_sched(CtSch<E, Rs...>, typename CT<R>::T (&v)[E], int t, int T, int m,
                                          const Stages&, const typename CT<R>::T* tw, int s, typename CT<R>::T* xbuf,
                                          int sl, int pitch, int S) {
    (void)T; (void)m; (void)S;
    ct_stages<R, E, CtSch<E, Rs...>::T, CtSch<E, Rs...>::M, 1, Rs...>(v, t, tw, s, xbuf + (i64)sl * pitch);
}

template <typename R, int E>
__device__ __forceinline__ void run_sched(RtSch<E>, typename CT<R>::T (&v)[E], int t, int T, int m, const Stages& st_,
                                          const typename CT<R>::T* tw, int s, typename CT<R>::T* xbuf, int sl, int pitch,
                                          int S) {
    int Ns = 1;
    const int ns = st_.ns;
    for (int st = 0; st < ns - 1; ++st) {
        const int rad = st_.radix[st];
        reg_stage_any<R, E, false, true>(rad, v, t, T, Ns, m, tw, s, xbuf, sl, pitch, S);
        __syncthreads();
#pragma unroll
        for (int q = 0; q < E; ++q) v[q] = xbuf[rslot<false>(sl, t + T * q, pitch, S)];
        __syncthreads();
        Ns *= rad;
    }
    if (ns > 0) reg_stage_any<R, E, false, false>(st_.radix[ns - 1], v, t, T, Ns, m, tw, s, xbuf, sl, pitch, S);
}

template <typename R, typename SCH, bool FUSED>
__global__ void __launch_bounds__(sizeof(R) == 8 ? 256 : 512) fft_pipe_kernel(PArgs<R> A) {
    typedef typename CT<R>::T C;
    constexpr int E = SCH::E;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw);
    const int S = A.S, m = A.m, s = A.sign, NST = A.nst;
    C* inbuf = reinterpret_cast<C*>(smem_raw + 128);
    C* xbuf = inbuf + (i64)NST * S * m;
    const int T = m / E;
    const int sl = threadIdx.x / T, t = threadIdx.x % T;

    if (threadIdx.x == 0) {
        for (int b = 0; b < NST; ++b) mbar_init(&bars[b], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int j = 0; j < NST; ++j) {
            const i64 tj = blockIdx.x + (i64)j * gridDim.x;
            if (tj < A.ntiles) issue_tile<R, FUSED>(A, tj, inbuf + (i64)j * S * m, &bars[j]);
        }
    }
    int k = 0;
    for (i64 tile = blockIdx.x; tile < A.ntiles; tile += gridDim.x, ++k) {
        const int b = k % NST;
        const uint32_t par = (uint32_t)((k / NST) & 1);
        const bool ok = mbar_wait_bounded(&bars[b], par);
        if (__syncthreads_or(!ok)) {
            // give up: record, drain this CTA's copies still in flight, leave
            if (threadIdx.x == 0) {
                report_status(A.status, 1);
                for (int j = 0; j < NST; ++j) {
                    const i64 tj = tile + (i64)j * gridDim.x;
                    if (tj >= A.ntiles) break;
                    mbar_wait_bounded(&bars[(k + j) % NST], (uint32_t)(((k + j) / NST) & 1));
                }
            }
            __syncthreads();
            return;
        }
        i64 row0, rs;
        int nrows, gi, u0, w;
        tile_rows<R, FUSED>(A, tile, row0, rs, nrows, gi, u0, w);
        const bool live = sl < nrows;
        const C* mine = inbuf + (i64)b * S * m + (i64)sl * m;
        C v[E];
#pragma unroll
        for (int q = 0; q < E; ++q) v[q] = mine[t + T * q];
        __syncthreads();   // buffer b fully read: refill it with tile + NST*grid
        if (threadIdx.x == 0) {
            fence_async_smem();
            const i64 tn = tile + (i64)NST * gridDim.x;
            if (tn < A.ntiles) issue_tile<R, FUSED>(A, tn, inbuf + (i64)b * S * m, &bars[b]);
        }
        run_sched<R>(SCH{}, v, t, T, m, A.st, A.tw, s, xbuf, sl, A.pitch, S);
        if constexpr (!FUSED) {
            if (live) {
                C* dst = A.out + row0 + (i64)sl * m;
#pragma unroll
                for (int q = 0; q < E; ++q) dst[t + T * q] = v[q];
            }
        } else {
            const int SP = S + 1;
            __syncthreads();
#pragma unroll
            for (int q = 0; q < E; ++q) xbuf[(t + T * q) * SP + sl] = v[q];
            __syncthreads();
            const FGroup& g = A.groups[gi];
            const int lgS = __ffs(S) - 1;   // S is a power of two
            for (int kk = 0; kk < g.nseg; ++kk) {
                const FSeg sg = A.segs[g.seg_first + kk];
                const int cnt = (sg.i1 - sg.i0) << lgS;
                C* dst = A.out + sg.dst_off + (i64)w * sg.dw + u0;
                const int di = (int)sg.di;
                const C* src = xbuf + sg.i0 * SP;
                for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
                    const int ii = e >> lgS, r = e & (S - 1);
                    if (r < nrows) dst[ii * di + r] = src[ii * SP + r];
                }
            }
        }
    }
}


// Lengths with a compile-time schedule, and their points per thread.
inline int ct_points_per_thread(int m) {
    switch (m) {
    case 8: case 32: case 64: case 512: return 8;
    case 16: case 128: case 256: case 1024: case 2048: case 4096: return 16;
    case 96: case 384: case 768: return 24;
    }
    return 0;
}

// Kernel entry points of one precision (defined in fft_inst_f32.cu / fft_inst_f64.cu).
template <typename R>
struct KPtr {
    static void* reg(int E, bool cols, bool c2c);    // fft_reg_kernel
    static void* generic(bool cols);                 // fft_kernel
    static void* xpose(int E);                       // fft_xpose_kernel
    static void* pipe(int m, int E, bool fused);     // fft_pipe_kernel
};

}  // namespace gb
