// Two-factor batched FFT for the 7-smooth lengths m = M1 * M2 (40 .. 1024)
// that have no warp-per-row tile kernel (105, 175, 225, 378, 1000, ...): the
// four-step decomposition inside one CTA, with both factor transforms held in
// one thread's registers.  Three forms: fft2f_kernel (rows or columns, loads
// straight from global memory), fft2f_pipe_kernel (contiguous rows streamed
// through a bulk-copy ring) and fft2f_xpose_kernel (rows fused with the grid
// transpose).  C2C rows and columns; rows of the real modes (R2C / C2R
// through an m-point core: half length for even n, full length for odd n),
// whose pre-processing is folded into phase A's loads and post-processing
// into phase B's stores (R2C of even n pairs outputs k and m - k, so it
// stages the core spectrum in shared memory for a phase C).
//
//   X[k1 + M1 k2] = sum_j2 W_M2^(j2 k2) [ W_m^(j2 k1) sum_j1 x[j2 + M2 j1] W_M1^(j1 k1) ]
//
// Phase A: for every (signal, j2) a thread loads the M1 points j2 + M2 j1
// straight from global memory, transforms them (codelet DFT_M1), applies the
// twiddles W_m^(j2 k1) and writes the row k1 of its signal's M1 x M2
// intermediate into shared memory.  Phase B: for every (signal, k1) a thread
// reads the M2 values of row k1, transforms them (DFT_M2) and stores outputs
// k1 + M1 k2 straight to global memory.  One barrier per CTA; every point is
// read from and written to HBM once.  Rows: consecutive threads take
// consecutive j2 (k1) of a signal, the intermediate rows are padded to an odd
// pitch so phase B's strided reads stay conflict-free.  Columns: consecutive
// threads take consecutive signals (adjacent columns), so every load and
// store is a contiguous run across the warp.
//
// The codelets are Cooley-Tukey in registers: DFT_N = DFT_P over the N/P
// interleaved subsequences, twiddles W_N^(q k) as compile-time constants
// (ktrig.h), then DFT_(N/P) recursively, with P the radix butterflies of
// fft_kernels.cuh (2, 3, 4, 5, 7, 8, 16).
#pragma once
#include <type_traits>

#include "fft_kernels.cuh"
#include "ktrig.h"

namespace gb {

template <int B, int E, typename F>
__device__ __forceinline__ void sfor(F&& f) {
    if constexpr (B < E) {
        f(std::integral_constant<int, B>{});
        sfor<B + 1, E>(f);
    }
}

// Radix split of a codelet of N points: the first butterfly (16, 8, 7, 5, 4,
// 3, 2) that divides N and leaves a second factor above 1.
template <int N>
constexpr int codelet_split() {
    constexpr int cand[7] = {16, 8, 7, 5, 4, 3, 2};
    for (int i = 0; i < 7; ++i)
        if (N % cand[i] == 0 && N > cand[i]) return cand[i];
    return N;
}

// v[k] <- sum_j v[j] exp(s 2 pi i j k / N), natural order in and out
template <typename R, int N, typename C>
__device__ __forceinline__ void dftc(C* v, int s) {
    if constexpr (N == 1) {
        (void)v; (void)s;
    } else if constexpr (N == 2 || N == 3 || N == 4 || N == 5 || N == 7 || N == 8 || N == 16) {
        dft_any<R, N>(v, s);
    } else {
        constexpr int P = codelet_split<N>(), Q = N / P;
        static_assert(P * Q == N && Q > 1, "codelet split");
        C a[Q][P];
        sfor<0, Q>([&](auto qc) {
            constexpr int q = decltype(qc)::value;
            sfor<0, P>([&](auto rc) { a[q][decltype(rc)::value] = v[q + Q * decltype(rc)::value]; });
            dft_any<R, P>(a[q], s);
            if constexpr (q > 0) {
                sfor<1, P>([&](auto kc) {
                    constexpr int k = decltype(kc)::value;
                    constexpr double c = ktrig::cos2pi((long long)q * k, N);
                    constexpr double sn = ktrig::sin2pi((long long)q * k, N);
                    C w;
                    w.x = (R)c;
                    w.y = s > 0 ? (R)sn : (R)-sn;
                    a[q][k] = cmul(a[q][k], w);
                });
            }
        });
        sfor<0, P>([&](auto kc) {
            constexpr int k1 = decltype(kc)::value;
            C b[Q];
            sfor<0, Q>([&](auto qc) { b[decltype(qc)::value] = a[decltype(qc)::value][k1]; });
            dftc<R, Q>(b, s);
            sfor<0, Q>([&](auto k2c) { v[k1 + P * decltype(k2c)::value] = b[decltype(k2c)::value]; });
        });
    }
}

template <typename R>
struct F2Args {
    typedef typename CT<R>::T C;
    const void* in;
    void* out;
    const C* tw;            // W_m^e = exp(-2 pi i e / m), e < m
    const C* ta;            // real modes: the pre/post twiddles of the shared-memory kernel's modes
    int n;                  // real modes: reals per signal
    i64 nsig;
    i64 idist, odist;       // rows: signal s at s * idist / s * odist, unit stride
    i64 plane;              // columns: signal s = column s % ncols of plane s / ncols,
    int ld, ncols;          //          point k at k * ld
    int sign;
    int per;                // signals per CTA
};

template <typename R, bool COLS>
__device__ __forceinline__ i64 f2_at(const F2Args<R>& A, i64 s, int k, bool in) {
    if (COLS) return (s / A.ncols) * A.plane + (s % A.ncols) + (i64)k * A.ld;
    return s * (in ? A.idist : A.odist) + k;
}

// Point j of the core sequence of signal sg (phase A).
template <typename R, int MODE, bool COLS>
__device__ __forceinline__ typename CT<R>::T f2_load(const F2Args<R>& A, i64 sg, int j, int m) {
    typedef typename CT<R>::T C;
    const C* inC = reinterpret_cast<const C*>(A.in);
    const R* inR = reinterpret_cast<const R*>(A.in);
    C v;
    if constexpr (MODE == M_C2C) {
        v = inC[f2_at<R, COLS>(A, sg, j, true)];
    } else if constexpr (MODE == M_R2C_HALF) {      // z[j] = x[2j] + i x[2j+1]
        const i64 g = f2_at<R, COLS>(A, sg, 2 * j, true);
        v.x = inR[g]; v.y = inR[g + 1];
    } else if constexpr (MODE == M_R2C_FULL) {
        v.x = inR[f2_at<R, COLS>(A, sg, j, true)]; v.y = 0;
    } else if constexpr (MODE == M_C2R_HALF) {      // Z[j] = E[j] + i O[j] from X[j], X[m - j]
        C xk = inC[f2_at<R, COLS>(A, sg, j, true)];
        C xm = inC[f2_at<R, COLS>(A, sg, m - j, true)];
        if (j == 0) { xk.y = 0; xm.y = 0; }
        const C cxm = cconj(xm);
        const C e = cadd(xk, cxm);
        const C o = cmul(csub(xk, cxm), cconj(A.ta[j]));
        v = cadd(e, cmul_is(o, 1));
    } else {                                        // M_C2R_FULL: Hermitian extension
        if (j <= A.n / 2) { v = inC[f2_at<R, COLS>(A, sg, j, true)]; if (j == 0) v.y = 0; }
        else v = cconj(inC[f2_at<R, COLS>(A, sg, A.n - j, true)]);
    }
    return v;
}

// Core spectrum point k of signal sg (phase B); R2C of even n keeps it in zs.
template <typename R, int MODE, bool COLS>
__device__ __forceinline__ void f2_store(const F2Args<R>& A, i64 sg, int k, typename CT<R>::T z,
                                         typename CT<R>::T* zs) {
    typedef typename CT<R>::T C;
    C* outC = reinterpret_cast<C*>(A.out);
    R* outR = reinterpret_cast<R*>(A.out);
    if constexpr (MODE == M_C2C) {
        outC[f2_at<R, COLS>(A, sg, k, false)] = z;
    } else if constexpr (MODE == M_R2C_HALF) {
        zs[k] = z;
    } else if constexpr (MODE == M_R2C_FULL) {
        if (k <= A.n / 2) outC[f2_at<R, COLS>(A, sg, k, false)] = z;
    } else if constexpr (MODE == M_C2R_HALF) {      // y[2k] = Re z, y[2k+1] = Im z
        const i64 g = f2_at<R, COLS>(A, sg, 2 * k, false);
        outR[g] = z.x; outR[g + 1] = z.y;
    } else {
        outR[f2_at<R, COLS>(A, sg, k, false)] = z.x;
    }
}

template <typename R, int M1, int M2, int MODE, bool COLS>
__global__ void __launch_bounds__(256) fft2f_kernel(const F2Args<R> A) {
    typedef typename CT<R>::T C;
    constexpr int M = M1 * M2;
    constexpr int PR = M2 | 1;   // rows: odd pitch of an intermediate row
    static_assert(MODE == M_C2C || !COLS, "real modes run along rows");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* ys = reinterpret_cast<C*>(smem_raw);
    const int per = A.per;
    C* zs = ys + (size_t)per * M1 * PR;            // R2C of even n: the core spectra
    const i64 s0 = (i64)blockIdx.x * per;
    const int ns = (int)min((i64)per, A.nsig - s0);
    if (ns <= 0) return;
    const int s = A.sign;
    // intermediate (signal sl, row k1, column j2)
    auto yat = [&](int sl, int k1, int j2) -> int {
        return COLS ? (k1 * M2 + j2) * per + sl : (sl * M1 + k1) * PR + j2;
    };

    for (int it = threadIdx.x; it < ns * M2; it += blockDim.x) {
        int sl, j2;
        if (COLS) { j2 = it / ns; sl = it - j2 * ns; } else { sl = it / M2; j2 = it - sl * M2; }
        const i64 sg = s0 + sl;
        C v[M1];
#pragma unroll
        for (int j1 = 0; j1 < M1; ++j1) v[j1] = f2_load<R, MODE, COLS>(A, sg, j2 + M2 * j1, M);
        dftc<R, M1>(v, s);
        int e = 0;   // j2 * k1 mod M
#pragma unroll
        for (int k1 = 1; k1 < M1; ++k1) {
            e += j2;
            if (e >= M) e -= M;
            C w = __ldg(&A.tw[e]);
            if (s > 0) w.y = -w.y;
            v[k1] = cmul(v[k1], w);
        }
#pragma unroll
        for (int k1 = 0; k1 < M1; ++k1) ys[yat(sl, k1, j2)] = v[k1];
    }
    __syncthreads();
    for (int it = threadIdx.x; it < ns * M1; it += blockDim.x) {
        int sl, k1;
        if (COLS) { k1 = it / ns; sl = it - k1 * ns; } else { sl = it / M1; k1 = it - sl * M1; }
        const i64 sg = s0 + sl;
        C u[M2];
#pragma unroll
        for (int j2 = 0; j2 < M2; ++j2) u[j2] = ys[yat(sl, k1, j2)];
        dftc<R, M2>(u, s);
#pragma unroll
        for (int k2 = 0; k2 < M2; ++k2) f2_store<R, MODE, COLS>(A, sg, k1 + M1 * k2, u[k2], zs + (size_t)sl * M);
    }
    if constexpr (MODE == M_R2C_HALF) {
        // phase C: X[k] = E[k] - i W_n^k O[k], E / O from Z[k] and conj Z[m - k], k <= m
        __syncthreads();
        C* outC = reinterpret_cast<C*>(A.out);
        for (int it = threadIdx.x; it < ns * (M + 1); it += blockDim.x) {
            const int sl = it / (M + 1), k = it - sl * (M + 1);
            const C* z = zs + (size_t)sl * M;
            const C zk = z[k == M ? 0 : k];
            const C zm = cconj(z[k == 0 ? 0 : M - k]);
            const C e = cscale(cadd(zk, zm), (R)0.5);
            const C o = cscale(csub(zk, zm), (R)0.5);
            const C t = cmul(A.ta[k], o);
            outC[f2_at<R, COLS>(A, s0 + sl, k, false)] = cadd(e, cmul_is(t, -1));
        }
    }
}

// ---------------------------------------------------------------------------
// Fused with the box-list transpose: a CTA takes a tile of S rows (u0 .. u0+S-1
// at one w) of one source rank's block (FGroup, as the tile kernels), runs
// phase A on them as above and, in phase B, writes output point i of row u to
// its destination rank's block (the FSeg holding i): dst_off + (i - i0) di +
// u + w dw.  The intermediate is kept row-fastest ((k1 M2 + j2) * P + r, P = S
// odd-padded) so that phase B's consecutive threads take consecutive rows and
// store runs of S adjacent destination points.
// ---------------------------------------------------------------------------
template <typename R>
struct F2XArgs {
    typedef typename CT<R>::T C;
    const C* in;
    C* out;
    const C* tw;
    const FGroup* groups;
    const FSeg* segs;
    int ngroups;
    int S;                  // rows per tile
    int sign;
};

template <typename R, int M1, int M2>
__global__ void __launch_bounds__(256) fft2f_xpose_kernel(const F2XArgs<R> A) {
    typedef typename CT<R>::T C;
    constexpr int M = M1 * M2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* ys = reinterpret_cast<C*>(smem_raw);
    const int S = A.S, P = A.S | 1;
    const i64 tile = blockIdx.x;
    int lo = 0, hi = A.ngroups - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (A.groups[mid].cta_begin <= tile) lo = mid; else hi = mid - 1;
    }
    const FGroup& g = A.groups[lo];
    const int tl = (int)(tile - g.cta_begin);
    const int u0 = (tl % g.tiles_u) * S, w = tl / g.tiles_u;
    const int nrows = min(S, g.nu - u0);
    const i64 row0 = g.src_off + (i64)u0 * g.su + (i64)w * g.sw;
    const int s = A.sign;

    for (int it = threadIdx.x; it < nrows * M2; it += blockDim.x) {
        const int r = it / M2, j2 = it - r * M2;
        const C* src = A.in + row0 + (i64)r * g.su + j2;
        C v[M1];
#pragma unroll
        for (int j1 = 0; j1 < M1; ++j1) v[j1] = src[M2 * j1];
        dftc<R, M1>(v, s);
        int e = 0;
#pragma unroll
        for (int k1 = 1; k1 < M1; ++k1) {
            e += j2;
            if (e >= M) e -= M;
            C t = __ldg(&A.tw[e]);
            if (s > 0) t.y = -t.y;
            v[k1] = cmul(v[k1], t);
        }
#pragma unroll
        for (int k1 = 0; k1 < M1; ++k1) ys[(k1 * M2 + j2) * P + r] = v[k1];
    }
    __syncthreads();
    const FSeg* sg = A.segs + g.seg_first;
    for (int it = threadIdx.x; it < nrows * M1; it += blockDim.x) {
        const int k1 = it / nrows, r = it - k1 * nrows;
        C u[M2];
#pragma unroll
        for (int j2 = 0; j2 < M2; ++j2) u[j2] = ys[(k1 * M2 + j2) * P + r];
        dftc<R, M2>(u, s);
        int q = 0;   // segment of point i (segments ascend in i and cover the row)
        int i0 = sg[0].i0, i1 = sg[0].i1;
        i64 base = sg[0].dst_off + (i64)w * sg[0].dw + u0 + r, di = sg[0].di;
#pragma unroll
        for (int k2 = 0; k2 < M2; ++k2) {
            const int i = k1 + M1 * k2;
            while (i >= i1 && q + 1 < g.nseg) {
                ++q;
                i0 = sg[q].i0; i1 = sg[q].i1;
                base = sg[q].dst_off + (i64)w * sg[q].dw + u0 + r;
                di = sg[q].di;
            }
            A.out[base + (i64)(i - i0) * di] = u[k2];
        }
    }
}

// ---------------------------------------------------------------------------
// Pipelined rows (contiguous C2C rows, idist = odist = m): persistent CTAs
// stream tiles of `per` rows into a ring of NST shared-memory buffers with
// one cp.async.bulk each (transaction-count mbarriers, bounded waits), so the
// loads of the next tiles are in flight while a tile is transformed; phase A
// reads its points from the buffer instead of global memory.  `per` is even,
// so every tile but the last starts 16-byte aligned; an odd tail of the last
// tile (odd m, odd rows) is read with a plain load.
// ---------------------------------------------------------------------------
template <typename R>
struct F2PArgs {
    typedef typename CT<R>::T C;
    const C* in;
    C* out;
    const C* tw;
    i64 nsig, ntiles;
    int per, nst, sign, wait_limit;
    int* status;
};

template <typename R, int M1, int M2>
__device__ __forceinline__ void f2p_issue(const F2PArgs<R>& A, i64 t, typename CT<R>::T* buf, uint64_t* bar) {
    constexpr int M = M1 * M2;
    const i64 r0 = t * A.per;
    const int nrows = (int)min((i64)A.per, A.nsig - r0);
    const uint32_t elems = (uint32_t)nrows * M;
    const uint32_t bytes = (elems & ~1u) * (uint32_t)sizeof(typename CT<R>::T);   // 16-byte multiple
    mbar_expect_tx(bar, bytes);
    bulk_load(buf, A.in + r0 * M, bytes, bar);
}

template <typename R, int M1, int M2>
__global__ void __launch_bounds__(256) fft2f_pipe_kernel(const F2PArgs<R> A) {
    typedef typename CT<R>::T C;
    constexpr int M = M1 * M2;
    constexpr int PR = M2 | 1;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw);
    const int per = A.per, NST = A.nst, s = A.sign;
    C* inbuf = reinterpret_cast<C*>(smem_raw + 128);
    C* ys = inbuf + (size_t)NST * per * M;
    if (threadIdx.x == 0) {
        for (int b = 0; b < NST; ++b) mbar_init(&bars[b], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        for (int j = 0; j < NST; ++j) {
            const i64 tj = blockIdx.x + (i64)j * gridDim.x;
            if (tj < A.ntiles) f2p_issue<R, M1, M2>(A, tj, inbuf + (size_t)j * per * M, &bars[j]);
        }
    }
    __syncthreads();
    int k = 0;
    for (i64 tile = blockIdx.x; tile < A.ntiles; tile += gridDim.x, ++k) {
        const int b = k % NST;
        const uint32_t par = (uint32_t)((k / NST) & 1);
        const bool ok = mbar_wait_limit(&bars[b], par, A.wait_limit);
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
        const i64 r0 = tile * per;
        const int nrows = (int)min((i64)per, A.nsig - r0);
        C* buf = inbuf + (size_t)b * per * M;
        if ((nrows * M) & 1) {   // odd tail of the last tile
            if (threadIdx.x == 0) buf[nrows * M - 1] = A.in[r0 * M + nrows * M - 1];
            __syncthreads();
        }
        for (int it = threadIdx.x; it < nrows * M2; it += blockDim.x) {
            const int r = it / M2, j2 = it - r * M2;
            const C* src = buf + r * M + j2;
            C v[M1];
#pragma unroll
            for (int j1 = 0; j1 < M1; ++j1) v[j1] = src[M2 * j1];
            dftc<R, M1>(v, s);
            int e = 0;
#pragma unroll
            for (int k1 = 1; k1 < M1; ++k1) {
                e += j2;
                if (e >= M) e -= M;
                C w = __ldg(&A.tw[e]);
                if (s > 0) w.y = -w.y;
                v[k1] = cmul(v[k1], w);
            }
#pragma unroll
            for (int k1 = 0; k1 < M1; ++k1) ys[(r * M1 + k1) * PR + j2] = v[k1];
        }
        __syncthreads();   // buffer b read: refill it with tile + NST * grid
        if (threadIdx.x == 0) {
            fence_async_smem();
            const i64 tn = tile + (i64)NST * gridDim.x;
            if (tn < A.ntiles) f2p_issue<R, M1, M2>(A, tn, buf, &bars[b]);
        }
        for (int it = threadIdx.x; it < nrows * M1; it += blockDim.x) {
            const int r = it / M1, k1 = it - r * M1;
            C u[M2];
#pragma unroll
            for (int j2 = 0; j2 < M2; ++j2) u[j2] = ys[(r * M1 + k1) * PR + j2];
            dftc<R, M2>(u, s);
            C* dst = A.out + (r0 + r) * M + k1;
#pragma unroll
            for (int k2 = 0; k2 < M2; ++k2) dst[M1 * k2] = u[k2];
        }
        __syncthreads();   // the intermediate is rewritten by the next tile
    }
}

inline size_t f2p_smem(int m1, int m2, int per, int nst, size_t es) {
    return 128 + (size_t)nst * per * m1 * m2 * es + (size_t)per * m1 * (m2 | 1) * es;
}

// Compiled pipelined kernels: float, the lengths of the C2C units; nullptr if none.
void* f2_pipe_kernel_f32(int m, int* m1, int* m2);

// Shared memory of a fused tile of S rows.
inline size_t f2x_smem(int m1, int m2, int S, size_t es) { return (size_t)m1 * m2 * (S | 1) * es; }

// Compiled fused kernels: float, core lengths of the C2C units; nullptr if none.
void* f2_xpose_kernel_f32(int m, int* m1, int* m2);

// Shared memory of a CTA of `per` signals.
inline size_t f2_smem(int m1, int m2, bool cols, int per, size_t es, int mode) {
    if (cols) return (size_t)m1 * m2 * per * es;
    return (size_t)per * m1 * (m2 | 1) * es + (mode == M_R2C_HALF ? (size_t)per * m1 * m2 * es : 0);
}

// Compiled two-factor kernels (fft_2f_f32_*.cu): the kernel for a core of m
// points (float) in `mode` (C2C rows or columns; R2C / C2R rows), its
// factors; nullptr when none is compiled.
void* f2_kernel_f32(int m, bool cols, int mode, int* m1, int* m2);

}  // namespace gb
