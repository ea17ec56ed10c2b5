// Runtime-schedule tile kernels: the warp-row tile design of fft_tile.cuh for
// every row length M with a register schedule of at most 32 threads per row
// (E = M / T points per thread, every radix dividing E; M * element size a
// multiple of 16 bytes for the bulk copies).
//
// A warp holds RPW = 32 / T rows at once (lane = row-in-warp * T + t); the
// radix of each stage is read at run time from the launch's schedule, so one
// instantiation per points-per-thread count E covers every length with that E.
// The Stockham exchange runs in the row's own slot of the tile buffer
// (XOR-swizzled when M % 16 == 0), with __syncwarp between stages.
//
//  fft_rtile_kernel       - plain rows: spectra go back into the row slots and
//                           the whole tile (contiguous rows) leaves with one
//                           cp.async.bulk store; the slot is reloaded once
//                           that store has read it.
//  fft_rtile_xpose_kernel - rows fused with the grid transpose: a tile is S
//                           rows along the destination's contiguous axis u
//                           times K slices along w, so small rows still make
//                           tiles of tens of KB; store warps write every
//                           (point, slice) as one S-element run.
//
// Every mbarrier wait is bounded (status word, abort flag), as in fft_tile.cuh.
#pragma once

#include "fft_tile.cuh"

namespace gb {

template <typename R>
struct RtArgs {
    typedef typename CT<R>::T C;
    const C* in;
    C* out;
    const C* tw;          // W_M^(sign*e), e < M, for this launch's direction
    int M, T, rpw;        // row length, threads per row, rows per warp
    int swz;              // exchange / read-out swizzles (M % 16 == 0)
    Stages st;            // radices, first stage first
    i64 nsig;             // plain: rows (row r at r*M of in and out)
    const FGroup* groups; // xpose
    const FSeg* segs;
    int ngroups;
    i64 ntiles;
    int S, K;             // rows along u per tile, w slices per tile (xpose; K = 1 plain)
    int nst;              // ring depth
    int pair_ok;
    int* status;
};

__device__ __forceinline__ int rxi(int i, int swz) { return swz ? xsw(i) : i; }

// One radix stage with run-time T, Ns, M; EX: write the Stockham exchange.
template <typename R, int SG, int E, int RAD, bool EX>
__device__ __forceinline__ void rt_stage(typename CT<R>::T (&v)[E], int t, int T, int Ns, int M,
                                         const typename CT<R>::T* __restrict__ tw, typename CT<R>::T* row, int swz,
                                         bool live) {
    typedef typename CT<R>::T C;
    constexpr int B = E / RAD;
    const int tstep = M / (Ns * RAD);
#pragma unroll
    for (int b = 0; b < B; ++b) {
        const int j = t + b * T;
        const int k = j % Ns;
        C w[RAD];
#pragma unroll
        for (int r = 0; r < RAD; ++r) w[r] = v[b + r * B];
        if (Ns > 1) {
            const int e1 = tstep * k;
#pragma unroll
            for (int r = 1; r < RAD; ++r) w[r] = cmul(w[r], __ldg(&tw[e1 * r]));
        }
        dft_any<R, RAD>(w, SG);
        if constexpr (EX) {
            const int base = (j - k) * RAD + k;
            if (live) {
#pragma unroll
                for (int r = 0; r < RAD; ++r) row[rxi(base + r * Ns, swz)] = w[r];
            }
        } else {
#pragma unroll
            for (int r = 0; r < RAD; ++r) v[b + r * B] = w[r];
        }
    }
}

template <typename R, int SG, int E, bool EX>
__device__ __forceinline__ void rt_stage_any(int rad, typename CT<R>::T (&v)[E], int t, int T, int Ns, int M,
                                             const typename CT<R>::T* tw, typename CT<R>::T* row, int swz, bool live) {
    switch (rad) {
    case 2: if constexpr (E % 2 == 0) rt_stage<R, SG, E, 2, EX>(v, t, T, Ns, M, tw, row, swz, live); break;
    case 3: if constexpr (E % 3 == 0) rt_stage<R, SG, E, 3, EX>(v, t, T, Ns, M, tw, row, swz, live); break;
    case 4: if constexpr (E % 4 == 0) rt_stage<R, SG, E, 4, EX>(v, t, T, Ns, M, tw, row, swz, live); break;
    case 5: if constexpr (E % 5 == 0) rt_stage<R, SG, E, 5, EX>(v, t, T, Ns, M, tw, row, swz, live); break;
    case 7: if constexpr (E % 7 == 0) rt_stage<R, SG, E, 7, EX>(v, t, T, Ns, M, tw, row, swz, live); break;
    case 8: if constexpr (E % 8 == 0) rt_stage<R, SG, E, 8, EX>(v, t, T, Ns, M, tw, row, swz, live); break;
    case 16: if constexpr (E % 16 == 0) rt_stage<R, SG, E, 16, EX>(v, t, T, Ns, M, tw, row, swz, live); break;
    }
}

// Transform the row in `row` (lanes t < T of this row group).  Dead lanes (no
// row, or past the tile's rows) run on zeros without touching shared memory
// except to read, so every lane reaches every __syncwarp.  The spectrum ends
// in registers: v[q] = point t + T*q.
template <typename R, int SG, int E>
__device__ __forceinline__ void rt_row_fft(typename CT<R>::T (&v)[E], typename CT<R>::T* row, bool live, int t,
                                           const RtArgs<R>& A) {
    const int T = A.T, M = A.M;
#pragma unroll
    for (int q = 0; q < E; ++q) {
        if (live) v[q] = row[t + T * q];
        else { v[q].x = 0; v[q].y = 0; }
    }
    __syncwarp();
    int Ns = 1;
    const int ns = A.st.ns;
    for (int s = 0; s < ns - 1; ++s) {
        const int rad = A.st.radix[s];
        rt_stage_any<R, SG, E, true>(rad, v, t, T, Ns, M, A.tw, row, A.swz, live);
        __syncwarp();
#pragma unroll
        for (int q = 0; q < E; ++q) v[q] = row[rxi(t + T * q, A.swz)];
        __syncwarp();
        Ns *= rad;
    }
    if (ns > 0) rt_stage_any<R, SG, E, false>(A.st.radix[ns - 1], v, t, T, Ns, M, A.tw, row, A.swz, live);
    __syncwarp();
}

__device__ __forceinline__ void bulk_store(void* dst, const void* src_smem, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_u32(src_smem)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read_le1() { asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// ---------------------------------------------------------------------------
// Plain rows
// ---------------------------------------------------------------------------
template <typename R, int SG, int NW, int E>
__global__ void __launch_bounds__(32 * NW, 1) fft_rtile_kernel(RtArgs<R> A) {
    typedef typename CT<R>::T C;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw);
    C* ring = reinterpret_cast<C*>(smem_raw + kTileHdrPlain);
    const int S = A.S, NST = A.nst, M = A.M, T = A.T;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int rw = lane / T, t = lane - rw * T;
    const bool lane_on = rw < A.rpw;
    const int rows_per_pass = NW * A.rpw;
    const uint32_t row_bytes = (uint32_t)(M * sizeof(C));

    if (threadIdx.x == 0) {
        for (int b = 0; b < NST; ++b) mbar_init(&bars[b], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    auto issue = [&](i64 tile, int b) {
        const i64 r0 = tile * S;
        const int nr = (int)min((i64)S, A.nsig - r0);
        mbar_expect_tx(&bars[b], row_bytes * (uint32_t)nr);
        bulk_load(ring + (i64)b * S * M, A.in + r0 * M, row_bytes * (uint32_t)nr, &bars[b]);
    };
    if (threadIdx.x == 0) {
        // the first NST - 1 tiles; each later load waits for the store that frees its buffer
        for (int j = 0; j < NST - 1; ++j) {
            const i64 tj = blockIdx.x + (i64)j * gridDim.x;
            if (tj < A.ntiles) issue(tj, j);
        }
    }
    int b = 0;
    uint32_t par = 0;
    for (i64 tile = blockIdx.x; tile < A.ntiles; tile += gridDim.x) {
        const bool ok = mbar_wait_bounded(&bars[b], par);
        if (__syncthreads_or(!ok)) {
            if (threadIdx.x == 0) {
                atomicExch(A.status, 1);
                int bb = b;
                uint32_t pp = par;
                for (int j = 0; j < NST - 1; ++j) {
                    const i64 tj = tile + (i64)j * gridDim.x;
                    if (tj >= A.ntiles) break;
                    mbar_wait_bounded(&bars[bb], pp);
                    if (++bb == NST) { bb = 0; pp ^= 1; }
                }
                bulk_wait_all();
            }
            __syncthreads();
            return;
        }
        const i64 r0 = tile * S;
        const int nrows = (int)min((i64)S, A.nsig - r0);
        C* tb = ring + (i64)b * S * M;
        for (int base = warp * A.rpw; base < nrows; base += rows_per_pass) {
            const int rl = base + rw;
            const bool live = lane_on && rl < nrows;
            C* row = tb + (i64)(live ? rl : base) * M;
            C v[E];
            rt_row_fft<R, SG, E>(v, row, live, t, A);
            if (live) {
#pragma unroll
                for (int q = 0; q < E; ++q) row[t + T * q] = v[q];
            }
        }
        fence_async_smem();
        __syncthreads();
        if (threadIdx.x == 0) {
            bulk_store(A.out + r0 * M, tb, row_bytes * (uint32_t)nrows);
            bulk_commit();
            // the buffer stored one tile ago has been read: load tile + NST - 1 into it
            bulk_wait_read_le1();
            const i64 tn = tile + (i64)(NST - 1) * gridDim.x;
            if (tn < A.ntiles) issue(tn, b == 0 ? NST - 1 : b - 1);
        }
        if (++b == NST) { b = 0; par ^= 1; }
    }
    if (threadIdx.x == 0) bulk_wait_all();
}

// ---------------------------------------------------------------------------
// Rows fused with the transpose (warp-specialised, K slices along w per tile)
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ void rt_geom(const RtArgs<R>& A, i64 tile, int& gi, int& u0, int& w0, int& nu, int& nk) {
    int lo = 0, hi = A.ngroups - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (A.groups[mid].cta_begin <= tile) lo = mid; else hi = mid - 1;
    }
    const FGroup& g = A.groups[lo];
    const int tl = (int)(tile - g.cta_begin);
    u0 = (tl % g.tiles_u) * A.S;
    w0 = (tl / g.tiles_u) * A.K;
    nu = min(A.S, g.nu - u0);
    nk = min(A.K, g.nw - w0);
    gi = lo;
}

template <typename R>
__device__ __forceinline__ void rt_issue(const RtArgs<R>& A, i64 tile, typename CT<R>::T* buf, uint64_t* bar) {
    typedef typename CT<R>::T C;
    int gi, u0, w0, nu, nk;
    rt_geom<R>(A, tile, gi, u0, w0, nu, nk);
    const FGroup& g = A.groups[gi];
    const uint32_t row_bytes = (uint32_t)(A.M * sizeof(C));
    mbar_expect_tx(bar, row_bytes * (uint32_t)(nu * nk));
    for (int kw = 0; kw < nk; ++kw) {
        const C* src = A.in + g.src_off + (i64)u0 * g.su + (i64)(w0 + kw) * g.sw;
        C* dst = buf + (i64)kw * A.S * A.M;
        if (g.su == A.M) bulk_load(dst, src, row_bytes * (uint32_t)nu, bar);
        else
            for (int r = 0; r < nu; ++r) bulk_load(dst + (i64)r * A.M, src + (i64)r * g.su, row_bytes, bar);
    }
}

template <typename R, int SG, int NCW, int NSW, int E>
__global__ void __launch_bounds__(32 * (NCW + NSW), 1) fft_rtile_xpose_kernel(RtArgs<R> A) {
    typedef typename CT<R>::T C;
    constexpr int ES = (int)sizeof(C);
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw);
    uint64_t* done = full + kTileMaxNst;
    uint64_t* empty = full + 2 * kTileMaxNst;
    volatile int* abort_flag = reinterpret_cast<volatile int*>(smem_raw + 24 * kTileMaxNst);
    C* ring = reinterpret_cast<C*>(smem_raw + kTileHdrXpose);
    const int S = A.S, K = A.K, NST = A.nst, M = A.M, T = A.T;
    const i64 tile_elems = (i64)S * K * M;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int lgS = __ffs(S) - 1;
    const int lgNP = ES == 8 ? lgS - 1 : lgS;
    const int lgsh = ES == 8 ? (4 - lgNP) : (3 - lgNP);
    const int swz = A.swz;

    if (threadIdx.x == 0) {
        for (int b = 0; b < NST; ++b) {
            mbar_init(&full[b], 1);
            mbar_init(&done[b], NCW);
            mbar_init(&empty[b], NSW);
        }
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    if (warp < NCW) {
        const int rw = lane / T, t = lane - rw * T;
        const bool lane_on = rw < A.rpw;
        const int rows_per_pass = NCW * A.rpw;
        int b = 0;
        uint32_t par = 0;
        for (i64 tile = blockIdx.x; tile < A.ntiles; tile += gridDim.x) {
            if (!mbar_wait_or_abort(&full[b], par, abort_flag)) {
                if (lane == 0) { atomicExch(A.status, 1); *abort_flag = 1; }
                return;
            }
            int gi, u0, w0, nu, nk;
            rt_geom<R>(A, tile, gi, u0, w0, nu, nk);
            C* tb = ring + (i64)b * tile_elems;
            const int nrows = S * nk;                     // slot index = kw * S + u
            for (int base = warp * A.rpw; base < nrows; base += rows_per_pass) {
                const int rl = base + rw;
                const bool live = lane_on && rl < nrows && (rl & (S - 1)) < nu;
                C* row = tb + (i64)(live ? rl : base) * M;
                C v[E];
                rt_row_fft<R, SG, E>(v, row, live, t, A);
                if (live) {
                    const int ru = rl & (S - 1);
#pragma unroll
                    for (int q = 0; q < E; ++q) row[swz ? osw<ES>(ru, t + T * q, lgsh) : t + T * q] = v[q];
                }
            }
            fence_async_smem();
            __syncwarp();
            if (lane == 0) mbar_arrive(&done[b]);
            if (++b == NST) { b = 0; par ^= 1; }
        }
        return;
    }

    const int st = threadIdx.x - NCW * 32;
    const bool producer = warp == NCW;
    uint32_t issued_par = 0;
    if (producer && lane == 0) {
        for (int j = 0; j < NST; ++j) {
            const i64 tj = blockIdx.x + (i64)j * gridDim.x;
            if (tj < A.ntiles) rt_issue<R>(A, tj, ring + (i64)j * tile_elems, &full[j]);
        }
    }
    const int lp = st & ((1 << lgNP) - 1);
    const int g0 = st >> lgNP;
    const int gstep = (32 * NSW) >> lgNP;
    int b = 0;
    uint32_t par = 0;
    bool failed = false;
    for (i64 tile = blockIdx.x; tile < A.ntiles; tile += gridDim.x) {
        if (!mbar_wait_or_abort(&done[b], par, abort_flag)) { failed = true; break; }
        int gi, u0, w0, nu, nk;
        rt_geom<R>(A, tile, gi, u0, w0, nu, nk);
        const C* tb = ring + (i64)b * tile_elems;
        const FGroup& g = A.groups[gi];
        for (int kk = 0; kk < g.nseg; ++kk) {
            const FSeg sg = A.segs[g.seg_first + kk];
            const int npts = sg.i1 - sg.i0;
            for (int kw = 0; kw < nk; ++kw) {
                C* dbase = A.out + sg.dst_off + (i64)(w0 + kw) * sg.dw + u0;
                const C* ts = tb + (i64)kw * S * M;
                if constexpr (ES == 8) {
                    const int r0 = 2 * lp;
                    if (r0 < nu) {
                        const bool two = r0 + 1 < nu;
                        const C* s0 = ts + r0 * M;
                        const C* s1 = s0 + M;
#pragma unroll 4
                        for (int ii = g0; ii < npts; ii += gstep) {
                            const int i = sg.i0 + ii;
                            const C a = s0[swz ? osw<ES>(r0, i, lgsh) : i];
                            C* d = dbase + (i64)ii * sg.di + r0;
                            if (two) {
                                const C c = s1[swz ? osw<ES>(r0 + 1, i, lgsh) : i];
                                if (A.pair_ok) {
                                    float4 q4;
                                    q4.x = a.x; q4.y = a.y; q4.z = c.x; q4.w = c.y;
                                    *reinterpret_cast<float4*>(d) = q4;
                                } else {
                                    d[0] = a;
                                    d[1] = c;
                                }
                            } else {
                                d[0] = a;
                            }
                        }
                    }
                } else {
                    const int r0 = lp;
                    if (r0 < nu) {
                        const C* s0 = ts + r0 * M;
                        for (int ii = g0; ii < npts; ii += gstep) {
                            const int i = sg.i0 + ii;
                            dbase[(i64)ii * sg.di + r0] = s0[swz ? osw<ES>(r0, i, lgsh) : i];
                        }
                    }
                }
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[b]);
        if (producer) {
            if (!mbar_wait_or_abort(&empty[b], par, abort_flag)) { failed = true; break; }
            if (lane == 0) {
                const i64 tn = tile + (i64)NST * gridDim.x;
                if (tn < A.ntiles) {
                    rt_issue<R>(A, tn, const_cast<C*>(tb), &full[b]);
                    issued_par = (issued_par & ~(1u << b)) | ((par ^ 1u) << b);
                }
            }
            __syncwarp();
        }
        if (++b == NST) { b = 0; par ^= 1; }
    }
    if (failed) {
        if (lane == 0) { atomicExch(A.status, 1); *abort_flag = 1; }
        if (producer && lane == 0) {
            for (int j = 0; j < NST && blockIdx.x + (i64)j * gridDim.x < A.ntiles; ++j)
                mbar_wait_bounded(&full[j], (issued_par >> j) & 1u);
        }
    }
}

// Runtime-schedule entry points of one precision (fft_rtile_*.cu); nullptr
// when E has no instantiation.
template <typename R>
struct RtilePtr {
    static void* get(int E, int sign, bool xpose);
    static bool has(int E);
};
// warps of the instantiations
constexpr int kRtilePlainWarps = 4;
constexpr int kRtileComputeWarps = 3;
constexpr int kRtileStoreWarps = 5;

}  // namespace gb
