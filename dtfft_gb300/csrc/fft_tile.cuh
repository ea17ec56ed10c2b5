// Warp-per-row tile kernels: batched C2C rows, optionally fused with the
// virtual-grid transpose that follows them in the execute schedule.
//
// A persistent CTA walks a list of tiles of S rows.  Rows of upcoming tiles
// stream from HBM into a ring of shared-memory buffers with cp.async.bulk
// (completion on a transaction-count mbarrier per buffer), so the loads of
// the next tiles overlap the work on this one.  A tile whose rows are
// contiguous in HBM lands with a single bulk copy.
//
// Each row of M = 32*E points belongs to one warp: lane t keeps points
// t + 32*q (q < E) in registers, every radix stage is local to the thread,
// and the Stockham permutation between stages goes through the row's own
// slot of the tile buffer.  A row therefore needs only __syncwarp between
// stages, never a CTA barrier.  The exchange addresses are XOR-swizzled,
// i ^ ((i >> 4) & 15), which keeps the radix-16 schedules free of
// shared-memory bank conflicts without padding the rows.
//
// Output:
//  plain (fft_tile_kernel) - the last stage stores straight from registers
//           to the output row (32 lanes on consecutive addresses);
//  xpose (fft_tile_xpose_kernel) - warp-specialised: compute warps transform
//           the rows of tile k and write the spectra back into the row slots
//           while store warps write earlier tiles out transposed.  For every
//           point i the S rows of a tile are consecutive along the
//           destination's contiguous axis, so each point becomes one
//           S-element run (128 B for S = 16 complex64 rows or S = 8
//           complex128 rows) of the destination rank's block.  A read-out
//           swizzle keeps those column reads conflict-free.  Each buffer
//           moves loading -> computed -> free through three mbarriers, so
//           transforms and scattered stores overlap instead of alternating.
//
// The xpose kernel replaces "FFT along the aligned axis, then transpose" pairs
// of the reference's execute_generic / execute_2d schedules
// (src/dtfft_plan.F90:877-913, 1060-1101: fft(1) then X->Y, fft(2) then Y->Z,
// and the backward counterparts) with one HBM pass.
//
// Every mbarrier wait is bounded.  A warp that gives up records an error in
// the status word and raises a CTA-wide abort flag that ends the other
// warps' waits; the warp that issues the bulk copies waits (bounded) for its
// copies still in flight before it returns.
#pragma once

#include <cuda.h>

#include "fft_kernels.cuh"

namespace gb {

template <typename R>
struct TArgs {
    typedef typename CT<R>::T C;
    const C* in;
    C* out;
    const C* tw;          // W_M^(sign*e), e < M, for this launch's direction
    i64 nsig;             // plain: rows, row r at r*M of in and out
    const FGroup* groups; // xpose: source rank blocks
    const FSeg* segs;     //        destination segments of each block
    int ngroups;
    i64 ntiles;
    int S;                // rows per tile (power of two)
    int nst;              // ring depth (at most kTileMaxNst)
    int pair_ok;          // xpose, complex64: destinations allow 16-byte stores of two rows
    int wait_limit;       // iteration limit of the waits for a tile's bulk copy
    int* status;
    int wfast;            // xpose: consecutive tiles of a block walk w first (else u first)
};

// Ring depth limit and the shared-memory header (mbarriers, flags) in front of
// the ring: plain kernel kTileHdrPlain bytes, fused kernel kTileHdrXpose.
constexpr int kTileMaxNst = 8;
constexpr int kTileHdrPlain = 128;
constexpr int kTileHdrXpose = 256;

// exchange swizzle (stays inside aligned 16-point blocks; M % 16 == 0)
__device__ __forceinline__ int xsw(int i) { return i ^ ((i >> 4) & 15); }

// read-out swizzle of row r: conflict-free column reads of the write-out
// (lgsh = log2 of the XOR step for this S)
template <int ES>
__device__ __forceinline__ int osw(int r, int i, int lgsh) {
    if constexpr (ES == 8) return i ^ (((r >> 1) << lgsh) & 15);
    else return i ^ ((r << lgsh) & 7);
}

// Radices of a compile-time schedule: first and second stage.
template <int A, int... Rest>
struct FirstRad { static constexpr int v = A; };
template <int A, int B_, int... Rest>
struct SecondRad { static constexpr int v = B_; };

// Twiddles of the second stage of a warp-row schedule.  When the first radix
// divides the 32 threads of a row, every butterfly of a lane in that stage
// uses the same twiddles (they depend on the lane only), so a thread loads
// them once per kernel and keeps them in registers (n > 0); else n = 0 and
// the stage reads the table.
template <typename R, int E, int... Rs>
struct Tw2 {
    typedef typename CT<R>::T C;
    static constexpr int R1 = FirstRad<Rs...>::v;
    static constexpr int R2 = SecondRad<Rs..., 1>::v;
    static constexpr int M = (Rs * ... * 1);
    static constexpr int n = (sizeof...(Rs) >= 2 && E % R2 == 0 && (M / E) % R1 == 0) ? R2 : 0;
    C w[n > 0 ? n : 1];
    __device__ __forceinline__ void load(int t, const C* __restrict__ tw) {
        if constexpr (n > 0) {
            const int e1 = (M / (R1 * R2)) * (t % R1);
#pragma unroll
            for (int r = 1; r < n; ++r) w[r] = __ldg(&tw[e1 * r]);
        }
    }
};

// Twiddles of the last stage: butterfly b of lane t is j = t + 32 b and its
// twiddles are W^(j r); with at most 8 of them per thread they stay in
// registers for the whole kernel (n > 0), else the stage reads the table.
template <int A, int... Rest>
struct LastRad { static constexpr int v = LastRad<Rest...>::v; };
template <int A>
struct LastRad<A> { static constexpr int v = A; };

template <typename R, int E, int... Rs>
struct Tw3 {
    typedef typename CT<R>::T C;
    static constexpr int RL = LastRad<Rs...>::v;
    static constexpr int B = E / RL;
    static constexpr int M = (Rs * ... * 1);
    static constexpr int n = (sizeof...(Rs) >= 2 && M / E == 32 && (RL - 1) * B <= 8) ? (RL - 1) * B : 0;
    C w[n > 0 ? n : 1];
    __device__ __forceinline__ void load(int t, const C* __restrict__ tw) {
        if constexpr (n > 0) {
#pragma unroll
            for (int b = 0; b < B; ++b)
#pragma unroll
                for (int r = 1; r < RL; ++r) w[b * (RL - 1) + r - 1] = __ldg(&tw[(t + 32 * b) * r]);
        }
    }
};

template <typename R, int SG, int E, int M, int Ns, int NT2, int NT3, int RAD, int... Rest>
__device__ __forceinline__ void tile_stages(typename CT<R>::T (&v)[E], int t, const typename CT<R>::T* __restrict__ tw,
                                            typename CT<R>::T* row, const typename CT<R>::T (&tw2)[NT2],
                                            const typename CT<R>::T (&tw3)[NT3]) {
    typedef typename CT<R>::T C;
    constexpr int T = M / E;
    constexpr int B = E / RAD;
    constexpr int tstep = M / (Ns * RAD);
    constexpr bool LAST = sizeof...(Rest) == 0;
    // second stage with its twiddles in registers (see Tw2)
    constexpr bool REG_TW = (NT2 == RAD) && (Ns > 1) && (T % Ns == 0);
    constexpr bool REG_TW3 = LAST && !REG_TW && (NT3 == (RAD - 1) * B) && (Ns > 1) && (Ns * RAD == M) && (T == 32);
#pragma unroll
    for (int b = 0; b < B; ++b) {
        const int j = t + b * T;
        const int k = (T % Ns == 0) ? (t % Ns) : (j % Ns);
        C w[RAD];
#pragma unroll
        for (int r = 0; r < RAD; ++r) w[r] = v[b + r * B];
        if constexpr (Ns > 1) {
            if constexpr (REG_TW) {
#pragma unroll
                for (int r = 1; r < RAD; ++r) w[r] = cmul(w[r], tw2[r]);
            } else if constexpr (REG_TW3) {
#pragma unroll
                for (int r = 1; r < RAD; ++r) w[r] = cmul(w[r], tw3[b * (RAD - 1) + r - 1]);
            } else {
                const int e1 = tstep * k;
#pragma unroll
                for (int r = 1; r < RAD; ++r) w[r] = cmul(w[r], __ldg(&tw[e1 * r]));
            }
        }
        dft_any<R, RAD>(w, SG);
        if constexpr (LAST) {
#pragma unroll
            for (int r = 0; r < RAD; ++r) v[b + r * B] = w[r];
        } else {
            const int base = (j - k) * RAD + k;
#pragma unroll
            for (int r = 0; r < RAD; ++r) row[xsw(base + r * Ns)] = w[r];
        }
    }
    if constexpr (!LAST) {
        __syncwarp();
#pragma unroll
        for (int q = 0; q < E; ++q) v[q] = row[xsw(t + T * q)];
        __syncwarp();
        // only the second stage may take the register twiddles
        constexpr int NT2_NEXT = (Ns == 1) ? NT2 : 1;
        if constexpr (NT2_NEXT == NT2) {
            tile_stages<R, SG, E, M, Ns * RAD, NT2, NT3, Rest...>(v, t, tw, row, tw2, tw3);
        } else {
            const C none[1] = {tw2[0]};
            tile_stages<R, SG, E, M, Ns * RAD, 1, NT3, Rest...>(v, t, tw, row, none, tw3);
        }
    }
}

// Source rows of `tile`: first row, row stride, row count, group, u0, w.
template <typename R, bool XPOSE, int M>
__device__ __forceinline__ void tile_geom(const TArgs<R>& A, i64 tile, i64& row0, i64& rs, int& nrows, int& gi,
                                          int& u0, int& w) {
    if constexpr (XPOSE) {
        int lo = 0, hi = A.ngroups - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (A.groups[mid].cta_begin <= tile) lo = mid; else hi = mid - 1;
        }
        const FGroup& g = A.groups[lo];
        const int tl = (int)(tile - g.cta_begin);
        if (A.wfast) {
            u0 = (tl / g.nw) * A.S;
            w = tl % g.nw;
        } else {
            u0 = (tl % g.tiles_u) * A.S;
            w = tl / g.tiles_u;
        }
        nrows = min(A.S, g.nu - u0);
        row0 = g.src_off + (i64)u0 * g.su + (i64)w * g.sw;
        rs = g.su;
        gi = lo;
    } else {
        row0 = tile * A.S * (i64)M;
        nrows = (int)min((i64)A.S, A.nsig - tile * A.S);
        rs = M;
        gi = 0; u0 = 0; w = 0;
    }
}

template <typename R, bool XPOSE, int M>
__device__ __forceinline__ void tile_issue(const TArgs<R>& A, i64 tile, typename CT<R>::T* buf, uint64_t* bar) {
    typedef typename CT<R>::T C;
    i64 row0, rs;
    int nrows, gi, u0, w;
    tile_geom<R, XPOSE, M>(A, tile, row0, rs, nrows, gi, u0, w);
    constexpr uint32_t row_bytes = (uint32_t)(M * sizeof(C));
    mbar_expect_tx(bar, row_bytes * (uint32_t)nrows);
    if (rs == M) {
        bulk_load(buf, A.in + row0, row_bytes * (uint32_t)nrows, bar);
    } else {
        for (int r = 0; r < nrows; ++r) bulk_load(buf + r * M, A.in + row0 + (i64)r * rs, row_bytes, bar);
    }
}

// Load one row from its slot, transform it, and leave the spectrum in
// registers (v[q] = point lane + 32*q).
template <typename R, int SG, int E, int... Rs>
__device__ __forceinline__ void tile_row_fft(typename CT<R>::T (&v)[E], typename CT<R>::T* row, int lane,
                                             const typename CT<R>::T* tw, const Tw2<R, E, Rs...>& t2,
                                             const Tw3<R, E, Rs...>& t3) {
    constexpr int M = (Rs * ... * 1);
    constexpr int NT2 = Tw2<R, E, Rs...>::n > 0 ? Tw2<R, E, Rs...>::n : 1;
    constexpr int NT3 = Tw3<R, E, Rs...>::n > 0 ? Tw3<R, E, Rs...>::n : 1;
#pragma unroll
    for (int q = 0; q < E; ++q) v[q] = row[lane + 32 * q];
    __syncwarp();
    tile_stages<R, SG, E, M, 1, NT2, NT3, Rs...>(v, lane, tw, row, t2.w, t3.w);
}

// ---------------------------------------------------------------------------
// Plain rows
// ---------------------------------------------------------------------------
template <typename R, int SG, int NW, int E, int... Rs>
__global__ void __launch_bounds__(32 * NW, 1) fft_tile_kernel(TArgs<R> A) {
    typedef typename CT<R>::T C;
    constexpr int M = (Rs * ... * 1);
    static_assert(M == E * 32, "one warp per row");
    static_assert(M % 16 == 0, "swizzles need 16-point blocks");
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw);
    C* ring = reinterpret_cast<C*>(smem_raw + kTileHdrPlain);
    const int S = A.S, NST = A.nst;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, W = blockDim.x >> 5;
    Tw2<R, E, Rs...> t2;
    t2.load(lane, A.tw);
    Tw3<R, E, Rs...> t3;
    t3.load(lane, A.tw);

    if (threadIdx.x == 0) {
        for (int b = 0; b < NST; ++b) mbar_init(&bars[b], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int j = 0; j < NST; ++j) {
            const i64 tj = blockIdx.x + (i64)j * gridDim.x;
            if (tj < A.ntiles) tile_issue<R, false, M>(A, tj, ring + (i64)j * S * M, &bars[j]);
        }
    }
    int b = 0;
    uint32_t par = 0;
    for (i64 tile = blockIdx.x; tile < A.ntiles; tile += gridDim.x) {
        const bool ok = mbar_wait_limit(&bars[b], par, A.wait_limit);
        if (__syncthreads_or(!ok)) {
            if (threadIdx.x == 0) {
                report_status(A.status, 1);
                int bb = b;
                uint32_t pp = par;
                for (int j = 0; j < NST; ++j) {
                    const i64 tj = tile + (i64)j * gridDim.x;
                    if (tj >= A.ntiles) break;
                    mbar_wait_bounded(&bars[bb], pp);
                    if (++bb == NST) { bb = 0; pp ^= 1; }
                }
            }
            __syncthreads();
            return;
        }
        i64 row0, rs;
        int nrows, gi, u0, w;
        tile_geom<R, false, M>(A, tile, row0, rs, nrows, gi, u0, w);
        C* tb = ring + (i64)b * S * M;
        for (int rl = warp; rl < nrows; rl += W) {
            C v[E];
            tile_row_fft<R, SG, E, Rs...>(v, tb + rl * M, lane, A.tw, t2, t3);
            C* dst = A.out + row0 + (i64)rl * M;
#pragma unroll
            for (int q = 0; q < E; ++q) dst[lane + 32 * q] = v[q];
        }
        // buffer b is consumed: hand it back to the bulk-copy engine
        fence_async_smem();
        __syncthreads();
        if (threadIdx.x == 0) {
            const i64 tn = tile + (i64)NST * gridDim.x;
            if (tn < A.ntiles) tile_issue<R, false, M>(A, tn, tb, &bars[b]);
        }
        if (++b == NST) { b = 0; par ^= 1; }
    }
}

// ---------------------------------------------------------------------------
// Rows fused with the transpose (warp-specialised)
// ---------------------------------------------------------------------------
// bounded mbarrier wait that also ends when the CTA aborts
__device__ __forceinline__ bool mbar_wait_or_abort(uint64_t* bar, uint32_t parity, volatile int* abort_flag,
                                                   int limit = kWaitLimitDefault) {
    for (int it = 0; it < limit; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 255) == 255 && *abort_flag) return false;
    }
    return false;
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

template <typename R, int SG, int NCW, int NSW, int E, int... Rs>
__global__ void __launch_bounds__(32 * (NCW + NSW), 1) fft_tile_xpose_kernel(TArgs<R> A) {
    typedef typename CT<R>::T C;
    constexpr int M = (Rs * ... * 1);
    static_assert(M == E * 32, "one warp per row");
    static_assert(M % 16 == 0, "swizzles need 16-point blocks");
    constexpr int ES = (int)sizeof(C);
    extern __shared__ __align__(128) unsigned char smem_raw[];
    // full[b]: the bulk copy into buffer b landed; done[b]: the NCW compute warps
    // wrote its spectra; empty[b]: the NSW store warps have read it
    uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw);
    uint64_t* done = full + kTileMaxNst;
    uint64_t* empty = full + 2 * kTileMaxNst;
    volatile int* abort_flag = reinterpret_cast<volatile int*>(smem_raw + 24 * kTileMaxNst);
    C* ring = reinterpret_cast<C*>(smem_raw + kTileHdrXpose);
    const int S = A.S, NST = A.nst;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int lgS = __ffs(S) - 1;
    const int lgNP = ES == 8 ? lgS - 1 : lgS;                 // log2 lanes per point of the read-out
    const int lgsh = ES == 8 ? (4 - lgNP) : (3 - lgNP);       // read-out XOR step

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
        // ---- compute warps ----
        Tw2<R, E, Rs...> t2;
        t2.load(lane, A.tw);
        Tw3<R, E, Rs...> t3;
        t3.load(lane, A.tw);
        int b = 0;
        uint32_t par = 0;
        for (i64 tile = blockIdx.x; tile < A.ntiles; tile += gridDim.x) {
            if (!mbar_wait_or_abort(&full[b], par, abort_flag, A.wait_limit)) {
                if (lane == 0) { report_status(A.status, 1); *abort_flag = 1; }
                return;
            }
            i64 row0, rs;
            int nrows, gi, u0, w;
            tile_geom<R, true, M>(A, tile, row0, rs, nrows, gi, u0, w);
            C* tb = ring + (i64)b * S * M;
            for (int rl = warp; rl < nrows; rl += NCW) {
                C* row = tb + rl * M;
                C v[E];
                tile_row_fft<R, SG, E, Rs...>(v, row, lane, A.tw, t2, t3);
                __syncwarp();
#pragma unroll
                for (int q = 0; q < E; ++q) row[osw<ES>(rl, lane + 32 * q, lgsh)] = v[q];
            }
            // a bulk copy rewrites the slot after the store warps: order these writes first
            fence_async_smem();
            __syncwarp();
            if (lane == 0) mbar_arrive(&done[b]);
            if (++b == NST) { b = 0; par ^= 1; }
        }
        return;
    }

    // ---- store warps; the first one also issues the bulk copies ----
    const int st = threadIdx.x - NCW * 32;             // 0 .. 32*NSW-1
    const bool producer = warp == NCW;
    uint32_t issued_par = 0;                            // bit b: parity of the last copy into buffer b
    if (producer && lane == 0) {
        for (int j = 0; j < NST; ++j) {
            const i64 tj = blockIdx.x + (i64)j * gridDim.x;
            if (tj < A.ntiles) tile_issue<R, true, M>(A, tj, ring + (i64)j * S * M, &full[j]);
        }
    }
    const int lp = st & ((1 << lgNP) - 1);             // row pair (complex64) / row (complex128)
    const int g0 = st >> lgNP;                          // first point of this thread
    const int gstep = (32 * NSW) >> lgNP;
    int b = 0;
    uint32_t par = 0;
    bool failed = false;
    for (i64 tile = blockIdx.x; tile < A.ntiles; tile += gridDim.x) {
        if (!mbar_wait_or_abort(&done[b], par, abort_flag)) { failed = true; break; }
        i64 row0, rs;
        int nrows, gi, u0, w;
        tile_geom<R, true, M>(A, tile, row0, rs, nrows, gi, u0, w);
        const C* tb = ring + (i64)b * S * M;
        const FGroup& g = A.groups[gi];
        for (int kk = 0; kk < g.nseg; ++kk) {
            const FSeg sg = A.segs[g.seg_first + kk];
            const int npts = sg.i1 - sg.i0;
            C* dbase = A.out + sg.dst_off + (i64)w * sg.dw + u0;
            if constexpr (ES == 8) {
                const int r0 = 2 * lp;
                if (r0 < nrows) {
                    const bool two = r0 + 1 < nrows;
                    const C* s0 = tb + r0 * M;
                    const C* s1 = s0 + M;
#pragma unroll 4
                    for (int ii = g0; ii < npts; ii += gstep) {
                        const int i = sg.i0 + ii;
                        const C a = s0[osw<ES>(r0, i, lgsh)];
                        C* d = dbase + (i64)ii * sg.di + r0;
                        if (two) {
                            const C c = s1[osw<ES>(r0 + 1, i, lgsh)];
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
                if (r0 < nrows) {
                    const C* s0 = tb + r0 * M;
                    for (int ii = g0; ii < npts; ii += gstep) {
                        const int i = sg.i0 + ii;
                        dbase[(i64)ii * sg.di + r0] = s0[osw<ES>(r0, i, lgsh)];
                    }
                }
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[b]);
        if (producer) {
            // every store warp has read buffer b: refill it
            if (!mbar_wait_or_abort(&empty[b], par, abort_flag)) { failed = true; break; }
            if (lane == 0) {
                const i64 tn = tile + (i64)NST * gridDim.x;
                if (tn < A.ntiles) {
                    tile_issue<R, true, M>(A, tn, const_cast<C*>(tb), &full[b]);
                    issued_par = (issued_par & ~(1u << b)) | ((par ^ 1u) << b);
                }
            }
            __syncwarp();
        }
        if (++b == NST) { b = 0; par ^= 1; }
    }
    if (failed) {
        if (lane == 0) { report_status(A.status, 1); *abort_flag = 1; }
        if (producer && lane == 0) {
            // wait (bounded) for the last copy issued into every buffer; a copy
            // that already landed completes its wait at once
            for (int j = 0; j < NST && blockIdx.x + (i64)j * gridDim.x < A.ntiles; ++j)
                mbar_wait_bounded(&full[j], (issued_par >> j) & 1u);
        }
    }
}

// ---------------------------------------------------------------------------
// Rows fused with the transpose, written out by TMA tensor stores
// ---------------------------------------------------------------------------
// The same pass as fft_tile_xpose_kernel with the write-out moved off the SMs:
//  - each compute warp transforms a pair of adjacent rows (u, u + 1) of the
//    tile, keeping both spectra in registers;
//  - after a barrier of the compute warps (every row of the tile has been read
//    and its exchanges are done) the warps write the tile back into its own
//    buffer transposed, [point i][row u] with u fastest: one 128-byte line per
//    point (S rows of 8 or 16 bytes), 16-byte stores of the row pair,
//    128-byte swizzled (16-byte chunk c of line i at chunk c ^ (i mod 8));
//  - one producer warp issues the bulk loads, and per destination segment
//    the cp.async.bulk.tensor stores of the transposed lines (boxes of
//    S rows x up to 256 points, the tensor map un-swizzles them), then reuses
//    the buffer for the next load once the store has read it.  The boxes'
//    extent along the points (256, 128, 64 or 32) is a launch parameter that
//    the autotuner chooses.
// No thread of the SM executes a global store; each point leaves as part of a
// 128-byte line of the destination rank's block.
constexpr int kTmaXMaxSegs = 48;
constexpr int kTileHdrXTma = 1024;   // header; the launch adds another 1 KB of alignment slack

constexpr int kTmaXMaxGroups = 16;
struct TmaXMaps {
    CUtensorMap map[kTmaXMaxSegs];   // per destination segment: (u words, i, w) of its block
    // per source group whose rows are not adjacent: (row words in 256-word
    // runs, run, u, w), one box = a whole tile of S rows; unused when `loads`
    // is 0 (every tile is then one contiguous bulk copy or per-row copies)
    CUtensorMap lmap[kTmaXMaxGroups];
    int loads;
};

template <typename R>
struct TXArgs {
    TArgs<R> a;
    int box_i;        // points per tensor store (the maps' box extent along i)
    TmaXMaps m;
};

__device__ __forceinline__ bool bar_red_or(int id, int nthreads, bool v) {
    uint32_t r;
    asm volatile(
        "{\n .reg .pred p, q;\n setp.ne.u32 q, %1, 0;\n bar.red.or.pred p, %2, %3, q;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(id), "r"(nthreads)
        : "memory");
    return r != 0;
}
__device__ __forceinline__ void bar_sync_n(int id, int nthreads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}
__device__ __forceinline__ void tma_load_4d(const CUtensorMap* map, void* smem, int c2, int c3, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(smem)),
        "l"(map), "r"(0), "r"(0), "r"(c2), "r"(c3), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void tma_store_3d(const CUtensorMap* map, const void* smem, int c0, int c1, int c2) {
    asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%2, %3, %4}], [%1];" ::"l"(map),
                 "r"(smem_u32(smem)), "r"(c0), "r"(c1), "r"(c2)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// Byte offset, inside a point's line of LB bytes, of the 16-byte chunk `chunk`
// under the tensor map's swizzle: 128-byte lines (SWIZZLE_128B) XOR the chunk
// index with i mod 8, 64-byte lines (SWIZZLE_64B) with (i / 2) mod 4 - the
// byte-address bits 7..9 (7..8) of line i in a 1024-byte aligned buffer.
template <int LB>
__device__ __forceinline__ int line_chunk(int i, int chunk) {
    if constexpr (LB == 128) return (chunk ^ (i & 7)) << 4;
    else return (chunk ^ ((i >> 1) & 3)) << 4;
}

template <typename R, int SG, int NCW, int RPW, int E, int... Rs>
__global__ void __launch_bounds__(32 * (NCW + 1), 1) fft_tile_xpose_tma_kernel(const __grid_constant__ TXArgs<R> X) {
    typedef typename CT<R>::T C;
    constexpr int M = (Rs * ... * 1);
    constexpr int ES = (int)sizeof(C);
    constexpr int S = NCW * RPW;                // rows per tile
    constexpr int LB = S * ES;                  // bytes of one point's line
    static_assert(M == E * 32, "one warp per row");
    static_assert(M % 16 == 0, "swizzles need 16-point blocks");
    static_assert(RPW == 1 || RPW == 2, "one row or a row pair per compute warp");
    static_assert(LB == 64 || LB == 128, "lines of 64 or 128 bytes");
    const TArgs<R>& A = X.a;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // full[b]: the load into buffer b landed; done[b]: the compute warps wrote
    // buffer b back transposed
    // the swizzle pattern of the staged lines is anchored at 1024-byte
    // boundaries: align the start of the header (the launch adds 1 KB of slack)
    unsigned char* base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    uint64_t* full = reinterpret_cast<uint64_t*>(base);
    uint64_t* done = full + kTileMaxNst;
    volatile int* abort_flag = reinterpret_cast<volatile int*>(base + 16 * kTileMaxNst);
    unsigned char* ring = base + kTileHdrXTma;              // 1024-byte aligned buffers of M lines
    const int NST = A.nst;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

    if (threadIdx.x == 0) {
        for (int b = 0; b < NST; ++b) {
            mbar_init(&full[b], 1);
            mbar_init(&done[b], NCW);
        }
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    if (warp < NCW) {
        // ---- compute warps: rows RPW*warp .. RPW*warp + RPW - 1 of every tile ----
        Tw2<R, E, Rs...> t2;
        t2.load(lane, A.tw);
        Tw3<R, E, Rs...> t3;
        t3.load(lane, A.tw);
        const int ua = RPW * warp;
        int b = 0;
        uint32_t par = 0;
        for (i64 tile = blockIdx.x; tile < A.ntiles; tile += gridDim.x) {
            const bool ok = mbar_wait_or_abort(&full[b], par, abort_flag, A.wait_limit);
            if (bar_red_or(1, 32 * NCW, !ok)) {
                if (threadIdx.x == 0) { report_status(A.status, 1); *abort_flag = 1; }
                return;
            }
            i64 row0, rs;
            int nrows, gi, u0, w;
            tile_geom<R, true, M>(A, tile, row0, rs, nrows, gi, u0, w);
            C* tb = reinterpret_cast<C*>(ring + (size_t)b * M * LB);
            C va[E], vb[RPW == 2 ? E : 1];
            if (ua < nrows) tile_row_fft<R, SG, E, Rs...>(va, tb + ua * M, lane, A.tw, t2, t3);
            if constexpr (RPW == 2)
                if (ua + 1 < nrows) tile_row_fft<R, SG, E, Rs...>(vb, tb + (ua + 1) * M, lane, A.tw, t2, t3);
            // every row of the tile has been read: the buffer takes the transposed lines
            bar_sync_n(2, 32 * NCW);
            unsigned char* lines = reinterpret_cast<unsigned char*>(tb);
#pragma unroll
            for (int q = 0; q < E; ++q) {
                const int i = lane + 32 * q;
                unsigned char* line = lines + (size_t)i * LB;
                if constexpr (ES == 8 && RPW == 2) {
                    // rows ua, ua + 1 share the 16-byte chunk `warp`
                    float4 v;
                    v.x = va[q].x; v.y = va[q].y; v.z = vb[q].x; v.w = vb[q].y;
                    *reinterpret_cast<float4*>(line + line_chunk<LB>(i, warp)) = v;
                } else if constexpr (ES == 8) {
                    // row ua is half of the 16-byte chunk ua / 2
                    *reinterpret_cast<C*>(line + line_chunk<LB>(i, ua >> 1) + 8 * (ua & 1)) = va[q];
                } else {
                    // one 16-byte chunk per row
                    *reinterpret_cast<C*>(line + line_chunk<LB>(i, ua)) = va[q];
                    if constexpr (RPW == 2) *reinterpret_cast<C*>(line + line_chunk<LB>(i, ua + 1)) = vb[q];
                }
            }
            // the tensor stores read the buffer through the async proxy
            fence_async_smem();
            __syncwarp();
            if (lane == 0) mbar_arrive(&done[b]);
            if (++b == NST) { b = 0; par ^= 1; }
        }
        return;
    }

    // ---- producer warp: bulk loads in, tensor stores out ----
    if (lane != 0) return;
    // strided source rows: one tensor load of the whole tile (its box always
    // fills S rows; rows past the block's end read as zeros), else bulk copies
    auto issue = [&](i64 tj, int bj) {
        C* buf = reinterpret_cast<C*>(ring + (size_t)bj * M * LB);
        if (X.m.loads) {
            i64 row0, rs;
            int nrows, gi, u0, w;
            tile_geom<R, true, M>(A, tj, row0, rs, nrows, gi, u0, w);
            if (rs != M) {
                mbar_expect_tx(&full[bj], (uint32_t)(M * sizeof(C)) * (uint32_t)S);
                tma_load_4d(&X.m.lmap[gi], buf, u0, w, &full[bj]);
                return;
            }
        }
        tile_issue<R, true, M>(A, tj, buf, &full[bj]);
    };
    uint32_t issued_par = 0;   // bit b: parity of the last load into buffer b
    for (int j = 0; j < NST; ++j) {
        const i64 tj = blockIdx.x + (i64)j * gridDim.x;
        if (tj < A.ntiles) issue(tj, j);
    }
    int b = 0;
    uint32_t par = 0;
    bool failed = false;
    for (i64 tile = blockIdx.x; tile < A.ntiles; tile += gridDim.x) {
        if (!mbar_wait_or_abort(&done[b], par, abort_flag)) { failed = true; break; }
        i64 row0, rs;
        int nrows, gi, u0, w;
        tile_geom<R, true, M>(A, tile, row0, rs, nrows, gi, u0, w);
        const unsigned char* tb = ring + (size_t)b * M * LB;
        const FGroup& g = A.groups[gi];
        for (int kk = 0; kk < g.nseg; ++kk) {
            const FSeg sg = A.segs[g.seg_first + kk];
            const CUtensorMap* map = &X.m.map[g.seg_first + kk];
            for (int i = sg.i0; i < sg.i1; i += X.box_i)
                tma_store_3d(map, tb + (size_t)i * LB, u0 * (ES / 8), i - sg.i0, w);
        }
        bulk_commit();
        // the store has read the buffer: refill it
        bulk_wait_read_all();
        const i64 tn = tile + (i64)NST * gridDim.x;
        if (tn < A.ntiles) {
            issue(tn, b);
            issued_par = (issued_par & ~(1u << b)) | ((par ^ 1u) << b);
        }
        if (++b == NST) { b = 0; par ^= 1; }
    }
    if (failed) {
        report_status(A.status, 1);
        *abort_flag = 1;
        // wait (bounded) for the last load issued into every buffer
        for (int j = 0; j < NST && blockIdx.x + (i64)j * gridDim.x < A.ntiles; ++j)
            mbar_wait_bounded(&full[j], (issued_par >> j) & 1u);
    }
    bulk_wait_all();
}

// Tile-kernel entry points of one precision (fft_tile_f32.cu / fft_tile_f64.cu):
// nullptr when no variant is compiled for M.
template <typename R>
struct TilePtr {
    // kernel for rows of M points; ncw/nsw select a compiled warp split
    // (plain: ncw = warps), 0 the default
    static void* get(int M, int sign, bool xpose, int ncw = 0, int nsw = 0);
    static int points_per_thread(int M);   // E of the compiled variants, 0 if none
    static int default_threads(int M, bool xpose);
    // fused kernel with tensor-store write-out (fft_tile_xpose_tma_kernel), nullptr if none for M;
    // *rows: rows per tile (one line of rows * sizeof(complex) bytes per point), *warps: compute warps
    static void* get_tma(int M, int sign, int* rows = nullptr, int* warps = nullptr);
};

}  // namespace gb
