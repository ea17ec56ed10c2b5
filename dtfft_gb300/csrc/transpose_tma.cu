// Box-list transpose with TMA tensor loads (4-, 8- and 16-byte elements).
//
// Each box of a virtual-grid transpose, src[src_off + a + b*sb + c*sc] ->
// dst[dst_off + b + a*da + c*dc], is described by a 3D tensor map over
// (a, b, c).  A CTA owns one 128 x 32 (4-byte), 64 x 32 (8-byte) or 32 x 32 (16-byte) (a, b)
// tile of one c-plane: one thread issues four cp.async.bulk.tensor loads of
// 128-byte-wide boxes, which land in shared memory with the 128-byte swizzle
// (16-byte chunk index XOR row index mod 8) and complete on an mbarrier.  The
// warps then read the tile along a with 16-byte loads - the swizzle makes the
// eight lanes of each load phase hit distinct banks - and write destination
// rows of 32 consecutive b values (256 or 512 contiguous bytes per warp
// store).  Loads past a box edge are zero-filled by the TMA unit and never
// stored.  The mbarrier wait is bounded (status word on timeout).
//
// The tensor maps depend on the input pointer, so they are encoded on the
// host when a pointer is first seen (a pure host computation, also legal
// while a stream is being captured) and passed by value as a kernel
// parameter.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstring>
#include <mutex>

#include "common.cuh"

namespace gb {

constexpr int kTmaMaxBoxes = 64;

struct TmaParams {
    CUtensorMap maps[kTmaMaxBoxes];
    const Box* boxes;
    int nboxes;
    int wait_limit;
    int* status;
};

__device__ __forceinline__ uint32_t tma_smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// bounded wait for phase 0 of the tile's mbarrier
__device__ __forceinline__ bool tma_wait(uint64_t* bar, int limit) {
    for (int it = 0; it < limit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(tma_smem_u32(bar))
            : "memory");
        if (done) return true;
    }
    return false;
}

template <int ES>
__global__ void __launch_bounds__(256) box_transpose_tma_kernel(const __grid_constant__ TmaParams P, char* out) {
    constexpr int IN = 128 / ES;          // elements of one 128-byte swizzle row
    constexpr int TA = 4 * IN;            // tile extent along a (four TMA boxes)
    constexpr int TB = 32;
    __shared__ __align__(1024) unsigned char tile[4 * TB * 128];
    __shared__ __align__(8) uint64_t bar;
    const i64 t = (i64)blockIdx.x;
    int lo = 0, hi = P.nboxes - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (P.boxes[mid].tile_begin <= t) lo = mid; else hi = mid - 1;
    }
    const Box& bx = P.boxes[lo];
    const int tiles_a = bx.tiles_a;
    const int per_c = tiles_a * bx.tiles_b;
    const i64 lt = t - bx.tile_begin;
    const int c = (int)(lt / per_c);
    const int r = (int)(lt - (i64)c * per_c);
    const int a0 = (r % tiles_a) * TA;
    const int b0 = (r / tiles_a) * TB;
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tma_smem_u32(&bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tma_smem_u32(&bar)),
                     "r"((uint32_t)(4 * TB * 128))
                     : "memory");
        const CUtensorMap* map = &P.maps[lo];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            // the map counts a in 8-byte words (4-byte elements: in elements):
            // x = element index * (ES / 8), always even (a multiple of 32 for 4 bytes)
            asm volatile(
                "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(tma_smem_u32(tile + k * TB * 128)),
                "l"(map), "r"(ES >= 8 ? (a0 + k * IN) * (ES / 8) : (a0 + k * IN)), "r"(b0), "r"(c),
                "r"(tma_smem_u32(&bar))
                : "memory");
        }
    }
    __syncthreads();
    bool ok = tma_wait(&bar, P.wait_limit);
    if (__syncthreads_or(!ok)) {
        // give up: record it, and let the loads still in flight land (bounded)
        // before the CTA's shared memory is released
        if (threadIdx.x == 0) {
            report_status(P.status, 3);
            tma_wait(&bar, kWaitLimitDefault);
        }
        __syncthreads();
        return;
    }
    const int ra = min(TA, bx.na - a0), rb = min(TB, bx.nb - b0);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int b = lane;
    if (b >= rb) return;
    char* dst = out + (bx.dst_off + (i64)c * bx.dc + b0 + b) * ES;
    const i64 da = bx.da_or_db * ES;
    if constexpr (ES == 4) {
        // thread: row b, the 16-byte chunk holding a .. a + 3
        for (int aq = warp; aq < TA / 4; aq += 8) {
            const int a = 4 * aq;
            if (a >= ra) break;
            const int k = a / IN, ai = a % IN;
            const int chunk = ((ai * ES) >> 4) ^ (b & 7);
            const uint4 v = *reinterpret_cast<const uint4*>(tile + k * TB * 128 + b * 128 + chunk * 16);
            const uint32_t w4[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (a + j < ra) *reinterpret_cast<uint32_t*>(dst + (i64)(a0 + a + j) * da) = w4[j];
        }
    } else if constexpr (ES == 8) {
        // thread: row b, the 16-byte chunk holding a and a + 1
        for (int ap = warp; ap < TA / 2; ap += 8) {
            const int a = 2 * ap;
            if (a >= ra) break;
            const int k = a / IN, ai = a % IN;
            const int chunk = ((ai * ES) >> 4) ^ (b & 7);
            const uint4 v = *reinterpret_cast<const uint4*>(tile + k * TB * 128 + b * 128 + chunk * 16);
            *reinterpret_cast<uint2*>(dst + (i64)(a0 + a) * da) = make_uint2(v.x, v.y);
            if (a + 1 < ra) *reinterpret_cast<uint2*>(dst + (i64)(a0 + a + 1) * da) = make_uint2(v.z, v.w);
        }
    } else {
        for (int a = warp; a < TA; a += 8) {
            if (a >= ra) break;
            const int k = a / IN, ai = a % IN;
            const int chunk = ai ^ (b & 7);
            const uint4 v = *reinterpret_cast<const uint4*>(tile + k * TB * 128 + b * 128 + chunk * 16);
            *reinterpret_cast<uint4*>(dst + (i64)(a0 + a) * da) = v;
        }
    }
}

// ---------------------------------------------------------------------------
// host
// ---------------------------------------------------------------------------
static PFN_cuTensorMapEncodeTiled_v12000 g_encode_fn = nullptr;
static std::once_flag g_encode_once;

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    std::call_once(g_encode_once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_encode_fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
        cudaGetLastError();
    });
    return g_encode_fn;
}

void* tma_encode_tiled_fn() { return (void*)encode_fn(); }

// Boxes of this list fit the TMA kernel: 8- or 16-byte elements, at most
// kTmaMaxBoxes boxes, every box start and source stride 16-byte aligned.
bool tma_eligible(const BoxList& bl) {
    if (bl.copy || (bl.elem != 4 && bl.elem != 8 && bl.elem != 16) || bl.host.empty() ||
        (int)bl.host.size() > kTmaMaxBoxes)
        return false;
    if (getenv("DTFFT_GB_NO_TMA")) return false;
    for (const Box& x : bl.host)
        if ((x.src_off * bl.elem) % 16 || (x.sb * bl.elem) % 16 || (x.sc * bl.elem) % 16 || x.nb < 1 || x.na < 1)
            return false;
    return encode_fn() != nullptr;
}

// tile extents of the TMA kernel (a x b)
int tma_tile_a(int elem) { return 4 * (128 / elem); }

// The default tile of a list: the TMA kernel's extents for 4-byte elements when
// the list fits it (8- and 16-byte defaults already are the TMA extents).
void tma_default_tile(BoxList& bl) {
    if (bl.elem == 4 && tma_eligible(bl)) {
        bl.cfg.tile_a = tma_tile_a(4);
        bl.cfg.tile_b = 32;
        bl.cfg.rows = 8;
    }
}

static std::mutex g_tma_mu;

// Box list of the TMA kernel: tiles per box of (tile_a x 32) and the maps for
// input pointer `in` (cached, a few pointers per list).
dtfft_error_t tma_launch(const BoxList& bl, const void* in, void* out, cudaStream_t s, int* status,
                         std::vector<std::pair<const void*, void*>>& cache) {
    // the launch takes a copy made under the lock: another thread may evict
    // the cached entry as soon as the lock is released
    if (!status) return DTFFT_ERROR_GPU_CALL_FAILED;
    TmaParams L;
    {
        TmaParams* P = nullptr;
        std::lock_guard<std::mutex> lk(g_tma_mu);
        for (auto& e : cache)
            if (e.first == in) P = (TmaParams*)e.second;
        if (!P) {
            P = new TmaParams();
            memset(P, 0, sizeof(TmaParams));
            const int es = bl.elem;
            // 8-byte words (16-byte elements are two words along a); 4-byte elements as themselves
            const CUtensorMapDataType dt = es == 4 ? CU_TENSOR_MAP_DATA_TYPE_UINT32 : CU_TENSOR_MAP_DATA_TYPE_UINT64;
            for (size_t i = 0; i < bl.host.size(); ++i) {
                const Box& x = bl.host[i];
                const cuuint64_t na = es == 4 ? (cuuint64_t)x.na : (cuuint64_t)x.na * (es / 8);
                cuuint64_t gdim[3] = {na, (cuuint64_t)x.nb, (cuuint64_t)x.nc};
                cuuint64_t gstr[2] = {(cuuint64_t)(x.sb * es), (cuuint64_t)(x.sc * es)};
                cuuint32_t box[3] = {es == 4 ? 32u : 16u, 32, 1};
                cuuint32_t estr[3] = {1, 1, 1};
                void* base = (char*)in + x.src_off * es;
                CUresult r = encode_fn()(&P->maps[i], dt, 3, base, gdim, gstr, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                         CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
                if (r != CUDA_SUCCESS) { delete P; return DTFFT_ERROR_GPU_CALL_FAILED; }
            }
            P->nboxes = (int)bl.host.size();
            if (cache.size() >= 4) { delete (TmaParams*)cache.front().second; cache.erase(cache.begin()); }
            cache.emplace_back(in, P);
        }
        memcpy(&L, P, sizeof(TmaParams));
    }
    L.status = status;
    L.wait_limit = g_wait_limit;
    L.boxes = bl.dev;   // re-read: an autotune re-upload may have moved the list
    if (bl.total_tiles == 0) return DTFFT_SUCCESS;
    if (bl.elem == 4) box_transpose_tma_kernel<4><<<(unsigned)bl.total_tiles, 256, 0, s>>>(L, (char*)out);
    else if (bl.elem == 8) box_transpose_tma_kernel<8><<<(unsigned)bl.total_tiles, 256, 0, s>>>(L, (char*)out);
    else box_transpose_tma_kernel<16><<<(unsigned)bl.total_tiles, 256, 0, s>>>(L, (char*)out);
    return DTFFT_SUCCESS;
}

void tma_cache_free(std::vector<std::pair<const void*, void*>>& cache) {
    std::lock_guard<std::mutex> lk(g_tma_mu);
    for (auto& e : cache) delete (TmaParams*)e.second;
    cache.clear();
}

}  // namespace gb
