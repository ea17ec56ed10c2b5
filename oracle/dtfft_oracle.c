/*
 * dtfft_oracle.c -- CPU restatement of dtFFT's data-movement path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle of the parity tests of the GPU library in
 * dtfft_gb300/: only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it.  Nothing in the product links or calls it.
 *
 * What is restated (reference paths are relative to the dtFFT project root):
 *   - local start/count rule of a pencil ........ src/dtfft_pencil.F90:237-279
 *   - pencil dims/comm permutations ............. src/dtfft_transpose_plan.F90:1045-1131
 *   - host permute/pack/unpack kernels .......... src/include/_dtfft_kernel_host_routines.inc:140-752
 *   - generic reshape handle for transposes
 *     (send/recv boxes, neighbour data, kernel
 *     choice, pack -> all-to-all-v -> unpack) ... src/dtfft_reshape_handle_generic.F90:174-759
 *   - communicator chosen per transpose ......... src/dtfft_abstract_reshape_handle.F90:141-204
 *
 * The P0 x P1 x P2 grid (P0 == 1) is simulated rank by rank: every virtual
 * rank owns its own buffers, the exchange is an explicit all-to-all-v between
 * the ranks of one sub-communicator, exactly as the reference's MPI run would
 * do it on a single host.  Buffers handed to the driver functions are the
 * ranks' local blocks packed one after the other in cartesian rank order
 * (rank = c1 * P2 + c2, row-major as MPI numbers cartesian ranks).
 *
 * Element size is a parameter (4, 8 or 16 bytes): every routine only moves
 * elements, so one byte-generic implementation serves all dtypes.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef int64_t i64;

/* ------------------------------------------------------------------ */
/* Element copy helpers                                                */
/* ------------------------------------------------------------------ */
static inline void cp_el(char* out, i64 oidx, const char* in, i64 iidx, int es) {
    switch (es) {
    case 4: ((uint32_t*)out)[oidx] = ((const uint32_t*)in)[iidx]; break;
    case 8: ((uint64_t*)out)[oidx] = ((const uint64_t*)in)[iidx]; break;
    default: memcpy(out + oidx * es, in + iidx * es, (size_t)es); break;
    }
}

/* ------------------------------------------------------------------ */
/* Pencil rule: src/dtfft_pencil.F90:237-279 (get_local_size).         */
/* The remainder n % P goes to the LAST ranks.                          */
/* ------------------------------------------------------------------ */
void orc_local_size(int n_global, int comm_size, int comm_rank, int* start, int* count) {
    if (comm_size == 1) { *start = 0; *count = n_global; return; }
    int res = n_global % comm_size;
    int base = n_global / comm_size;
    int s = 0;
    for (int i = 0; i < comm_rank; ++i) s += base + (i >= comm_size - res ? 1 : 0);
    *start = s;
    *count = base + (comm_rank >= comm_size - res ? 1 : 0);
}

/* Pencil `layout` (1 = X, 2 = Y, 3 = Z aligned) of cartesian rank `rank`
 * in a grid (1, g1, g2) for ndims == 3 or (1, g1) for ndims == 2.
 * Data permutations dperm and communicator permutations cperm follow
 * src/dtfft_transpose_plan.F90:1045-1082; counts are returned in the
 * pencil's own (aligned-first) order. */
void orc_pencil(int ndims, const int* gdims, const int* grid, int layout, int rank,
                int* starts, int* counts) {
    /* cartesian coordinates of `rank` (row-major over (1, g1, g2)) */
    int c[3] = {0, 0, 0};
    if (ndims == 3) { c[1] = rank / grid[2]; c[2] = rank % grid[2]; }
    else            { c[1] = rank; }
    int dperm[3], cperm[3];
    if (ndims == 2) {
        if (layout == 1) { dperm[0] = 0; dperm[1] = 1; }
        else             { dperm[0] = 1; dperm[1] = 0; }
        cperm[0] = 0; cperm[1] = 1;
    } else {
        if (layout == 1)      { dperm[0] = 0; dperm[1] = 1; dperm[2] = 2; cperm[0] = 0; cperm[1] = 1; cperm[2] = 2; }
        else if (layout == 2) { dperm[0] = 1; dperm[1] = 2; dperm[2] = 0; cperm[0] = 0; cperm[1] = 2; cperm[2] = 1; }
        else                  { dperm[0] = 2; dperm[1] = 0; dperm[2] = 1; cperm[0] = 0; cperm[1] = 1; cperm[2] = 2; }
    }
    for (int d = 0; d < ndims; ++d) {
        int comm = cperm[d];
        orc_local_size(gdims[dperm[d]], grid[comm], c[comm], &starts[d], &counts[d]);
    }
}

/* ------------------------------------------------------------------ */
/* Host kernels: src/include/_dtfft_kernel_host_routines.inc            */
/* (write-access variants; `dims` are the kernel's local dims)          */
/* ------------------------------------------------------------------ */

/* :140-196  (nx,ny,nz) -> (ny,nz,nx); 2D: (nx,ny) -> (ny,nx) */
void orc_permute_forward(const void* vin, void* vout, int ndims, const int* dims, int es) {
    const char* in = (const char*)vin; char* out = (char*)vout;
    i64 nx = dims[0], ny = dims[1];
    if (ndims == 2) {
        #pragma omp parallel for schedule(static)
        for (i64 x = 0; x < nx; ++x)
            for (i64 y = 0; y < ny; ++y) cp_el(out, x * ny + y, in, y * nx + x, es);
        return;
    }
    i64 nz = dims[2];
    #pragma omp parallel for collapse(2) schedule(static)
    for (i64 x = 0; x < nx; ++x)
        for (i64 z = 0; z < nz; ++z)
            for (i64 y = 0; y < ny; ++y)
                cp_el(out, x * ny * nz + z * ny + y, in, z * nx * ny + y * nx + x, es);
}

/* :262-302  (nx,ny,nz) -> (nz,nx,ny) */
void orc_permute_backward(const void* vin, void* vout, const int* dims, int es) {
    const char* in = (const char*)vin; char* out = (char*)vout;
    i64 nx = dims[0], ny = dims[1], nz = dims[2];
    #pragma omp parallel for collapse(2) schedule(static)
    for (i64 y = 0; y < ny; ++y)
        for (i64 x = 0; x < nx; ++x)
            for (i64 z = 0; z < nz; ++z)
                cp_el(out, y * nz * nx + x * nz + z, in, z * nx * ny + y * nx + x, es);
}

/* :351-390  (nx,ny,nz) -> (nz,ny,nx) : first half of the two-step permute */
void orc_permute_backward_start(const void* vin, void* vout, const int* dims, int es) {
    const char* in = (const char*)vin; char* out = (char*)vout;
    i64 nx = dims[0], ny = dims[1], nz = dims[2];
    #pragma omp parallel for collapse(2) schedule(static)
    for (i64 x = 0; x < nx; ++x)
        for (i64 y = 0; y < ny; ++y)
            for (i64 z = 0; z < nz; ++z)
                cp_el(out, x * nz * ny + y * nz + z, in, z * nx * ny + y * nx + x, es);
}

/* :439-502  second half of the two-step permute, one neighbour block.
 * nb = {nxx, nyy, nzz, din, dout} */
void orc_permute_backward_end_one(const void* vin, void* vout, const int* dims, const int* nb, int es) {
    const char* in = (const char*)vin; char* out = (char*)vout;
    i64 nx = dims[0], ny = dims[1];
    i64 nxx = nb[0], nyy = nb[1], nzz = nb[2], din = nb[3], dout = nb[4];
    #pragma omp parallel for collapse(2) schedule(static)
    for (i64 z = 0; z < nzz; ++z)
        for (i64 y = 0; y < nyy; ++y)
            for (i64 x = 0; x < nxx; ++x)
                cp_el(out, dout + z * nx * ny + y * nx + x, in, din + z * nxx + y * nzz * nxx + x, es);
}

/* :575-652  unpack of one neighbour block */
void orc_unpack_one(const void* vin, void* vout, int ndims, const int* dims, const int* nb, int es) {
    const char* in = (const char*)vin; char* out = (char*)vout;
    i64 nx = dims[0], ny = dims[1];
    i64 nxx = nb[0], nyy = nb[1], nzz = (ndims == 2) ? 1 : nb[2], din = nb[3], dout = nb[4];
    #pragma omp parallel for collapse(2) schedule(static)
    for (i64 z = 0; z < nzz; ++z)
        for (i64 y = 0; y < nyy; ++y)
            for (i64 x = 0; x < nxx; ++x)
                cp_el(out, dout + z * nx * ny + y * nx + x, in, din + z * nxx * nyy + y * nxx + x, es);
}

/* :657-737  pack of one neighbour block */
void orc_pack_one(const void* vin, void* vout, int ndims, const int* dims, const int* nb, int es) {
    const char* in = (const char*)vin; char* out = (char*)vout;
    i64 nx = dims[0], ny = dims[1];
    i64 nxx = nb[0], nyy = nb[1], nzz = (ndims == 2) ? 1 : nb[2], din = nb[3], dout = nb[4];
    #pragma omp parallel for collapse(2) schedule(static)
    for (i64 z = 0; z < nzz; ++z)
        for (i64 y = 0; y < nyy; ++y)
            for (i64 x = 0; x < nxx; ++x)
                cp_el(out, dout + z * nxx * nyy + y * nxx + x, in, din + z * nx * ny + y * nx + x, es);
}

/* ------------------------------------------------------------------ */
/* Transpose types (include/dtfft_config.h.in:38-43)                   */
/* ------------------------------------------------------------------ */
enum { T_X_TO_Y = 1, T_Y_TO_X = -1, T_Y_TO_Z = 2, T_Z_TO_Y = -2, T_X_TO_Z = 3, T_Z_TO_X = -3 };

static int send_layout(int t) {
    switch (t) { case T_X_TO_Y: case T_X_TO_Z: return 1; case T_Y_TO_X: case T_Y_TO_Z: return 2; default: return 3; }
}
static int recv_layout(int t) {
    switch (t) { case T_Y_TO_X: case T_Z_TO_X: return 1; case T_X_TO_Y: case T_Z_TO_Y: return 2; default: return 3; }
}

static i64 prod(int n, const int* v) { i64 p = 1; for (int i = 0; i < n; ++i) p *= v[i]; return p; }

/* Element offset of `rank`'s block in a packed buffer of `layout`. */
i64 orc_rank_offset(int ndims, const int* gdims, const int* grid, int layout, int rank) {
    i64 off = 0;
    for (int r = 0; r < rank; ++r) {
        int s[3], c[3];
        orc_pencil(ndims, gdims, grid, layout, r, s, c);
        off += prod(ndims, c);
    }
    return off;
}

int orc_nranks(int ndims, const int* grid) { return ndims == 3 ? grid[1] * grid[2] : grid[1]; }

/* Ranks (in cartesian numbering) of the sub-communicator that `rank` uses for
 * transpose `t`, and rank's position in it.  comm_id 2 keeps grid dim 1,
 * comm_id 3 keeps grid dim 2, comm_id 1 is the whole cartesian comm
 * (src/dtfft_abstract_reshape_handle.F90:155-163). */
static int sub_comm(int ndims, const int* grid, int t, int rank, int* members) {
    int id = (abs(t) == 1) ? 2 : (abs(t) == 2 ? 3 : 1);
    int n = 0;
    if (ndims == 2 || id == 1) {
        int P = orc_nranks(ndims, grid);
        for (int r = 0; r < P; ++r) members[n++] = r;
        return n;
    }
    int c1 = rank / grid[2], c2 = rank % grid[2];
    if (id == 2) { for (int i = 0; i < grid[1]; ++i) members[n++] = i * grid[2] + c2; }
    else         { for (int i = 0; i < grid[2]; ++i) members[n++] = c1 * grid[2] + i; }
    return n;
}

/*
 * One transpose of the whole virtual grid, following
 * src/dtfft_reshape_handle_generic.F90:174-759 with a non-pipelined,
 * non-fused backend (pack -> all-to-all-v -> unpack; :748-758).
 * `in` and `out` are packed multi-rank buffers in the send/recv layouts.
 * `in` is left intact (the reference uses `in` as the receive buffer of the
 * exchange; the oracle uses separate scratch so the input stays readable).
 * Returns 0 on success.
 */
int orc_vgrid_transpose(int ndims, const int* gdims, const int* grid, int t,
                        const void* vin, void* vout, int es) {
    const char* in = (const char*)vin; char* out = (char*)vout;
    int P = orc_nranks(ndims, grid);
    int sl = send_layout(t), rl = recv_layout(t);
    if (ndims == 2 && (abs(t) != 1)) return 2;

    /* per-rank send buffers after the pack kernel */
    char** sendbuf = (char**)calloc((size_t)P, sizeof(char*));
    int* members = (int*)malloc(sizeof(int) * (size_t)P);
    if (!sendbuf || !members) return 1;

    int two_step = (t == T_Y_TO_X || t == T_Z_TO_Y) && ndims == 3;
    int fwd_kernel = (t == T_X_TO_Y || t == T_Y_TO_Z || t == T_Z_TO_X);

    for (int r = 0; r < P; ++r) {
        int s[3], c[3];
        orc_pencil(ndims, gdims, grid, sl, r, s, c);
        i64 n = prod(ndims, c);
        sendbuf[r] = (char*)malloc((size_t)(n > 0 ? n : 1) * (size_t)es);
        if (n == 0) continue;
        const char* src = in + orc_rank_offset(ndims, gdims, grid, sl, r) * es;
        int m = sub_comm(ndims, grid, t, r, members);
        if (m == 1) {
            /* no exchange: the pack kernel writes straight to out (:246-253) */
            char* dst = out + orc_rank_offset(ndims, gdims, grid, rl, r) * es;
            /* 2D backward permutes alias the forward one (src/dtfft_abstract_kernel.F90:272-282) */
            if (fwd_kernel || ndims == 2) orc_permute_forward(src, dst, ndims, c, es);
            else                          orc_permute_backward(src, dst, c, es);
            continue;
        }
        if (ndims == 2 || fwd_kernel)  orc_permute_forward(src, sendbuf[r], ndims, c, es);
        else if (two_step)             orc_permute_backward_start(src, sendbuf[r], c, es);
        else                           orc_permute_backward(src, sendbuf[r], c, es);
    }

    for (int me = 0; me < P; ++me) {
        int m = sub_comm(ndims, grid, t, me, members);
        if (m == 1) continue;
        int my_pos = 0;
        for (int i = 0; i < m; ++i) if (members[i] == me) my_pos = i;
        (void)my_pos;
        int rs[3], rc[3];
        orc_pencil(ndims, gdims, grid, rl, me, rs, rc);
        if (prod(ndims, rc) == 0) continue;
        char* dst = out + orc_rank_offset(ndims, gdims, grid, rl, me) * es;
        int ms[3], mc[3];               /* my send pencil */
        orc_pencil(ndims, gdims, grid, sl, me, ms, mc);
        for (int i = 0; i < m; ++i) {
            int peer = members[i];
            int ps[3], pc[3];           /* peer's send pencil (in%sizes(:,i)) */
            orc_pencil(ndims, gdims, grid, sl, peer, ps, pc);
            /* displacement of my chunk inside peer's send buffer: sum over the
             * peer's destinations that precede me (the sdispl loop, :395-409) */
            i64 sdispl = 0, rsize = 0;
            for (int k = 0; k < m; ++k) {
                int ks[3], kc[3];      /* recv pencil of destination k (out%sizes(:,k)) */
                orc_pencil(ndims, gdims, grid, rl, members[k], ks, kc);
                int ln[3];
                if (ndims == 2) { ln[0] = kc[1]; ln[1] = pc[1]; ln[2] = 1; }
                else if (t == T_X_TO_Z) { ln[0] = pc[0]; ln[1] = kc[2]; ln[2] = pc[2]; }
                else if (t == T_Z_TO_X) { ln[0] = kc[2]; ln[1] = pc[1]; ln[2] = pc[2]; }
                else if (t == T_X_TO_Y || t == T_Y_TO_Z) { ln[0] = kc[2]; ln[1] = pc[1]; ln[2] = pc[2]; }
                else { ln[0] = kc[1]; ln[1] = pc[1]; ln[2] = pc[2]; }
                i64 sz = (i64)ln[0] * ln[1] * ln[2];
                if (members[k] == me) { rsize = sz; break; }
                sdispl += sz;
            }
            if (rsize == 0) continue;
            const char* chunk = sendbuf[peer] + sdispl * es;
            /* receive-side box (out%ln / out%ls, :488-531) and unpack data (:559-571) */
            int nb[5];
            if (ndims == 2) {
                nb[0] = pc[1]; nb[1] = rc[1]; nb[2] = 1; nb[4] = ps[1];
            } else if (t == T_X_TO_Z) {
                nb[0] = pc[2]; nb[1] = rc[1]; nb[2] = rc[2]; nb[4] = ps[2];
            } else if (t == T_Z_TO_X) {
                nb[0] = rc[0]; nb[1] = pc[2]; nb[2] = rc[2]; nb[4] = rc[0] * ps[2];
            } else if (t == T_X_TO_Y || t == T_Y_TO_Z) {
                nb[0] = pc[1]; nb[1] = rc[1]; nb[2] = rc[2]; nb[4] = ps[1];
            } else {
                nb[0] = pc[2]; nb[1] = rc[1]; nb[2] = rc[2]; nb[4] = ps[2];
            }
            nb[3] = 0;  /* the chunk pointer already carries the receive displacement */
            if (two_step) orc_permute_backward_end_one(chunk, dst, rc, nb, es);
            else          orc_unpack_one(chunk, dst, ndims, rc, nb, es);
        }
    }
    for (int r = 0; r < P; ++r) free(sendbuf[r]);
    free(sendbuf);
    free(members);
    return 0;
}

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
