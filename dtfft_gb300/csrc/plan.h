// Internal plan structures of the GB300 execute path.
#pragma once

#include <vector>

#include "common.cuh"
#include "dtfft_gb300.h"
#include "fft.cuh"

namespace gb {

// Local box of one virtual rank in one layout, pencil-dim order (aligned dim first).
struct RankBox {
    int start[3];
    int count[3];
};

// One data layout of the whole virtual grid: every rank's box plus the
// element offset of its block in the packed buffer.
struct Layout {
    int id = 0;          // aligned dim 1 (X), 2 (Y), 3 (Z)
    int nd = 3;
    int axes[3] = {0, 1, 2};   // global axis of pencil dim d (0 = X)
    int gsize[3] = {1, 1, 1};  // global extent of pencil dim d
    std::vector<RankBox> r;
    std::vector<i64> off;      // size P + 1
    i64 total = 0;
    i64 max_local = 0;
};

Layout make_pencil_layout(int ndims, const int* gdims, const int* grid, int aligned);
// Even split of n points over P ranks, remainder to the last ranks.
void split(int n, int P, int r, int& start, int& count);
// Global axis and grid-comm index of each pencil dim of layout `aligned`.
void perms(int ndims, int aligned, int* axes, int* comms);
// Layout of pencil order `aligned` from every rank's box (pencil-dim order).
Layout layout_from_boxes(int ndims, int aligned, const int* gdims, const std::vector<RankBox>& boxes);

// Plans over user-defined blocks (bricks.cpp).
struct UserGeometry {
    int dims[3] = {1, 1, 1};   // global dims of the user's data (real dims for R2C)
    int grid[3] = {1, 1, 1};   // sizes of the pencil grid communicators
    bool z_slab = false, y_slab = false;
    bool reshape = false;      // the blocks split X: brick <-> pencil reshapes
    int final_grid = 1;        // ranks that share one Fourier-space brick split
    Layout pen[3];             // pencils of the transformed type
    Layout real_x;             // R2C: real X pencils
    Layout brick_x;            // the user's blocks (real space)
    Layout brick_z;            // Fourier-space bricks (aligned like the last pencil)
};
dtfft_error_t user_geometry(int ndims, int nranks, const int* starts, const int* counts, bool r2c,
                            bool z_slab_conf, bool y_slab_conf, UserGeometry& g);
BoxList make_boxes(const Layout& S, const Layout& R, int elem);
TransposeConfig default_tile(int elem);
const dtfft_config_t& config();

// What a communicator handle stands for (dtfft_mpi_shim.h).
struct VCommInfo { bool known; bool cart; int nprocs; int ndims; int dims[3]; };
VCommInfo comm_info(MPI_Comm comm);
// Blocks registered with dtfft_vgrid_pencils_create (starts/counts: nprocs x ndims).
bool comm_blocks(MPI_Comm comm, int* ndims, std::vector<int32_t>* starts, std::vector<int32_t>* counts);
void default_config(dtfft_config_t* c);

// Measured choice of a transpose tile (autotune.cpp).
dtfft_error_t autotune_boxes(BoxList& bl, i64 max_elems, cudaStream_t s, int warmup, int iters, bool log);

}  // namespace gb
