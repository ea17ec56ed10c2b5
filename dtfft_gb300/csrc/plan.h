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
BoxList make_boxes(const Layout& S, const Layout& R, int elem);
TransposeConfig default_tile(int elem);
const dtfft_config_t& config();

// What a communicator handle stands for (dtfft_mpi_shim.h).
struct VCommInfo { bool known; bool cart; int nprocs; int ndims; int dims[3]; };
VCommInfo comm_info(MPI_Comm comm);
void default_config(dtfft_config_t* c);

// Measured choice of a transpose tile (autotune.cpp).
dtfft_error_t autotune_boxes(BoxList& bl, i64 max_elems, cudaStream_t s, int warmup, int iters, bool log);

}  // namespace gb
