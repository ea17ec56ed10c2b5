// Geometry of plans built from user-defined blocks: every virtual rank's own
// (starts, counts), registered with dtfft_vgrid_pencils_create and passed to
// dtfft_create_plan_*_pencil.  When the blocks split the X axis they are
// "bricks" and the plan adds the brick <-> pencil reshapes.
//
// For ranks that all live in this process this restates:
//   create_pencil_init       src/dtfft_pencil.F90:777-908  (checks, 1D comms)
//   create_1d_comm           src/dtfft_pencil.F90:1034-1081
//   from_bricks              src/dtfft_pencil.F90:520-775  (X pencils of X-split bricks)
//   pencil%create, get_local_size  src/dtfft_pencil.F90:109-279 (kept starts/counts)
//   create_pencils_and_comm  src/dtfft_transpose_plan.F90:1084-1131
//   reshape_plan%create      src/dtfft_reshape_plan.F90:98-260 (Fourier-space bricks)
// An MPI communicator becomes an ordered group of virtual ranks; a split
// orders its members by (key, rank in the parent) as MPI_Comm_split does.
#include <algorithm>
#include <array>
#include <map>

#include "plan.h"

namespace gb {

namespace {

using I3 = std::array<int, 3>;

// Disjoint sub-communicators covering ranks 0..P-1.
struct Comms {
    std::vector<std::vector<int>> groups;
    std::vector<int> of, pos;
    void finish(int P) {
        of.assign(P, -1);
        pos.assign(P, -1);
        for (int g = 0; g < (int)groups.size(); ++g)
            for (int i = 0; i < (int)groups[g].size(); ++i) {
                of[groups[g][i]] = g;
                pos[groups[g][i]] = i;
            }
    }
    int size(int r) const { return (int)groups[of[r]].size(); }
    int rank(int r) const { return pos[r]; }
    const std::vector<int>& members(int r) const { return groups[of[r]]; }
};

Comms self_comms(int P) {
    Comms c;
    for (int r = 0; r < P; ++r) c.groups.push_back({r});
    c.finish(P);
    return c;
}

Comms world_comm(int P) {
    Comms c;
    c.groups.emplace_back();
    for (int r = 0; r < P; ++r) c.groups[0].push_back(r);
    c.finish(P);
    return c;
}

// MPI_Comm_split of every group of `parent`.
Comms split_comm(const Comms& parent, const std::vector<int>& color, const std::vector<int>& key) {
    Comms c;
    for (const auto& g : parent.groups) {
        std::map<int, std::vector<int>> by;   // color -> members in parent order
        for (int r : g) by[color[r]].push_back(r);
        for (auto& kv : by) {
            std::vector<int> m = kv.second;
            std::stable_sort(m.begin(), m.end(), [&](int a, int b) { return key[a] < key[b]; });
            c.groups.push_back(m);
        }
    }
    c.finish((int)parent.of.size());
    return c;
}

// get_local_size without kept values: even split by rank in the communicator.
void even(int n, const Comms& c, int r, int& start, int& count) {
    if (c.size(r) == 1) { start = 0; count = n; return; }
    split(n, c.size(r), c.rank(r), start, count);
}

// get_local_size with kept start/count: a one-rank communicator owns all of n.
void kept(int n, const Comms& c, int r, int ks, int kc, int& start, int& count) {
    if (c.size(r) == 1) { start = 0; count = n; return; }
    start = ks;
    count = kc;
}

int min_over(const Comms& c, int r, const std::vector<I3>& v, int d) {
    int m = v[r][d];
    for (int q : c.members(r)) m = std::min(m, v[q][d]);
    return m;
}

// The user's blocks after create_pencil_init.
struct Blocks {
    int nd = 3, P = 1;
    int dims[3] = {1, 1, 1};
    std::vector<I3> s, c;   // Fortran order
    Comms comms[3];
};

bool zero_volume(const I3& c, int nd) {
    for (int d = 0; d < nd; ++d) if (c[d] == 0) return true;
    return false;
}

// create_1d_comm: the ranks whose blocks line up with rank r along `var`.
std::vector<int> line_of(const Blocks& b, int r, int var) {
    std::vector<int> nb, coord;
    for (int i = 0; i < b.P; ++i) {
        bool matched = true;
        for (int j = 0; j < b.nd; ++j) {
            if (j == var) continue;
            if (b.s[i][j] != b.s[r][j] || b.c[i][j] != b.c[r][j]) matched = false;
        }
        const bool same = b.s[i][var] == b.s[r][var];
        if ((matched && !same) || i == r || (matched && same && (b.c[i][var] == 0 || b.c[r][var] == 0))) {
            nb.push_back(i);
            coord.push_back(b.s[i][var]);
        }
    }
    // stable insertion order by coordinate (sort_by_varying_dim)
    std::vector<int> idx(nb.size());
    for (size_t i = 0; i < idx.size(); ++i) idx[i] = (int)i;
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int q) { return coord[a] < coord[q]; });
    std::vector<int> out;
    for (int i : idx) out.push_back(nb[i]);
    return out;
}

dtfft_error_t pencil_init(int nd, int P, const int* starts, const int* counts, Blocks& b) {
    b.nd = nd;
    b.P = P;
    b.s.assign(P, I3{0, 0, 0});
    b.c.assign(P, I3{1, 1, 1});
    for (int r = 0; r < P; ++r)
        for (int d = 0; d < nd; ++d) { b.s[r][d] = starts[r * nd + d]; b.c[r][d] = counts[r * nd + d]; }
    for (int r = 0; r < P; ++r)
        for (int d = 0; d < nd; ++d) if (b.s[r][d] < 0) return DTFFT_ERROR_PENCIL_INVALID_STARTS;
    for (int r = 0; r < P; ++r)
        for (int d = 0; d < nd; ++d) if (b.c[r][d] < 0) return DTFFT_ERROR_PENCIL_INVALID_COUNTS;
    for (int d = 0; d < nd; ++d) {
        b.dims[d] = 0;
        for (int r = 0; r < P; ++r) b.dims[d] = std::max(b.dims[d], b.s[r][d] + b.c[r][d]);
    }
    // equal starts on two axes need equal counts on both
    for (int p1 = 0; p1 < P; ++p1) {
        if (zero_volume(b.c[p1], nd)) continue;
        for (int p2 = p1 + 1; p2 < P; ++p2) {
            if (zero_volume(b.c[p2], nd)) continue;
            for (int d1 = 0; d1 < nd; ++d1)
                for (int d2 = d1 + 1; d2 < nd; ++d2)
                    if (b.s[p1][d1] == b.s[p2][d1] && b.s[p1][d2] == b.s[p2][d2] &&
                        (b.c[p1][d1] != b.c[p2][d1] || b.c[p1][d2] != b.c[p2][d2]))
                        return DTFFT_ERROR_PENCIL_SHAPE_MISMATCH;
        }
    }
    for (int i = 0; i < P; ++i)
        for (int j = i + 1; j < P; ++j) {
            if (zero_volume(b.c[i], nd) || zero_volume(b.c[j], nd)) continue;
            bool ov = true;
            for (int d = 0; d < nd; ++d)
                if (b.s[i][d] + b.c[i][d] <= b.s[j][d] || b.s[j][d] + b.c[j][d] <= b.s[i][d]) ov = false;
            if (ov) return DTFFT_ERROR_PENCIL_OVERLAP;
        }
    i64 vol = 0, gvol = 1;
    for (int r = 0; r < P; ++r) {
        if (zero_volume(b.c[r], nd)) continue;
        i64 v = 1;
        for (int d = 0; d < nd; ++d) v *= b.c[r][d];
        vol += v;
    }
    for (int d = 0; d < nd; ++d) gvol *= b.dims[d];
    if (vol != gvol) return DTFFT_ERROR_PENCIL_NOT_CONTINUOUS;
    // 1D communicators; every member of a line must see the same line
    for (int d = 0; d < nd; ++d) {
        Comms& c = b.comms[d];
        std::vector<int> seen(P, -1);
        for (int r = 0; r < P; ++r) {
            if (seen[r] >= 0) continue;
            std::vector<int> g = line_of(b, r, d);
            for (int q : g) {
                if (seen[q] >= 0 || line_of(b, q, d) != g) return DTFFT_ERROR_PENCIL_SHAPE_MISMATCH;
                seen[q] = (int)c.groups.size();
            }
            c.groups.push_back(g);
        }
        c.finish(P);
    }
    for (int r = 0; r < P; ++r) {
        i64 prod = 1;
        for (int d = 0; d < nd; ++d) prod *= b.comms[d].size(r);
        if (prod != P) return DTFFT_ERROR_PENCIL_SHAPE_MISMATCH;
    }
    return DTFFT_SUCCESS;
}

// MPI_Dims_create(n, 2): the most balanced a x b = n with a >= b.
void dims_create2(int n, int& a, int& b) {
    a = n; b = 1;
    for (int q = 1; q * q <= n; ++q)
        if (n % q == 0) { a = n / q; b = q; }
}

// X pencils of X-split bricks on a communicator without topology
// (from_bricks); the result is a Blocks with X whole on every rank.
Blocks from_bricks(const Blocks& br) {
    const int nd = br.nd, P = br.P;
    const Comms& B1 = br.comms[0];
    const int fast = B1.size(0);
    const int tile = 32;   // DEF_TILE_SIZE, src/dtfft_parameters.F90:555
    const I3& c0 = br.c[0];   // rank 0's brick decides for everyone (MPI_Bcast)
    int ys = 0, zs = 0;
    bool nice = false;
    if (nd == 3 && c0[2] > tile * fast) { ys = 1; zs = fast; nice = true; }
    else if (c0[1] > tile * fast || nd == 2) { ys = fast; zs = 1; nice = true; }
    else {
        for (int i = 2; i <= fast; ++i) {
            if (fast % i != 0) continue;
            if (c0[nd - 1] < tile * i || c0[nd - 1] % i != 0) continue;
            if (c0[1] < tile * i || c0[1] % i != 0) continue;
            nice = true;
            ys = std::min(i, fast / i);
            zs = std::max(i, fast / i);
            break;
        }
    }
    if (!nice) dims_create2(fast, ys, zs);

    Comms self = self_comms(P);
    Comms pc2, pc3;
    std::vector<int> ay(P, 0), az(P, 0);
    if (ys == 1) {
        pc2 = self;
        pc3 = B1;
        for (int r = 0; r < P; ++r) az[r] = B1.rank(r);
    } else if (zs == 1) {
        pc2 = B1;
        pc3 = self;
        for (int r = 0; r < P; ++r) ay[r] = B1.rank(r);
    } else {
        // MPI_Cart_create(B1, (ys, zs), reorder = false) + MPI_Cart_sub
        std::vector<int> cy(P), cz(P), ky(P), kz(P);
        for (int r = 0; r < P; ++r) {
            const int k = B1.rank(r);
            ay[r] = k / zs;
            az[r] = k % zs;
            cy[r] = az[r]; ky[r] = ay[r];
            cz[r] = ay[r]; kz[r] = az[r];
        }
        pc2 = split_comm(B1, cy, ky);
        pc3 = split_comm(B1, cz, kz);
    }
    Blocks o;
    o.nd = nd;
    o.P = P;
    for (int d = 0; d < 3; ++d) o.dims[d] = br.dims[d];
    o.s.assign(P, I3{0, 0, 0});
    o.c.assign(P, I3{1, 1, 1});
    for (int r = 0; r < P; ++r) {
        o.s[r][0] = 0;
        o.c[r][0] = br.dims[0];
        int st, ct;
        even(br.c[r][1], pc2, r, st, ct);
        o.s[r][1] = st + min_over(pc2, r, br.s, 1);   // own start when pc2 is a single rank
        o.c[r][1] = ct;
        if (nd == 3) {
            even(br.c[r][2], pc3, r, st, ct);
            o.s[r][2] = st + min_over(pc3, r, br.s, 2);
            o.c[r][2] = ct;
        }
    }
    Comms world = world_comm(P);
    o.comms[0] = self;
    std::vector<int> color(P), key(P);
    if (nd == 2) {
        for (int r = 0; r < P; ++r) { color[r] = 0; key[r] = o.s[r][1]; }
        o.comms[1] = split_comm(world, color, key);
    } else {
        for (int r = 0; r < P; ++r) { color[r] = br.comms[2].rank(r) * zs + az[r]; key[r] = o.s[r][1]; }
        o.comms[1] = split_comm(world, color, key);
        for (int r = 0; r < P; ++r) { color[r] = br.comms[1].rank(r) * ys + ay[r]; key[r] = o.s[r][2]; }
        o.comms[2] = split_comm(world, color, key);
    }
    return o;
}

}  // namespace

dtfft_error_t user_geometry(int nd, int P, const int* starts, const int* counts, bool r2c, bool zs_conf,
                            bool ys_conf, UserGeometry& g) {
    Blocks br;
    GB_TRY(pencil_init(nd, P, starts, counts, br));
    for (int d = 0; d < 3; ++d) g.dims[d] = d < nd ? br.dims[d] : 1;
    int tdims[3] = {g.dims[0], g.dims[1], g.dims[2]};
    if (r2c) tdims[0] = g.dims[0] / 2 + 1;

    g.reshape = br.comms[0].size(0) > 1;
    Blocks ip = g.reshape ? from_bricks(br) : br;   // the X pencils the transpose plan starts from
    const Comms* cm = ip.comms;

    // create(): grid from the pencil communicators (src/dtfft_transpose_plan.F90:115-132)
    for (int d = 0; d < 3; ++d) g.grid[d] = d < nd ? cm[d].size(0) : 1;
    if (g.grid[0] != 1) return DTFFT_ERROR_INVALID_COMM_FAST_DIM;
    g.z_slab = g.y_slab = false;
    if (nd == 3) {
        if (g.grid[1] == 1 && zs_conf) g.z_slab = true;
        else if (g.grid[2] == 1 && ys_conf) g.y_slab = true;
    }

    // pencils chained from the X pencil (create_pencils_and_comm with ipencil)
    std::vector<RankBox> bx(P), by(P), bz(P), breal(P);
    for (int r = 0; r < P; ++r) {
        for (int d = 0; d < 3; ++d) { bx[r].start[d] = ip.s[r][d]; bx[r].count[d] = ip.c[r][d]; }
        breal[r] = bx[r];
        if (r2c) bx[r].count[0] = tdims[0];
        RankBox& y = by[r];
        if (nd == 3) {
            // (Y, Z, X) over (c1, c3, c2)
            even(tdims[1], cm[0], r, y.start[0], y.count[0]);
            kept(tdims[2], cm[2], r, bx[r].start[2], bx[r].count[2], y.start[1], y.count[1]);
            even(tdims[0], cm[1], r, y.start[2], y.count[2]);
            // (Z, X, Y) over (c1, c2, c3)
            RankBox& z = bz[r];
            even(tdims[2], cm[0], r, z.start[0], z.count[0]);
            kept(tdims[0], cm[1], r, y.start[2], y.count[2], z.start[1], z.count[1]);
            even(tdims[1], cm[2], r, z.start[2], z.count[2]);
        } else {
            // (Y, X) over (c1, c2)
            even(tdims[1], cm[0], r, y.start[0], y.count[0]);
            even(tdims[0], cm[1], r, y.start[1], y.count[1]);
            y.start[2] = 0; y.count[2] = 1;
        }
    }
    g.pen[0] = layout_from_boxes(nd, 1, tdims, bx);
    g.pen[1] = layout_from_boxes(nd, 2, tdims, by);
    if (nd == 3) g.pen[2] = layout_from_boxes(nd, 3, tdims, bz);
    if (r2c) g.real_x = layout_from_boxes(nd, 1, g.dims, breal);
    if (!g.reshape) return DTFFT_SUCCESS;

    // user bricks (real space) and the Fourier-space bricks of the last pencil
    std::vector<RankBox> b1(P), b2(P);
    for (int r = 0; r < P; ++r)
        for (int d = 0; d < 3; ++d) { b1[r].start[d] = br.s[r][d]; b1[r].count[d] = br.c[r][d]; }
    g.brick_x = layout_from_boxes(nd, 1, g.dims, b1);
    const Layout& last = g.pen[nd - 1];
    const Comms& local = cm[nd - 1];
    // neighbour groups of c_size consecutive ranks (create_custom_comm, NEIGHBOR_GROUP)
    std::vector<int> color(P), key(P);
    for (int r = 0; r < P; ++r) {
        const int cs = br.comms[nd - 1].size(r);
        color[r] = local.rank(r) / cs;
        key[r] = local.rank(r);
    }
    Comms R3 = split_comm(local, color, key);
    std::vector<I3> ls(P);
    for (int r = 0; r < P; ++r) for (int d = 0; d < 3; ++d) ls[r][d] = last.r[r].start[d];
    for (int r = 0; r < P; ++r) {
        int slow = 0;
        for (int q : R3.members(r)) slow += last.r[q].count[nd - 1];
        RankBox& z = b2[r];
        even(g.dims[nd - 1], R3, r, z.start[0], z.count[0]);
        if (nd == 3) {
            z.start[1] = last.r[r].start[1];
            z.count[1] = last.r[r].count[1];
        }
        z.start[nd - 1] = min_over(R3, r, ls, nd - 1);
        z.count[nd - 1] = slow;
        if (nd == 2) { z.start[2] = 0; z.count[2] = 1; }
    }
    g.brick_z = layout_from_boxes(nd, nd, tdims, b2);
    g.final_grid = R3.size(0);
    return DTFFT_SUCCESS;
}

}  // namespace gb
