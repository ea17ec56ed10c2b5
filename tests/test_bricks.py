"""Plans over user-defined blocks (CPU part): the oracle's decomposition against
the facts the reference's own brick test asserts, the oracle's data placement
against the pencil oracle, and the library's block checks (they run before any
device call, so they need no GPU).

Reference test: tests/c/test_c2c_3d_c.c:105-186 (96 x 64 x 512 in dtFFT's
dims order, 2 / 4 / 8 ranks, z-slab and y-slab off, Fourier reshape on)."""
import numpy as np
import pytest

from oracle import bricks as ob


def ref_test_blocks(comm_size, nx=512, ny=64, nz=96):
    """The blocks tests/c/test_c2c_3d_c.c:105-136 gives each rank (dims order
    [nz, ny, nx], dims[0] fastest)."""
    grid_z = 2 if comm_size == 8 else 1
    grid_y = 2 if comm_size >= 4 else 1
    grid_x = comm_size // (grid_z * grid_y)
    blocks = []
    for r in range(comm_size):
        rz = r // (grid_y * grid_x)
        ry = (r // grid_x) % grid_y
        rx = r % grid_x
        st = [rz * (nz // grid_z), ry * (ny // grid_y), rx * (nx // grid_x)]
        ct = [nz // grid_z, ny // grid_y, nx // grid_x]
        if comm_size == 2:
            st[2], ct[2] = (nx // 4, 3 * nx // 4) if r == 0 else (0, nx // 4)
        blocks.append((st, ct))
    return blocks


@pytest.mark.parametrize("comm_size,grid", [(2, [1, 1, 2]), (4, [1, 2, 2]), (8, [1, 2, 4])])
def test_oracle_matches_reference_brick_test(comm_size, grid):
    blocks = ref_test_blocks(comm_size)
    g = ob.geometry([b[0] for b in blocks], [b[1] for b in blocks], z_slab=False, y_slab=False,
                    fourier_reshape=True)
    assert g["dims"] == [96, 64, 512]
    assert g["grid"] == grid
    assert g["reshape"] == (comm_size == 8)
    if comm_size != 8:
        # "in_starts == pencil.starts": X pencils are the user's blocks
        for r, (st, ct) in enumerate(blocks):
            assert g["x"][r] == (st, ct)
    else:
        assert g["final_reshape"]


CONFIGS = [
    # (blocks builder args)  bricks grid along (X, Y, Z), dims
    ((2, 2, 2), [96, 64, 512]),
    ((2, 2, 2), [33, 17, 40]),
    ((4, 1, 2), [40, 30, 20]),       # fast = 4 with thin Z: Dims_create branch
    ((2, 1, 1), [20, 300, 16]),      # Y-split X pencils
    ((2, 3, 1), [12, 9, 200]),
    ((4, 2, 1), [64, 256, 256]),     # 2 x 2 cartesian sub-grid of the X line
    ((1, 2, 2), [18, 33, 15]),       # X not split: no reshape
]

CONFIGS_2D = [((2, 2), [40, 36]), ((3, 1), [25, 70]), ((1, 3), [25, 70])]


def grid_blocks(bgrid, dims):
    nd = len(dims)
    blocks = []
    P = int(np.prod(bgrid))
    for r in range(P):
        idx, rem = [], r
        for d in range(nd):
            idx.append(rem % bgrid[d])
            rem //= bgrid[d]
        st, ct = [], []
        for d in range(nd):
            base, res = divmod(dims[d], bgrid[d])
            cnts = [base + (1 if i >= bgrid[d] - res else 0) for i in range(bgrid[d])]
            st.append(sum(cnts[:idx[d]]))
            ct.append(cnts[idx[d]])
        blocks.append((st, ct))
    return blocks


def _partition_ok(g, nd, aligned_of):
    rng = np.random.default_rng(0)
    for name, aligned in aligned_of.items():
        if name not in g or not g[name]:
            continue
        gd = g["tdims"] if name in ("x", "y", "z", "zb") else g["dims"]
        arr = rng.standard_normal(tuple(gd[::-1]))
        boxes = g[name]
        assert sum(int(np.prod(c)) for _, c in boxes) == arr.size, name
        back = ob.unpack(ob.pack(arr, boxes, aligned), gd, boxes, aligned)
        assert np.array_equal(back, arr), name


@pytest.mark.parametrize("bgrid,dims", CONFIGS + CONFIGS_2D)
@pytest.mark.parametrize("r2c", [False, True])
def test_oracle_layouts_partition_the_domain(bgrid, dims, r2c):
    blocks = grid_blocks(bgrid, dims)
    g = ob.geometry([b[0] for b in blocks], [b[1] for b in blocks], r2c=r2c, z_slab=False)
    nd = len(dims)
    aligned = {"x": 1, "xr": 1, "y": 2, "xb": 1, "zb": nd}
    if nd == 3:
        aligned["z"] = 3
    _partition_ok(g, nd, aligned)
    assert g["reshape"] == (bgrid[0] > 1)


@pytest.mark.parametrize("dims,grid,layout", [([18, 33, 15], [1, 2, 3], 1), ([18, 33, 15], [1, 2, 3], 2),
                                              ([18, 33, 15], [1, 2, 3], 3), ([17, 23], [1, 3], 2)])
def test_oracle_pack_matches_pencil_oracle(orc, dims, grid, layout):
    nd = len(dims)
    P = grid[1] * (grid[2] if nd == 3 else 1)
    boxes = [tuple(map(list, orc.pencil(nd, dims, grid, layout, r))) for r in range(P)]
    g = np.random.default_rng(1).standard_normal(tuple(dims[::-1]))
    assert np.array_equal(ob.pack(g, boxes, layout), orc.global_to_packed(g, nd, grid, layout))


BAD = [
    ("overlap", [([0, 0, 0], [4, 4, 4]), ([2, 0, 0], [4, 4, 4])], ob.E_OVERLAP),
    ("gap", [([0, 0, 0], [4, 4, 4]), ([5, 0, 0], [3, 4, 4])], ob.E_CONT),
    ("negative start", [([0, 0, -1], [4, 4, 4]), ([4, 0, 0], [4, 4, 4])], ob.E_STARTS),
    ("negative count", [([0, 0, 0], [4, 4, -4]), ([4, 0, 0], [4, 4, 4])], ob.E_COUNTS),
    ("shape mismatch", [([0, 0, 0], [4, 4, 4]), ([4, 0, 0], [4, 4, 2]), ([4, 0, 2], [4, 4, 2]),
                        ([0, 4, 0], [8, 4, 4])], ob.E_SHAPE),
]


@pytest.mark.parametrize("name,blocks,code", BAD, ids=[b[0] for b in BAD])
def test_invalid_blocks_are_refused(dt, name, blocks, code):
    with pytest.raises(ob.PencilError) as e:
        ob.geometry([b[0] for b in blocks], [b[1] for b in blocks])
    assert e.value.code == code
    comm = dt.pencils_comm(blocks)
    with pytest.raises(dt.DtfftError) as e2:
        dt.PlanC2C(dt.Pencil(*blocks[0]), comm=comm, precision=dt.Precision.SINGLE)
    assert e2.value.code == code


def test_pencil_must_be_rank0_block(dt):
    blocks = grid_blocks((1, 2, 1), [8, 8, 8])
    comm = dt.pencils_comm(blocks)
    with pytest.raises(dt.DtfftError) as e:
        dt.PlanC2C(dt.Pencil(*blocks[1]), comm=comm, precision=dt.Precision.SINGLE)
    assert e.value.code == 29
