"""CPU tests of the oracle itself (no GPU).

The reference ships no golden vectors for this path (its tests pin transposes
by device == host kernels and FFTs by round trips), so the oracle is pinned by:
  * two independent derivations of every transpose agreeing bit-exactly: the
    step-by-step restatement of the reference's pack -> all-to-all-v -> unpack
    (dtfft_oracle.c) and the pencil semantics (global sub-boxes);
  * scipy/pocketfft checked against the DFT / DCT / DST definitions FFTW
    documents for the kinds the executors use;
  * the reference's own round-trip scale conventions
    (tests/python/test_r2r_kinds_py.py) and error threshold
    (tests/test_utils.F90:89-109).
"""
import itertools

import numpy as np
import pytest

GRIDS_3D = [
    ([18, 33, 155], [1, 1, 1]),
    ([18, 33, 155], [1, 2, 3]),
    ([17, 10, 9], [1, 3, 2]),
    ([16, 8, 12], [1, 1, 4]),
    ([16, 12, 8], [1, 4, 1]),
    ([5, 7, 9], [1, 4, 4]),
    ([3, 7, 9], [1, 4, 4]),     # ranks with zero-sized blocks (3 split over 4)
    ([64, 48, 32], [1, 2, 4]),
]
GRIDS_2D = [([18, 155], [1, 1]), ([17, 23], [1, 3]), ([31, 44], [1, 4]), ([3, 5], [1, 4])]


def _types(nd, grid):
    if nd == 2:
        return [1, -1]
    return [1, -1, 2, -2] + ([3, -3] if grid[1] == 1 else [])


@pytest.mark.parametrize("gd,grid", GRIDS_3D + GRIDS_2D)
@pytest.mark.parametrize("dtype", [np.float32, np.complex64, np.complex128])
def test_restatement_matches_pencil_semantics(orc, gd, grid, dtype):
    nd = len(gd)
    rng = np.random.default_rng(7)
    g = rng.standard_normal(tuple(gd[::-1]))
    if np.issubdtype(dtype, np.complexfloating):
        g = g + 1j * rng.standard_normal(g.shape)
    g = g.astype(dtype)
    for t in _types(nd, grid):
        sl = {1: 1, -1: 2, 2: 2, -2: 3, 3: 1, -3: 3}[t]
        rl = {1: 2, -1: 1, 2: 3, -2: 2, 3: 3, -3: 1}[t]
        pin = orc.global_to_packed(g, nd, grid, sl)
        out = orc.vgrid_transpose(nd, gd, grid, t, pin)
        assert np.array_equal(out, orc.global_to_packed(g, nd, grid, rl)), (gd, grid, t)


def test_full_cycles_are_identity(orc):
    gd, grid = [20, 14, 11], [1, 3, 2]
    g = np.arange(np.prod(gd), dtype=np.float64).reshape(gd[::-1])   # ramp input, as test_host_kernels.F90
    x = orc.global_to_packed(g, 3, grid, 1)
    y = orc.vgrid_transpose(3, gd, grid, 1, x)
    z = orc.vgrid_transpose(3, gd, grid, 2, y)
    y2 = orc.vgrid_transpose(3, gd, grid, -2, z)
    x2 = orc.vgrid_transpose(3, gd, grid, -1, y2)
    assert np.array_equal(x, x2)


def test_local_size_rule(orc):
    # remainder goes to the last ranks (src/dtfft_pencil.F90:258-262)
    assert [orc.local_size(513, 4, r) for r in range(4)] == [(0, 128), (128, 128), (256, 128), (384, 129)]
    assert [orc.local_size(10, 4, r) for r in range(4)] == [(0, 2), (2, 2), (4, 3), (7, 3)]
    assert orc.local_size(7, 1, 0) == (0, 7)


def test_pencils_partition_global(orc):
    # mirrors tests/python/test_pencil_api_py.py: sizes over all ranks sum to the grid size
    for gd, grid in GRIDS_3D:
        for layout in (1, 2, 3):
            tot = sum(int(np.prod(orc.pencil(3, gd, grid, layout, r)[1])) for r in range(orc.nranks(3, grid)))
            assert tot == int(np.prod(gd))


def test_config2_pencils(orc):
    # 512^3 on a 2x4 grid: X (512,256,128), Y (512,128,256), Z (512,256,128)
    gd, grid = [512, 512, 512], [1, 2, 4]
    assert orc.pencil(3, gd, grid, 1, 0)[1] == [512, 256, 128]
    assert orc.pencil(3, gd, grid, 2, 0)[1] == [512, 128, 256]
    assert orc.pencil(3, gd, grid, 3, 0)[1] == [512, 256, 128]


def test_config3_pencils(orc):
    # R2C 1024x1024x512 on 4x4: complex X dim 513 -> Y pencil X counts 128|129 (last rank)
    gd, grid = [513, 1024, 512], [1, 4, 4]
    xs = [orc.pencil(3, gd, grid, 2, r)[1][2] for r in range(0, 16, 4)]
    assert xs == [128, 128, 128, 129]


@pytest.mark.parametrize("n", [1, 2, 3, 5, 7, 8, 12, 17, 23, 30])
def test_numpy_fft_pinned_to_definition(orc, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal((3, n)) + 1j * rng.standard_normal((3, n))
    np.testing.assert_allclose(np.fft.fft(x), orc.dft_direct(x, -1), rtol=0, atol=1e-11 * n)
    np.testing.assert_allclose(np.fft.ifft(x) * n, orc.dft_direct(x, +1), rtol=0, atol=1e-11 * n)


@pytest.mark.parametrize("kind", [3, 4, 5, 6, 7, 8, 9, 10])
@pytest.mark.parametrize("n", [2, 3, 8, 17, 23])
def test_r2r_pinned_to_fftw_definitions(orc, kind, n):
    rng = np.random.default_rng(kind * 100 + n)
    x = rng.standard_normal((2, n))
    np.testing.assert_allclose(orc.r2r(x, kind, axis=-1), orc.r2r_direct(x, kind), rtol=0, atol=1e-10 * n)


@pytest.mark.parametrize("kinds,scale", [
    ((5, 5), lambda nx, ny: 4 * nx * ny),
    ((4, 4), lambda nx, ny: 4 * nx * ny),
    ((3, 3), lambda nx, ny: 4 * (nx - 1) * (ny - 1)),
    ((6, 6), lambda nx, ny: 4 * nx * ny),
    ((7, 7), lambda nx, ny: 4 * (nx + 1) * (ny + 1)),
    ((9, 9), lambda nx, ny: 4 * nx * ny),
    ((10, 10), lambda nx, ny: 4 * nx * ny),
])
def test_r2r_roundtrip_scales_of_reference(orc, kinds, scale):
    # tests/python/test_r2r_kinds_py.py on a 17 x 23 grid
    nx, ny = 17, 23
    x = np.random.default_rng(0).uniform(-1, 1, (ny, nx))
    y = orc.forward_values(x, "r2r", kinds=list(kinds))
    z = orc.backward_values(y, "r2r", kinds=list(kinds))
    assert orc.r2r_roundtrip_scale([nx, ny], kinds) == scale(nx, ny)
    np.testing.assert_allclose(z / scale(nx, ny), x, atol=1e-10)


def test_roundtrip_threshold(orc):
    # 5 * log2(N) * (nearest(1,1) - nearest(1,-1))
    assert abs(orc.roundtrip_threshold(1024, True) - 5 * 10 * 1.5 * 2.0 ** -23) < 1e-12
    assert abs(orc.roundtrip_threshold(1024, False) - 5 * 10 * 1.5 * 2.0 ** -52) < 1e-20


def test_grid_choice(orc):
    # default single-process 3D plan on CUDA is Z-slab when nz >= 32
    assert orc.choose_grid(3, [64, 64, 64], 1) == ([1, 1, 1], True, False)
    assert orc.choose_grid(3, [64, 64, 16], 1) == ([1, 1, 1], False, False)
    assert orc.choose_grid(3, [512, 512, 512], 8) == ([1, 1, 8], True, False)
    assert orc.choose_grid(3, [512, 512, 512], 8, z_slab=False) == ([1, 1, 8], False, False)
    assert orc.choose_grid(3, [64, 64, 64], 8) == ([1, 4, 2], False, False)  # 64 / 8 < DEF_TILE_SIZE
    assert orc.choose_grid(3, [16, 16, 16], 8) == ([1, 4, 2], False, False)
    assert orc.choose_grid(3, [512, 512, 512], 8, cart=[1, 2, 4]) == ([1, 2, 4], False, False)
    assert orc.choose_grid(3, [512, 512, 512], 8, cart=[1, 1, 8]) == ([1, 1, 8], True, False)


def test_forward_backward_values_roundtrip(orc):
    rng = np.random.default_rng(3)
    g = rng.standard_normal((6, 5, 8))
    G = orc.forward_values(g, "r2c")
    assert G.shape == (6, 5, 5)
    np.testing.assert_allclose(orc.backward_values(G, "r2c", real_dims=[8, 5, 6]) / g.size, g, atol=1e-12)
    c = g + 1j * rng.standard_normal(g.shape)
    np.testing.assert_allclose(orc.backward_values(orc.forward_values(c, "c2c"), "c2c") / c.size, c, atol=1e-12)


def _ramp(n):
    return np.arange(1, n + 1, dtype=np.float32)


@pytest.mark.parametrize("dims", [[33, 77, 21], [90, 57]])
def test_reference_host_kernel_identities(orc, dims):
    """The known answers of the reference's host-kernel test
    (src/tests/test_host_kernels.F90:7-22, :26-236, :287-330) on its dims and
    ramp input: forward / backward permutes move element (x, y, z) to
    (y, z, x) / (z, x, y); backward_start followed by backward_end with the
    neighbour data {nz, nx, ny, 0, 0} equals the one-step backward permute;
    pack and unpack of a single full block are the identity."""
    import ctypes
    L = orc.lib()
    nd = len(dims)
    n = int(np.prod(dims))
    x = _ramp(n)
    out = np.full(n, -1, dtype=np.float32)
    ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    dv = (ctypes.c_int * 3)(*(dims + [1] * (3 - nd)))
    L.orc_permute_forward(ptr(x), ptr(out), nd, dv, 4)
    if nd == 3:
        nx, ny, nz = dims
        g = x.reshape(nz, ny, nx)
        np.testing.assert_array_equal(out, g.transpose(2, 0, 1).ravel())     # out[x][z][y]
        back = np.full(n, -1, dtype=np.float32)
        L.orc_permute_backward(ptr(x), ptr(back), dv, 4)
        np.testing.assert_array_equal(back, g.transpose(1, 2, 0).ravel())    # out[y][x][z]
        temp = np.full(n, -1, dtype=np.float32)
        L.orc_permute_backward_start(ptr(x), ptr(temp), dv, 4)
        np.testing.assert_array_equal(temp, g.transpose(2, 1, 0).ravel())    # out[x][y][z]
        tdims = [nz, nx, ny]
        two = np.full(n, -1, dtype=np.float32)
        L.orc_permute_backward_end_one(ptr(temp), ptr(two), (ctypes.c_int * 3)(*tdims),
                                       (ctypes.c_int * 5)(*(tdims + [0, 0])), 4)
        np.testing.assert_array_equal(two, back)
    else:
        nx, ny = dims
        np.testing.assert_array_equal(out, x.reshape(ny, nx).T.ravel())
    nb = (ctypes.c_int * 5)(*(dims + [1] * (3 - nd) + [0, 0]))
    for name in ("orc_unpack_one", "orc_pack_one"):
        cp = np.full(n, -1, dtype=np.float32)
        getattr(L, name)(ptr(x), ptr(cp), nd, dv, nb, 4)
        np.testing.assert_array_equal(cp, x)


@pytest.mark.parametrize("dims,grid", [([16, 12, 10], [1, 2, 2]), ([9, 14, 6], [1, 3, 2])])
def test_cpu_port_computes_the_transform(orc, dims, grid):
    """The timed CPU baseline (the reference arm of bench.py) runs the real
    schedule: its forward result is the 3D spectrum in the Z-pencil layout of
    the grid, and backward(forward(x)) / N returns x."""
    from oracle import cpu_execute
    rng = np.random.default_rng(4)
    g = (rng.uniform(-1, 1, dims[::-1]) + 1j * rng.uniform(-1, 1, dims[::-1])).astype(np.complex64)
    x = orc.global_to_packed(g, 3, grid, 1)
    plan = cpu_execute.CpuC2C(dims, grid)
    y = plan.forward(x)
    expect = orc.global_to_packed(orc.forward_values(g, "c2c"), 3, grid, 3)
    assert orc.rel_l2(y[:expect.size], expect) <= 1e-5
    back = plan.backward(y)[:x.size] / np.prod(dims)
    assert orc.rel_l2(back, x) <= 1e-5


@pytest.mark.parametrize("kind", ["c2c", "r2c", "r2r"])
def test_sampled_lines_equal_full_transform(orc, kind):
    """The separable line oracle used at full sizes equals the full FP64
    transform on every sampled line, for lines along each axis."""
    rng = np.random.default_rng(7)
    shape = (10, 12, 14)
    g = rng.standard_normal(shape) + (1j * rng.standard_normal(shape) if kind == "c2c" else 0)
    kinds = [orc.DCT_2, orc.DST_3, orc.DCT_4] if kind == "r2r" else None
    F = orc.forward_values(g, kind, kinds)          # [kz][ky][kx]
    nx_out = F.shape[2]
    for axis, pts in ((0, [(1, 2), (5, 9)]), (1, [(3, 4), (0, 7)]), (2, [(2, 11), (4, 0)])):
        lines = orc.sampled_lines(g, kind, axis, pts, kinds, chunk=3)
        for i, p in enumerate(pts):
            if axis == 0:
                ref = F[p[1], p[0], :]
            elif axis == 1:
                ref = F[p[1], :, p[0]]
            else:
                ref = F[:, p[1], p[0]]
            assert lines[i].shape == ref.shape
            np.testing.assert_allclose(lines[i], ref, rtol=0, atol=1e-12 * np.abs(F).max())
    assert nx_out == (8 if kind == "r2c" else 14)


def test_packed_index_matches_global_to_packed(orc):
    rng = np.random.default_rng(8)
    dims, grid = [10, 12, 14], [1, 2, 3]
    g = rng.standard_normal(tuple(dims[::-1]))
    co = np.stack(np.meshgrid(np.arange(10), np.arange(12), np.arange(14), indexing="ij"), -1).reshape(-1, 3)
    for lay in (1, 2, 3):
        p = orc.global_to_packed(g, 3, grid, lay)
        idx = orc.packed_index(3, dims, grid, lay, co)
        assert np.array_equal(p[idx], g[co[:, 2], co[:, 1], co[:, 0]])
    g2 = rng.standard_normal((9, 11))
    co2 = np.stack(np.meshgrid(np.arange(11), np.arange(9), indexing="ij"), -1).reshape(-1, 2)
    for lay in (1, 2):
        p = orc.global_to_packed(g2, 2, [1, 3], lay)
        idx = orc.packed_index(2, [11, 9], [1, 3], lay, co2)
        assert np.array_equal(p[idx], g2[co2[:, 1], co2[:, 0]])
