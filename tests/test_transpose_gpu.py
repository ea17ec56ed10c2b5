"""GPU parity of the data movement: every transpose of the virtual grid, run
through the dtfft_* C ABI, must equal the oracle's restatement of the
reference's pack -> all-to-all-v -> unpack bit for bit; the kernel plug-in
(gb_kernel_*) must equal the reference's host kernels, on the shapes of
src/tests/test_device_kernels.F90 ([18,155] and [18,33,155])."""
import ctypes

import numpy as np
import pytest

from gpu_util import comm_for, empty, from_dev, random_global, to_dev

pytestmark = pytest.mark.gpu

CASES = [
    ([18, 33, 155], [1, 1, 1]),
    ([18, 33, 155], [1, 2, 3]),
    ([17, 10, 9], [1, 3, 2]),
    ([16, 8, 40], [1, 1, 4]),       # Z-slab grid: X<->Z transposes too
    ([5, 7, 9], [1, 4, 4]),
    ([3, 7, 9], [1, 4, 4]),         # some ranks hold nothing
    ([64, 48, 32], [1, 2, 4]),
    ([130, 66, 33], [1, 2, 2]),
    ([18, 155], [1, 1]),
    ([17, 23], [1, 3]),
    ([3, 5], [1, 4]),
    ([200, 129], [1, 2]),
]

DTYPES = [("f32", np.float32), ("c64", np.complex64), ("c128", np.complex128), ("f64", np.float64)]


def _plan(dt, dims, grid, np_dtype):
    comm = comm_for(dt, grid)
    cfg = dt.Config(enable_z_slab=True)
    if np_dtype in (np.float32, np.float64):
        prec = dt.Precision.SINGLE if np_dtype == np.float32 else dt.Precision.DOUBLE
        return dt.PlanR2R(dims, comm=comm, precision=prec, config=cfg)
    prec = dt.Precision.SINGLE if np_dtype == np.complex64 else dt.Precision.DOUBLE
    return dt.PlanC2C(dims, comm=comm, precision=prec, config=cfg)


@pytest.mark.parametrize("dims,grid", CASES)
@pytest.mark.parametrize("name,np_dtype", DTYPES)
def test_transposes_bit_exact(dt, orc, cuda, dims, grid, name, np_dtype):
    nd = len(dims)
    plan = _plan(dt, dims, grid, np_dtype)
    assert plan.grid_dims == list(grid)
    g = random_global(tuple(dims[::-1]), np_dtype, seed=sum(dims) + len(name))
    types = [1, -1] if nd == 2 else [1, -1, 2, -2] + ([3, -3] if plan.z_slab_enabled else [])
    n_alloc = plan.alloc_size
    for t in types:
        sl = {1: 1, -1: 2, 2: 2, -2: 3, 3: 1, -3: 3}[t]
        pin = orc.global_to_packed(g, nd, grid, sl)
        expect = orc.vgrid_transpose(nd, dims, grid, t, pin)
        a = to_dev(pin, n_alloc, cuda)
        b = empty(n_alloc, np_dtype, cuda)
        plan.transpose(a, b, dt.Transpose(t))
        out = from_dev(b, expect.size, np_dtype)
        assert out.view(np.uint8).tobytes() == expect.view(np.uint8).tobytes(), f"transpose {t}"
    plan.destroy()


@pytest.mark.parametrize("dims,grid", [([18, 33, 155], [1, 2, 3]), ([16, 8, 40], [1, 1, 4]), ([17, 23], [1, 3]),
                                       ([40, 36, 34], [1, 1, 1])])
def test_transpose_only_execute_cycle(dt, orc, cuda, dims, grid):
    """execute() of a transpose-only plan runs the reference's schedule
    (src/dtfft_plan.F90:877-1101): forward ends in the last layout, backward restores X."""
    nd = len(dims)
    plan = _plan(dt, dims, grid, np.complex64)
    g = random_global(tuple(dims[::-1]), np.complex64, seed=5)
    pin = orc.global_to_packed(g, nd, grid, 1)
    last = 2 if nd == 2 else 3
    expect = orc.global_to_packed(g, nd, grid, last)
    a = to_dev(pin, plan.alloc_size, cuda)
    b = empty(plan.alloc_size, np.complex64, cuda)
    plan.execute(a, b, dt.Execute.FORWARD)
    assert np.array_equal(from_dev(b, expect.size, np.complex64), expect)
    c = empty(plan.alloc_size, np.complex64, cuda)
    plan.execute(b, c, dt.Execute.BACKWARD)
    assert np.array_equal(from_dev(c, pin.size, np.complex64), pin)
    plan.destroy()


def test_large_virtual_grid_cycle(dt, orc, cuda):
    """The 2x4 grid of the headline workload, at a size the oracle finishes in seconds."""
    dims, grid = [128, 96, 80], [1, 2, 4]
    plan = _plan(dt, dims, grid, np.complex64)
    g = random_global(tuple(dims[::-1]), np.complex64, seed=11)
    x = orc.global_to_packed(g, 3, grid, 1)
    a = to_dev(x, plan.alloc_size, cuda)
    b = empty(plan.alloc_size, np.complex64, cuda)
    c = empty(plan.alloc_size, np.complex64, cuda)
    plan.transpose(a, b, dt.Transpose.X_TO_Y)
    y = orc.vgrid_transpose(3, dims, grid, 1, x)
    assert np.array_equal(from_dev(b, y.size, np.complex64), y)
    plan.transpose(b, c, dt.Transpose.Y_TO_Z)
    z = orc.vgrid_transpose(3, dims, grid, 2, y)
    assert np.array_equal(from_dev(c, z.size, np.complex64), z)
    plan.destroy()


def test_transpose_errors(dt, cuda):
    import torch
    plan = dt.PlanC2C([16, 8, 40], precision=dt.Precision.SINGLE)
    a = torch.zeros(plan.alloc_size, dtype=torch.complex64, device=cuda)
    b = torch.zeros_like(a)
    with pytest.raises(dt.DtfftError) as e:
        plan.transpose(a, a, dt.Transpose.X_TO_Y)
    assert e.value.code == 14
    h = torch.zeros(plan.alloc_size, dtype=torch.complex64)
    with pytest.raises(dt.DtfftError) as e:
        plan.transpose(h, b, dt.Transpose.X_TO_Y)
    assert e.value.code == 300
    with pytest.raises(dt.DtfftError) as e:
        plan.transpose(a, b, 7)
    assert e.value.code == 2
    with pytest.raises(dt.DtfftError) as e:
        plan.execute(a, b, dt.Execute.FORWARD, aux=a)
    assert e.value.code == 15
    plan.destroy()
    plan2 = dt.PlanC2C([16, 8], precision=dt.Precision.SINGLE)
    with pytest.raises(dt.DtfftError) as e:
        plan2.transpose(a, b, dt.Transpose.Y_TO_Z)
    assert e.value.code == 2
    plan2.destroy()


def test_local_sizes_and_pencils(dt, orc, cuda):
    dims, grid = [30, 20, 10], [1, 2, 3]
    plan = dt.PlanC2C(dims, comm=dt.cart_comm(grid), precision=dt.Precision.SINGLE)
    assert plan.nranks == 6
    for layout, lid in ((dt.Layout.X_PENCILS, 1), (dt.Layout.Y_PENCILS, 2), (dt.Layout.Z_PENCILS, 3)):
        for r in range(6):
            p, off = plan.vrank_pencil(layout, r)
            s, c = orc.pencil(3, dims, grid, lid, r)
            assert p.starts == s and p.counts == c
            assert off == orc.rank_offset(3, dims, grid, lid, r)
    assert plan.alloc_size == 30 * 20 * 10
    assert plan.element_size == 8
    assert plan.aux_bytes == plan.alloc_bytes
    plan.destroy()
    one = dt.PlanC2C([64, 64, 64], precision=dt.Precision.DOUBLE)
    assert one.z_slab_enabled and one.grid_dims == [1, 1, 1]
    ins, inc, outs, outc, al = one.local_sizes
    assert inc == [64, 64, 64] and outc == [64, 64, 64] and al == 64 ** 3
    assert one.element_size == 16
    one.destroy()


# ---- kernel plug-in, shapes of src/tests/test_device_kernels.F90 -------------

def _kernel(dt, dims, ktype, es, nbr=None):
    L = dt.lib()
    h = ctypes.c_void_p()
    d = (ctypes.c_int32 * 3)(*(list(dims) + [1] * (3 - len(dims))))
    if nbr is None:
        rc = L.gb_kernel_create(len(dims), d, es, ktype, None, 0, 0, ctypes.byref(h))
    else:
        arr = (ctypes.c_int32 * len(nbr))(*nbr)
        rc = L.gb_kernel_create(len(dims), d, es, ktype, arr, len(nbr) // 5, 0, ctypes.byref(h))
    assert rc == 0, rc
    return h


@pytest.mark.parametrize("dims", [[18, 155], [18, 33, 155]])
@pytest.mark.parametrize("ktype", [7, 8, 9, 1, 3, 10])
def test_kernel_plugin_vs_host_kernels(dt, orc, cuda, dims, ktype):
    import torch
    nd = len(dims)
    if nd == 2 and ktype in (9, 10):
        pytest.skip("two-step permute is 3D only")
    es = 4
    n = int(np.prod(dims))
    rng = np.random.default_rng(ktype)
    x = (rng.random(n).astype(np.float32) * np.arange(1, n + 1, dtype=np.float32))
    # full-box neighbour data, as the reference test builds it: locals(1:3) = dims, displs 0
    nbr = list(dims) + [1] * (3 - nd) + [0, 0]
    L = orc.lib()
    dims_c = (ctypes.c_int * 3)(*(list(dims) + [1] * (3 - nd)))
    nb_c = (ctypes.c_int * 5)(*nbr)
    gold = np.zeros(n, np.float32)
    xp, gp = x.ctypes.data, gold.ctypes.data
    if ktype == 7:
        L.orc_permute_forward(xp, gp, nd, dims_c, es)
    elif ktype == 8:
        if nd == 2:
            L.orc_permute_forward(xp, gp, nd, dims_c, es)
        else:
            L.orc_permute_backward(xp, gp, dims_c, es)
    elif ktype == 9:
        L.orc_permute_backward_start(xp, gp, dims_c, es)
    elif ktype == 10:
        L.orc_permute_backward_end_one(xp, gp, dims_c, nb_c, es)
    elif ktype == 1:
        L.orc_pack_one(xp, gp, nd, dims_c, nb_c, es)
    elif ktype == 3:
        L.orc_unpack_one(xp, gp, nd, dims_c, nb_c, es)
    h = _kernel(dt, dims, ktype, es, nbr if ktype in (1, 3, 10) else None)
    a = torch.from_numpy(x).to(cuda)
    b = torch.zeros(n, dtype=torch.float32, device=cuda)
    assert dt.lib().gb_kernel_execute(h, a.data_ptr(), b.data_ptr(), None, 1) == 0
    torch.cuda.synchronize()
    assert np.array_equal(b.cpu().numpy(), gold)
    assert dt.lib().gb_kernel_destroy(ctypes.byref(h)) == 0


def test_kernel_plugin_pipelined_unpack(dt, orc, cuda):
    """UNPACK_PIPELINED moves one neighbour's block (1-based neighbour index)."""
    import torch
    dims = [20, 6, 4]
    # two neighbours: x in [0,8) and [8,20), packed one after the other
    nbr = [8, 6, 4, 0, 0, 12, 6, 4, 8 * 6 * 4, 8]
    n = 20 * 6 * 4
    x = np.arange(n, dtype=np.float32)
    L = orc.lib()
    dims_c = (ctypes.c_int * 3)(*dims)
    gold = np.zeros(n, np.float32)
    for k in range(2):
        L.orc_unpack_one(x.ctypes.data, gold.ctypes.data, 3, dims_c, (ctypes.c_int * 5)(*nbr[5 * k:5 * k + 5]), 4)
    h = _kernel(dt, dims, 5, 4, nbr)
    a = torch.from_numpy(x).to(cuda)
    b = torch.zeros(n, dtype=torch.float32, device=cuda)
    for k in (1, 2):
        assert dt.lib().gb_kernel_execute(h, a.data_ptr(), b.data_ptr(), None, k) == 0
    torch.cuda.synchronize()
    assert np.array_equal(b.cpu().numpy(), gold)
    dt.lib().gb_kernel_destroy(ctypes.byref(h))
