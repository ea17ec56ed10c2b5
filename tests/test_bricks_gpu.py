"""GPU parity of plans over user-defined blocks (dtfft_create_plan_*_pencil on
a dtfft_vgrid_pencils_create communicator), against the oracle's restatement
of the reference's decomposition (oracle/bricks.py):

* every layout of every virtual rank equals the oracle's box, at the offset
  the packed layout gives it;
* the four brick <-> pencil reshapes are bit-exact moves;
* transpose-only execute with bricks equals reshape + transposes, bit-exact;
* execute with FFTs equals the FP64 spectrum (rel-L2 <= 1e-5 single,
  <= 1e-12 double) and the backward pass returns N x the input.

The 8-rank case is the reference's tests/c/test_c2c_3d_c.c:105-136 (2x2x2
bricks of 96 x 64 x 512, Fourier reshape on)."""
import numpy as np
import pytest

from gpu_util import empty, from_dev, random_global, to_dev
from oracle import bricks as ob
from test_bricks import CONFIGS, CONFIGS_2D, grid_blocks, ref_test_blocks

pytestmark = pytest.mark.gpu

TOL = {"single": 1e-5, "double": 1e-12}


def _plan(dt, kind, blocks, prec, executor, fourier, z_slab=False):
    comm = dt.pencils_comm(blocks)
    cfg = dt.Config(enable_z_slab=z_slab, enable_y_slab=False, enable_fourier_reshape=fourier)
    pen = dt.Pencil(*blocks[0])
    p = dt.Precision.SINGLE if prec == "single" else dt.Precision.DOUBLE
    if kind == "c2c":
        return dt.PlanC2C(pen, comm=comm, precision=p, executor=executor, config=cfg)
    return dt.PlanR2C(pen, comm=comm, precision=p, executor=executor, config=cfg)


def _geom(blocks, r2c, fourier, z_slab=False):
    return ob.geometry([b[0] for b in blocks], [b[1] for b in blocks], r2c=r2c, z_slab=z_slab,
                       fourier_reshape=fourier)


LAYOUTS = {1: "xb", 3: "x", 4: "y", 5: "z", 6: "zb"}

CASES = [(b, d) for b, d in CONFIGS + CONFIGS_2D] + [("ref8", None)]


def _blocks(bgrid, dims):
    if bgrid == "ref8":
        return ref_test_blocks(8)
    return grid_blocks(bgrid, dims)


@pytest.mark.parametrize("bgrid,dims", CASES)
@pytest.mark.parametrize("kind", ["c2c", "r2c"])
@pytest.mark.parametrize("fourier", [False, True])
def test_layouts_match_oracle(dt, cuda, bgrid, dims, kind, fourier):
    blocks = _blocks(bgrid, dims)
    nd = len(blocks[0][0])
    g = _geom(blocks, kind == "r2c", fourier)
    plan = _plan(dt, kind, blocks, "single", dt.Executor.NONE, fourier)
    assert plan.grid_dims == g["grid"]
    assert plan.dims == g["dims"]
    P = len(blocks)
    assert plan.nranks == P
    for lay, name in LAYOUTS.items():
        if name in ("xb", "zb") and not g["reshape"]:
            continue
        if name == "z" and nd == 2:
            continue
        ref = g[name]
        if lay == 3 and kind == "c2c":
            continue
        off = 0
        for r in range(P):
            pen, o = plan.vrank_pencil(dt.Layout(lay), r)
            assert (pen.starts, pen.counts) == (list(ref[r][0]), list(ref[r][1])), (name, r)
            assert o == off, (name, r)
            off += int(np.prod(ref[r][1]))
    # X pencils in real space
    ref = g["xr"] if kind == "r2c" else g["x"]
    for r in range(P):
        pen, _ = plan.vrank_pencil(dt.Layout.X_PENCILS, r)
        assert (pen.starts, pen.counts) == (list(ref[r][0]), list(ref[r][1]))
    plan.destroy()


def _bytes(a):
    return np.ascontiguousarray(a).view(np.uint8).tobytes()


@pytest.mark.parametrize("bgrid,dims", [c for c in CASES if c[0] == "ref8" or c[0][0] > 1])
@pytest.mark.parametrize("np_dtype", [np.complex64, np.complex128])
def test_reshapes_bit_exact(dt, cuda, bgrid, dims, np_dtype):
    blocks = _blocks(bgrid, dims)
    nd = len(blocks[0][0])
    g = _geom(blocks, False, True)
    prec = "single" if np_dtype == np.complex64 else "double"
    plan = _plan(dt, "c2c", blocks, prec, dt.Executor.NONE, True)
    assert plan.get_pencil(dt.Layout.X_BRICKS).ndims == nd
    gd = g["dims"]
    arr = random_global(tuple(gd[::-1]), np_dtype, seed=sum(gd))
    n_alloc = plan.alloc_size
    moves = [(dt.Reshape.X_BRICKS_TO_PENCILS, ("xb", 1), ("x", 1)),
             (dt.Reshape.X_PENCILS_TO_BRICKS, ("x", 1), ("xb", 1)),
             (dt.Reshape.Z_PENCILS_TO_BRICKS, ("z" if nd == 3 else "y", nd), ("zb", nd)),
             (dt.Reshape.Z_BRICKS_TO_PENCILS, ("zb", nd), ("z" if nd == 3 else "y", nd))]
    for rt, (src, sa), (dst, da) in moves:
        pin = ob.pack(arr, g[src], sa)
        expect = ob.pack(arr, g[dst], da)
        a = to_dev(pin, n_alloc, cuda)
        b = empty(n_alloc, np_dtype, cuda)
        if rt == dt.Reshape.X_BRICKS_TO_PENCILS:
            req = plan.reshape_start(a, b, rt)
            plan.reshape_end(req)
        else:
            plan.reshape(a, b, rt)
        assert _bytes(from_dev(b, expect.size, np_dtype)) == _bytes(expect), rt
    plan.destroy()


@pytest.mark.parametrize("bgrid,dims", [c for c in CASES if c[0] == "ref8" or c[0][0] > 1])
@pytest.mark.parametrize("fourier", [False, True])
def test_transpose_only_execute_with_bricks(dt, cuda, bgrid, dims, fourier):
    blocks = _blocks(bgrid, dims)
    nd = len(blocks[0][0])
    g = _geom(blocks, False, fourier)
    plan = _plan(dt, "c2c", blocks, "double", dt.Executor.NONE, fourier)
    gd = g["dims"]
    arr = random_global(tuple(gd[::-1]), np.complex128, seed=3)
    n_alloc = plan.alloc_size
    last = ("zb", nd) if g["final_reshape"] else (("z", 3) if nd == 3 else ("y", 2))
    a = to_dev(ob.pack(arr, g["xb"], 1), n_alloc, cuda)
    b = empty(n_alloc, np.complex128, cuda)
    plan.execute(a, b, dt.Execute.FORWARD)
    expect = ob.pack(arr, g[last[0]], last[1])
    assert _bytes(from_dev(b, expect.size, np.complex128)) == _bytes(expect)
    c = empty(n_alloc, np.complex128, cuda)
    plan.execute(b, c, dt.Execute.BACKWARD)
    expect = ob.pack(arr, g["xb"], 1)
    assert _bytes(from_dev(c, expect.size, np.complex128)) == _bytes(expect)
    plan.destroy()


FFT_CASES = [("ref8", None, "c2c", "single", True), ((2, 2, 2), [33, 17, 40], "c2c", "double", False),
             ((2, 2, 2), [33, 17, 40], "c2c", "single", True), ((4, 1, 2), [40, 30, 20], "r2c", "double", True),
             ((2, 3, 1), [12, 9, 200], "r2c", "single", False), ((2, 2), [40, 36], "c2c", "double", True),
             ((3, 1), [25, 70], "r2c", "double", True)]


@pytest.mark.parametrize("bgrid,dims,kind,prec,fourier", FFT_CASES)
def test_execute_with_bricks_matches_fp64(dt, orc, cuda, bgrid, dims, kind, prec, fourier):
    blocks = _blocks(bgrid, dims)
    nd = len(blocks[0][0])
    g = _geom(blocks, kind == "r2c", fourier)
    plan = _plan(dt, kind, blocks, prec, dt.Executor.CUFFT, fourier)
    gd = g["dims"]
    cdt = np.complex64 if prec == "single" else np.complex128
    rdt = np.float32 if prec == "single" else np.float64
    in_dt = cdt if kind == "c2c" else rdt
    arr = random_global(tuple(gd[::-1]), in_dt, seed=11)
    G = orc.forward_values(arr, kind)
    n_alloc = plan.alloc_size
    last = ("zb", nd) if g["final_reshape"] else (("z", 3) if nd == 3 else ("y", 2))
    a = to_dev(ob.pack(arr, g["xb"], 1), n_alloc, cuda)
    b = empty(n_alloc if kind == "c2c" else n_alloc // 2, cdt, cuda)
    plan.execute(a, b, dt.Execute.FORWARD)
    expect = ob.pack(G, g[last[0]], last[1])
    got = from_dev(b, expect.size, cdt)
    assert orc.rel_l2(got, expect) <= TOL[prec]
    c = empty(n_alloc, in_dt, cuda)
    plan.execute(b, c, dt.Execute.BACKWARD)
    n = int(np.prod(gd))
    back = from_dev(c, arr.size, in_dt)
    assert orc.rel_l2(back / n, ob.pack(arr, g["xb"], 1)) <= TOL[prec]
    plan.destroy()


def test_reshape_errors(dt, cuda):
    import torch
    blocks = grid_blocks((1, 2, 2), [16, 16, 16])          # X not split: no reshape
    plan = _plan(dt, "c2c", blocks, "single", dt.Executor.NONE, False)
    a = torch.zeros(plan.alloc_size, dtype=torch.complex64, device=cuda)
    b = torch.zeros_like(a)
    with pytest.raises(dt.DtfftError) as e:
        plan.reshape(a, b, dt.Reshape.X_BRICKS_TO_PENCILS)
    assert e.value.code == 44                               # RESHAPE_NOT_SUPPORTED
    plan.destroy()
    blocks = grid_blocks((2, 2, 1), [16, 16, 16])
    plan = _plan(dt, "c2c", blocks, "single", dt.Executor.NONE, False)
    with pytest.raises(dt.DtfftError) as e:
        plan.reshape(a, a, dt.Reshape.X_BRICKS_TO_PENCILS)
    assert e.value.code == 41                               # INPLACE_RESHAPE
    with pytest.raises(dt.DtfftError) as e:
        plan.reshape(a, b, 10)
    assert e.value.code == 38                               # INVALID_RESHAPE_TYPE
    with pytest.raises(dt.DtfftError) as e:
        plan.execute(a, a, dt.Execute.FORWARD)              # transpose-only in place, no final reshape
    assert e.value.code == 14                               # INPLACE_TRANSPOSE
    plan.destroy()
