"""Public entry points beyond execute/transpose, through the C ABI:

- dtfft_transpose_start / dtfft_transpose_end (src/dtfft_plan.F90:599-693):
  every transpose of a virtual grid bit-exact against the oracle, and the
  request errors;
- dtfft_mem_alloc / dtfft_mem_free (src/dtfft_plan.F90:2655-2717): buffers
  from the plan drive a full execute, and the argument errors;
- the Y-slab schedule forward and backward (src/dtfft_plan.F90:839-1016 with
  is_y_slab), C2C and R2C, one process and a 2-rank grid;
- dtfft_get_pencil (src/dtfft_plan.F90:1286-1336) against the oracle's
  pencil rule (src/dtfft_pencil.F90:237-279) for every layout;
- the failure path of the bounded waits: kernels whose waits give up record
  it, the next public call returns DTFFT_ERROR_GPU_WAIT_TIMEOUT once, and the
  plan then runs correctly again.
"""
import ctypes

import numpy as np
import pytest

from gpu_util import comm_for, empty, from_dev, random_global, to_dev

pytestmark = pytest.mark.gpu


# ---- transpose_start / transpose_end ---------------------------------------

@pytest.mark.parametrize("dims,grid,np_dtype", [
    ([64, 48, 40], [1, 2, 2], np.complex64),
    ([18, 33, 155], [1, 2, 3], np.complex128),
    ([30, 20, 16], [1, 1, 4], np.float32),       # Z-slab grid: X<->Z too
    ([17, 23], [1, 3], np.complex64),
])
def test_transpose_start_end_bit_exact(dt, orc, cuda, dims, grid, np_dtype):
    nd = len(dims)
    comm = comm_for(dt, grid)
    cfg = dt.Config(enable_z_slab=True)
    if np_dtype == np.float32:
        plan = dt.PlanR2R(dims, comm=comm, precision=dt.Precision.SINGLE, config=cfg)
    else:
        prec = dt.Precision.SINGLE if np_dtype == np.complex64 else dt.Precision.DOUBLE
        plan = dt.PlanC2C(dims, comm=comm, precision=prec, config=cfg)
    g = random_global(tuple(dims[::-1]), np_dtype, seed=21)
    types = [1, -1] if nd == 2 else [1, -1, 2, -2] + ([3, -3] if plan.z_slab_enabled else [])
    for t in types:
        sl = {1: 1, -1: 2, 2: 2, -2: 3, 3: 1, -3: 3}[t]
        pin = orc.global_to_packed(g, nd, grid, sl)
        expect = orc.vgrid_transpose(nd, dims, grid, t, pin)
        a = to_dev(pin, plan.alloc_size, cuda)
        b = empty(plan.alloc_size, np_dtype, cuda)
        req = plan.transpose_start(a, b, dt.Transpose(t))
        plan.transpose_end(req)
        out = from_dev(b, expect.size, np_dtype)
        assert out.view(np.uint8).tobytes() == expect.view(np.uint8).tobytes(), f"transpose {t}"
        # a finished request is no longer valid
        with pytest.raises(dt.DtfftError) as e:
            plan.transpose_end(req)
        assert e.value.code == 35
    plan.destroy()


def test_transpose_start_errors(dt, cuda):
    import torch
    plan = dt.PlanC2C([16, 8, 40], precision=dt.Precision.SINGLE)
    a = torch.zeros(plan.alloc_size, dtype=torch.complex64, device=cuda)
    b = torch.zeros_like(a)
    with pytest.raises(dt.DtfftError) as e:
        plan.transpose_start(a, a, dt.Transpose.X_TO_Y)
    assert e.value.code == 14                      # DTFFT_ERROR_INPLACE_TRANSPOSE
    with pytest.raises(dt.DtfftError) as e:
        plan.transpose_start(a, b, 5)
    assert e.value.code == 2                       # DTFFT_ERROR_INVALID_TRANSPOSE_TYPE
    with pytest.raises(dt.DtfftError) as e:
        plan.transpose_end(ctypes.c_void_p(None))
    assert e.value.code == 35                      # DTFFT_ERROR_INVALID_REQUEST
    L = dt.lib()
    assert L.dtfft_transpose_start(plan._h, a.data_ptr(), b.data_ptr(), 1, None, None) == 17
    plan.destroy()


# ---- mem_alloc / mem_free ----------------------------------------------------

class _DevBuf:
    """A device pointer seen by torch through __cuda_array_interface__."""

    def __init__(self, ptr, n, typestr):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False), "version": 3,
                                         "strides": None}


@pytest.mark.parametrize("kind", ["c2c", "r2c"])
def test_mem_alloc_buffers_drive_execute(dt, orc, cuda, kind):
    import torch
    L = dt.lib()
    dims, grid = [40, 36, 32], [1, 2, 2]
    if kind == "c2c":
        plan = dt.PlanC2C(dims, comm=dt.cart_comm(grid), precision=dt.Precision.SINGLE, executor=dt.Executor.CUFFT)
        rdt, cdt = np.complex64, np.complex64
    else:
        plan = dt.PlanR2C(dims, comm=dt.cart_comm(grid), precision=dt.Precision.SINGLE, executor=dt.Executor.CUFFT)
        rdt, cdt = np.float32, np.complex64
    ptrs = []
    for nbytes in (plan.alloc_bytes, plan.alloc_bytes, plan.aux_bytes):
        p = ctypes.c_void_p()
        assert L.dtfft_mem_alloc(plan._h, nbytes, ctypes.byref(p)) == 0
        assert p.value
        ptrs.append(p.value)
    n_real = plan.alloc_bytes // np.dtype(rdt).itemsize
    n_cplx = plan.alloc_bytes // np.dtype(cdt).itemsize
    ts = {np.complex64: "<c8", np.float32: "<f4"}
    a = torch.as_tensor(_DevBuf(ptrs[0], n_real, ts[rdt]), device=cuda)
    b = torch.as_tensor(_DevBuf(ptrs[1], n_cplx, ts[cdt]), device=cuda)
    g = random_global(tuple(dims[::-1]), rdt, seed=8, dist="normal")
    x = orc.global_to_packed(g, 3, grid, 1)
    a.zero_()
    a[: x.size] = torch.from_numpy(x).to(cuda)
    torch.cuda.synchronize()
    plan.execute(a, b, dt.Execute.FORWARD, aux=ptrs[2])
    expect = orc.global_to_packed(orc.forward_values(g, kind), 3, grid, 3)
    assert orc.rel_l2(from_dev(b, expect.size, cdt), expect) <= 1e-5
    plan.execute(b, a, dt.Execute.BACKWARD, aux=ptrs[2])
    back = from_dev(a, x.size, rdt).astype(np.complex128) / np.prod(dims)
    assert orc.rel_l2(back, x) <= 1e-5
    del a, b
    for p in ptrs:
        assert L.dtfft_mem_free(plan._h, p) == 0
    # argument errors of mem_alloc_ptr (src/dtfft_plan.F90:2667-2671)
    p = ctypes.c_void_p()
    assert L.dtfft_mem_alloc(plan._h, 2, ctypes.byref(p)) == 21     # DTFFT_ERROR_INVALID_ALLOC_BYTES
    assert L.dtfft_mem_alloc(plan._h, 64, None) == 17                # DTFFT_ERROR_INVALID_USAGE
    assert L.dtfft_mem_alloc(None, 64, ctypes.byref(p)) == 1         # DTFFT_ERROR_PLAN_NOT_CREATED
    plan.destroy()


# ---- Y-slab schedule ---------------------------------------------------------

@pytest.mark.parametrize("dims,grid,kind,np_dtype", [
    ([48, 40, 36], [1, 1, 1], "c2c", np.complex64),
    ([64, 48, 20], [1, 2, 1], "c2c", np.complex128),
    ([64, 36, 24], [1, 1, 1], "r2c", np.float32),
    ([34, 32, 18], [1, 2, 1], "r2c", np.float64),
])
def test_y_slab_forward_backward(dt, orc, cuda, dims, grid, kind, np_dtype):
    cfg = dt.Config(enable_z_slab=False, enable_y_slab=True)
    comm = comm_for(dt, grid)
    single = np_dtype in (np.complex64, np.float32)
    prec = dt.Precision.SINGLE if single else dt.Precision.DOUBLE
    if kind == "c2c":
        plan = dt.PlanC2C(dims, comm=comm, precision=prec, executor=dt.Executor.VKFFT, config=cfg)
        cdt = np_dtype
    else:
        plan = dt.PlanR2C(dims, comm=comm, precision=prec, executor=dt.Executor.VKFFT, config=cfg)
        cdt = np.complex64 if single else np.complex128
    dt.set_config(dt.Config())
    assert plan.y_slab_enabled and not plan.z_slab_enabled
    g = random_global(tuple(dims[::-1]), np_dtype, seed=17, dist="normal")
    x = orc.global_to_packed(g, 3, grid, 1)
    a = to_dev(x, plan.alloc_size, cuda)
    b = empty(plan.alloc_size, cdt, cuda)
    plan.execute(a, b, dt.Execute.FORWARD)
    # forward ends in Y pencils for a Y-slab plan
    expect = orc.global_to_packed(orc.forward_values(g, kind), 3, grid, 2)
    tol = 1e-5 if single else 1e-12
    assert orc.rel_l2(from_dev(b, expect.size, cdt), expect) <= tol
    c = empty(plan.alloc_size, np_dtype, cuda)
    plan.execute(b, c, dt.Execute.BACKWARD)
    back = from_dev(c, x.size, np_dtype).astype(np.complex128) / np.prod(dims)
    assert orc.rel_l2(back, x) <= tol
    plan.destroy()


# ---- get_pencil --------------------------------------------------------------

@pytest.mark.parametrize("dims,kind", [([30, 20, 10], "c2c"), ([33, 20, 12], "r2c"), ([24, 18], "c2c"),
                                       ([26, 14], "r2c")])
def test_get_pencil_matches_oracle(dt, orc, cuda, dims, kind):
    nd = len(dims)
    if kind == "c2c":
        plan = dt.PlanC2C(dims, precision=dt.Precision.SINGLE)
    else:
        plan = dt.PlanR2C(dims, precision=dt.Precision.SINGLE, executor=dt.Executor.CUFFT)
    one = [1] * nd
    cdims = [dims[0] // 2 + 1] + list(dims[1:]) if kind == "r2c" else list(dims)
    layouts = [(dt.Layout.X_PENCILS, 1, dims), (dt.Layout.Y_PENCILS, 2, cdims)]
    if nd == 3:
        layouts.append((dt.Layout.Z_PENCILS, 3, cdims))
    if kind == "r2c":
        layouts.append((dt.Layout.X_PENCILS_FOURIER, 1, cdims))
    for layout, lid, gd in layouts:
        p = plan.get_pencil(layout)
        s, c = orc.pencil(nd, gd, one, lid, 0)
        assert (p.dim, p.ndims, p.starts, p.counts, p.size) == (lid, nd, s, c, int(np.prod(c))), layout
    # layouts the plan does not have
    bad = [dt.Layout.X_BRICKS, dt.Layout.Z_BRICKS] + ([dt.Layout.Z_PENCILS] if nd == 2 else []) + \
          ([dt.Layout.X_PENCILS_FOURIER] if kind == "c2c" else [])
    for layout in bad:
        with pytest.raises(dt.DtfftError) as e:
            plan.get_pencil(layout)
        assert e.value.code == 16                  # DTFFT_ERROR_INVALID_LAYOUT
    with pytest.raises(dt.DtfftError) as e:
        plan.get_pencil(9)
    assert e.value.code == 16
    plan.destroy()


# ---- failure path of the bounded waits ---------------------------------------

def test_wait_timeout_is_reported_once_then_clean(dt, orc, cuda):
    """With a wait limit of 0 the tile FFT kernels (fused X pass, plain Z rows)
    and the TMA transpose give up at once: they record the timeout, wait for
    the copies they issued and return.  The status is read without a device
    synchronisation by the next public call, which returns
    DTFFT_ERROR_GPU_WAIT_TIMEOUT (603) once; the plan then runs correctly."""
    dims, grid = [256, 32, 256], [1, 2, 2]
    plan = dt.PlanC2C(dims, comm=dt.cart_comm(grid), precision=dt.Precision.SINGLE, executor=dt.Executor.CUFFT)
    g = random_global(tuple(dims[::-1]), np.complex64, seed=31)
    x = orc.global_to_packed(g, 3, grid, 1)
    expect = orc.global_to_packed(orc.forward_values(g, "c2c"), 3, grid, 3)
    expect_y = orc.vgrid_transpose(3, dims, grid, 1, x)
    assert dt.device_status(reset=True) == 0

    def run_execute():
        plan.execute(to_dev(x, plan.alloc_size, cuda), empty(plan.alloc_size, np.complex64, cuda),
                     dt.Execute.FORWARD)

    def run_transpose():
        plan.transpose(to_dev(x, plan.alloc_size, cuda), empty(plan.alloc_size, np.complex64, cuda),
                       dt.Transpose.X_TO_Y)

    for run, code in ((run_execute, 1), (run_transpose, 3)):
        dt.set_wait_limit(0)
        try:
            run()
        finally:
            dt.set_wait_limit(dt.WAIT_LIMIT_DEFAULT)
        # device_status synchronises and sees the code (kept: no reset)
        assert dt.device_status() == code
        with pytest.raises(dt.DtfftError) as e:
            run()
        assert e.value.code == 603
        # reported once: the word is clear again
        assert dt.device_status() == 0
    # the plan runs correctly afterwards
    a = to_dev(x, plan.alloc_size, cuda)
    b = empty(plan.alloc_size, np.complex64, cuda)
    plan.execute(a, b, dt.Execute.FORWARD)
    assert orc.rel_l2(from_dev(b, expect.size, np.complex64), expect) <= 1e-5
    a = to_dev(x, plan.alloc_size, cuda)
    plan.transpose(a, b, dt.Transpose.X_TO_Y)
    assert np.array_equal(from_dev(b, expect_y.size, np.complex64), expect_y)
    assert dt.device_status() == 0
    with pytest.raises(dt.DtfftError):
        dt.set_wait_limit(-1)
    plan.destroy()
