"""GPU parity of the FFT path: dtfft_execute through the C ABI against the
FP64 oracle (FFTW conventions).

Tolerances (relative L2 against the FP64 oracle): 1e-5 for single precision,
1e-12 for double precision.  Round trips (forward, scale by 1/N, backward) are
also held to the reference's max-abs threshold 5*log2(N)*eps
(tests/test_utils.F90:89-109), with the scale conventions of
tests/python/test_r2r_kinds_py.py for R2R kinds."""
import ctypes

import numpy as np
import pytest

from gpu_util import comm_for, empty, from_dev, random_global, to_dev

pytestmark = pytest.mark.gpu

TOL = {np.complex64: 1e-5, np.complex128: 1e-12, np.float32: 1e-5, np.float64: 1e-12}


def _prec(dt, np_dtype):
    return dt.Precision.SINGLE if np_dtype in (np.complex64, np.float32) else dt.Precision.DOUBLE


def _final_layout(plan, nd):
    return 2 if (nd == 2 or plan.y_slab_enabled) else 3


C2C_CASES = [
    ([256, 256], [1, 1], np.complex128),            # 2D C2C c128 256x256, one process
    ([64, 48, 40], [1, 2, 4], np.complex64),         # 2x4 grid, generic schedule
    ([60, 45, 42], [1, 1, 1], np.complex64),         # Z-slab, radices 3/5/7
    ([17, 23, 11], [1, 1, 1], np.complex64),         # odd primes (generic schedule, nz < 32)
    ([48, 36, 40], [1, 3, 2], np.complex128),
    ([96, 80, 64], [1, 1, 4], np.complex64),         # Z-slab on 4 ranks
    ([31, 44], [1, 3], np.complex64),
    ([512, 24], [1, 1], np.complex64),
    # tile-kernel row lengths with a ragged last tile (rows % 16 != 0)
    ([512, 7, 3], [1, 1, 1], np.complex64),
    ([1024, 5, 3], [1, 1, 1], np.complex64),
    ([768, 9, 2], [1, 1, 2], np.complex64),
    ([256, 256, 3], [1, 1, 1], np.complex128),
    ([512, 3, 5], [1, 1, 1], np.complex128),
    ([48, 320, 288], [1, 1, 1], np.complex64),       # Z-slab plan on the fused generic route
    ([120, 7, 3], [1, 1, 1], np.complex64),          # runtime-schedule rows, ragged last tile
    ([50, 90, 13], [1, 2, 1], np.complex64),
]


@pytest.mark.parametrize("dims,grid,np_dtype", C2C_CASES)
def test_c2c_forward_backward(dt, orc, cuda, dims, grid, np_dtype):
    nd = len(dims)
    plan = dt.PlanC2C(dims, comm=comm_for(dt, grid), precision=_prec(dt, np_dtype), executor=dt.Executor.CUFFT)
    g = random_global(tuple(dims[::-1]), np_dtype, seed=sum(dims))
    x = orc.global_to_packed(g, nd, grid, 1)
    a = to_dev(x, plan.alloc_size, cuda)
    b = empty(plan.alloc_size, np_dtype, cuda)
    plan.execute(a, b, dt.Execute.FORWARD)
    lay = _final_layout(plan, nd)
    expect = orc.global_to_packed(orc.forward_values(g, "c2c"), nd, grid, lay)
    out = from_dev(b, expect.size, np_dtype)
    assert orc.rel_l2(out, expect) <= TOL[np_dtype]
    c = empty(plan.alloc_size, np_dtype, cuda)
    plan.execute(b, c, dt.Execute.BACKWARD)
    back = from_dev(c, x.size, np_dtype).astype(np.complex128) / np.prod(dims)
    assert orc.rel_l2(back, x) <= TOL[np_dtype]
    thr = orc.roundtrip_threshold(int(np.prod(dims)), np_dtype == np.complex64)
    assert np.max(np.abs(back - x)) <= thr
    plan.destroy()


@pytest.mark.parametrize("dims,grid,np_dtype", [
    ([64, 48, 40], [1, 2, 4], np.complex64),
    ([512, 32, 24], [1, 2, 2], np.complex64),
    ([48, 36, 40], [1, 3, 2], np.complex128),
    ([96, 64], [1, 2], np.complex64),
    ([32, 24, 40], [1, 1, 1], np.float32),          # R2C: Y and Z axes fuse
    # rows the warp-per-row tile kernel takes (M = 256 / 512 / 768 / 1024)
    ([512, 512, 16], [1, 2, 2], np.complex64),
    ([256, 256, 48], [1, 2, 4], np.complex64),
    ([256, 40, 36], [1, 2, 2], np.complex64),        # ragged tiles: 20 and 18 rows per rank
    ([256, 33, 21], [1, 2, 2], np.complex64),        # odd destination strides (8-byte stores)
    ([768, 24, 20], [1, 2, 1], np.complex64),
    ([1024, 16, 20], [1, 1, 2], np.complex64),
    ([256, 256, 24], [1, 2, 2], np.complex128),
    ([512, 40, 12], [1, 3, 1], np.complex128),
    ([256, 512], [1, 2], np.complex64),
    ([512, 256, 32], [1, 1, 1], np.float32),        # R2C: the Y axis (256) fuses
    # runtime-schedule tile kernels (several rows per warp, K w-slices per tile)
    ([96, 40, 36], [1, 2, 2], np.complex64),         # M = 96: 4 threads per row, 8 rows per warp
    ([160, 48, 20], [1, 2, 1], np.complex64),
    ([384, 36, 10], [1, 3, 1], np.complex64),
    ([48, 320, 288], [1, 1, 1], np.complex64),       # Z-slab plan on the fused generic route
    ([100, 96, 160], [1, 1, 1], np.float32),         # R2C Z-slab plan on the fused generic route
    ([72, 50, 27], [1, 2, 2], np.complex64),         # odd Z (27): that axis stays unfused
])
def test_fused_fft_transpose(dt, orc, cuda, monkeypatch, dims, grid, np_dtype):
    """Plans built with the fused FFT + transpose passes (DTFFT_GB_FUSE=1)."""
    monkeypatch.setenv("DTFFT_GB_FUSE", "1")
    nd = len(dims)
    cfg = dt.Config(enable_z_slab=False)
    if np_dtype == np.float32:
        plan = dt.PlanR2C(dims, comm=comm_for(dt, grid), precision=dt.Precision.SINGLE,
                          executor=dt.Executor.CUFFT, config=cfg)
        cdt = np.complex64
    else:
        plan = dt.PlanC2C(dims, comm=comm_for(dt, grid), precision=_prec(dt, np_dtype),
                          executor=dt.Executor.CUFFT, config=cfg)
        cdt = np_dtype
    dt.set_config(dt.Config())
    g = random_global(tuple(dims[::-1]), np_dtype, seed=11)
    x = orc.global_to_packed(g, nd, grid, 1)
    a = to_dev(x, plan.alloc_size, cuda)
    b = empty(plan.alloc_size, cdt, cuda)
    plan.execute(a, b, dt.Execute.FORWARD)
    kind = "r2c" if np_dtype == np.float32 else "c2c"
    expect = orc.global_to_packed(orc.forward_values(g, kind), nd, grid, _final_layout(plan, nd))
    assert orc.rel_l2(from_dev(b, expect.size, cdt), expect) <= TOL[np_dtype]
    c = empty(plan.alloc_size, np_dtype, cuda)
    plan.execute(b, c, dt.Execute.BACKWARD)
    back = from_dev(c, x.size, np_dtype) / np.prod(dims)
    assert orc.rel_l2(back, x) <= TOL[np_dtype]
    plan.destroy()


@pytest.mark.parametrize("dims,grid,np_dtype,inplace", [
    ([256, 256, 256], [1, 1, 1], np.complex64, False),   # Z-slab plan, all three axes on tile kernels
    ([256, 256, 256], [1, 1, 1], np.complex64, True),
    ([256, 512, 256], [1, 1, 2], np.complex128, False),  # Z-slab on two virtual ranks
    ([512, 256, 48], [1, 2, 2], np.complex64, True),     # generic schedule, in == out
    ([256, 512], [1, 2], np.complex64, True),            # 2D, in == out
    ([256, 50, 36], [1, 2, 2], np.complex64, False),     # 25 rows per rank: ragged odd tiles, odd destinations
    ([512, 50, 36], [1, 2, 2], np.complex128, False),
    ([768, 24, 20], [1, 2, 1], np.complex64, False),     # store warps write straight from shared memory
    ([105, 84, 60], [1, 2, 2], np.complex64, True),      # fused two-factor passes, in == out
    ([225, 98, 45], [1, 1, 1], np.complex64, True),      # Z-slab on the two-factor generic route, in == out
])
def test_tile_schedules(dt, orc, cuda, dims, grid, np_dtype, inplace):
    """Fused tile passes on the default path: Z-slab plans take the generic
    X -> Y -> Z route when every pass fuses, and in-place execution (in ==
    out) never lets a fused pass read and write the same buffer."""
    nd = len(dims)
    plan = dt.PlanC2C(dims, comm=comm_for(dt, grid), precision=_prec(dt, np_dtype), executor=dt.Executor.CUFFT)
    if nd == 3 and grid[1] == 1:
        assert plan.z_slab_enabled
    g = random_global(tuple(dims[::-1]), np_dtype, seed=7)
    x = orc.global_to_packed(g, nd, grid, 1)
    a = to_dev(x, plan.alloc_size, cuda)
    b = a if inplace else empty(plan.alloc_size, np_dtype, cuda)
    plan.execute(a, b, dt.Execute.FORWARD)
    expect = orc.global_to_packed(orc.forward_values(g, "c2c"), nd, grid, _final_layout(plan, nd))
    assert orc.rel_l2(from_dev(b, expect.size, np_dtype), expect) <= TOL[np_dtype]
    c = b if inplace else empty(plan.alloc_size, np_dtype, cuda)
    plan.execute(b, c, dt.Execute.BACKWARD)
    back = from_dev(c, x.size, np_dtype).astype(np.complex128) / np.prod(dims)
    assert orc.rel_l2(back, x) <= TOL[np_dtype]
    plan.destroy()


def _profiled_names(L):
    L.dtfft_gb_profile_count.restype = ctypes.c_int32
    names = []
    for i in range(L.dtfft_gb_profile_count()):
        buf = ctypes.create_string_buffer(128)
        n, ms = ctypes.c_int64(), ctypes.c_double()
        L.dtfft_gb_profile_get(i, buf, 128, ctypes.byref(n), ctypes.byref(ms))
        names.append(buf.value.decode())
    return names


@pytest.mark.parametrize("dims,grid", [
    ([768, 84, 60], [1, 2, 1]),     # 5040 X rows: 16-row store-warp tiles, 8-row tensor-store tiles; 42 rows per rank
    ([768, 64, 40], [1, 2, 1]),     # 2560 X rows: both kernels tile by 8
    ([1024, 52, 48], [1, 2, 1]),    # 26 rows per rank: a ragged last tile of 2 rows
    ([512, 84, 60], [1, 2, 1]),     # 128-byte lines of 16-row tiles, ragged (42 rows per rank)
])
def test_tensor_store_fused_pass(dt, orc, cuda, monkeypatch, dims, grid):
    """The fused X pass with the tensor-store write-out (64-byte lines of
    8-row tiles for 768- and 1024-point rows, 128-byte lines of 16-row tiles
    for 512): the profiled launch list shows the kernel, and forward and
    backward match the oracle."""
    monkeypatch.setenv("DTFFT_GB_FUSE", "1")
    L = dt.lib()
    plan = dt.PlanC2C(dims, comm=comm_for(dt, grid), precision=dt.Precision.SINGLE, executor=dt.Executor.CUFFT,
                      config=dt.Config(enable_z_slab=False))
    dt.set_config(dt.Config())
    g = random_global(tuple(dims[::-1]), np.complex64, seed=23)
    x = orc.global_to_packed(g, 3, grid, 1)
    a = to_dev(x, plan.alloc_size, cuda)
    b = empty(plan.alloc_size, np.complex64, cuda)
    c = empty(plan.alloc_size, np.complex64, cuda)
    expect = orc.global_to_packed(orc.forward_values(g, "c2c"), 3, grid, _final_layout(plan, 3))
    L.dtfft_gb_profile_start()
    plan.execute(a, b, dt.Execute.FORWARD)
    fwd = from_dev(b, expect.size, np.complex64)       # backward may overwrite its input
    plan.execute(b, c, dt.Execute.BACKWARD)
    L.dtfft_gb_profile_stop()
    names = _profiled_names(L)
    assert ("ffttile_xtma_m%d_f32" % dims[0]) in names, names
    assert L.dtfft_gb_device_status(1) == 0
    assert orc.rel_l2(fwd, expect) <= TOL[np.complex64]
    back = from_dev(c, x.size, np.complex64).astype(np.complex128) / np.prod(dims)
    assert orc.rel_l2(back, x) <= TOL[np.complex64]
    plan.destroy()


@pytest.mark.parametrize("n,howmany", [(105, 777), (378, 300), (225, 1001), (343, 100), (40, 5000), (400, 64),
                                        (245, 3), (1000, 300), (882, 97), (729, 200), (405, 50)])
def test_two_factor_rows(dt, cuda, monkeypatch, n, howmany):
    """Batched C2C rows on the two-factor kernel (fft_2f.cuh; DTFFT_GB_F2=1
    makes every C2C float step with a compiled split take it): forward and
    backward against numpy FP64, ragged last CTA included."""
    import torch
    monkeypatch.setenv("DTFFT_GB_F2", "1")
    monkeypatch.setenv("DTFFT_GB_F2P", "0")      # the unpipelined kernel (pipelined rows: below)
    L = dt.lib()
    h = ctypes.c_void_p()
    sizes = (ctypes.c_int32 * 1)(n)
    assert L.gb_fft_create(1, 0, 0, n, n, howmany, sizes, sizes, sizes, None, None, ctypes.byref(h)) == 0
    rng = np.random.default_rng(n)
    x = (rng.uniform(-1, 1, (howmany, n)) + 1j * rng.uniform(-1, 1, (howmany, n))).astype(np.complex64)
    a = torch.from_numpy(x).to(cuda)
    b = torch.empty_like(a)
    torch.cuda.synchronize()
    L.dtfft_gb_profile_start()
    assert L.gb_fft_execute(h, a.data_ptr(), b.data_ptr(), -1) == 0
    torch.cuda.synchronize()
    fwd = b.cpu().numpy()
    assert L.gb_fft_execute(h, b.data_ptr(), a.data_ptr(), 1) == 0
    torch.cuda.synchronize()
    L.dtfft_gb_profile_stop()
    assert ("fft2f_rows_c2c_m%d_f32" % n) in _profiled_names(L)
    ref = np.fft.fft(x.astype(np.complex128), axis=1)
    assert np.linalg.norm(fwd - ref) / np.linalg.norm(ref) <= 1e-5
    back = a.cpu().numpy() / n
    assert np.linalg.norm(back - x) / np.linalg.norm(x) <= 1e-5
    assert L.gb_fft_destroy(ctypes.byref(h)) == 0


@pytest.mark.parametrize("n,howmany,shape", [(105, 777, "256,8,2"), (378, 301, "128,4,3"), (225, 1000, "256,16,2"),
                                              (343, 99, "128,16,3"), (40, 5001, "256,4,2"), (1008, 63, "128,4,2"),
                                              (945, 100, "256,2,2")])
@pytest.mark.parametrize("offset", [0, 1])
def test_two_factor_pipelined_rows(dt, cuda, monkeypatch, n, howmany, shape, offset):
    """Pipelined two-factor rows (bulk-copy ring of row tiles): odd lengths
    with an odd last tile (the 8-byte tail read apart), and an input one
    element off 16-byte alignment, which runs the unpipelined kernel."""
    import torch
    monkeypatch.setenv("DTFFT_GB_F2P", shape)
    L = dt.lib()
    h = ctypes.c_void_p()
    sizes = (ctypes.c_int32 * 1)(n)
    assert L.gb_fft_create(1, 0, 0, n, n, howmany, sizes, sizes, sizes, None, None, ctypes.byref(h)) == 0
    rng = np.random.default_rng(n + offset)
    x = (rng.uniform(-1, 1, (howmany, n)) + 1j * rng.uniform(-1, 1, (howmany, n))).astype(np.complex64)
    buf = torch.zeros(howmany * n + 2, dtype=torch.complex64, device=cuda)
    a = buf[offset:offset + howmany * n]
    a.copy_(torch.from_numpy(x.ravel()).to(cuda))
    b = torch.empty(howmany * n, dtype=torch.complex64, device=cuda)
    torch.cuda.synchronize()
    L.dtfft_gb_profile_start()
    assert L.gb_fft_execute(h, a.data_ptr(), b.data_ptr(), -1) == 0
    torch.cuda.synchronize()
    L.dtfft_gb_profile_stop()
    names = _profiled_names(L)
    want = ("fft2f_rows_c2c_m%d_f32" if offset else "fft2f_pipe_c2c_m%d_f32") % n
    assert want in names, names
    assert L.dtfft_gb_device_status(1) == 0
    fwd = b.cpu().numpy().reshape(howmany, n)
    ref = np.fft.fft(x.astype(np.complex128), axis=1)
    assert np.linalg.norm(fwd - ref) / np.linalg.norm(ref) <= 1e-5
    assert L.gb_fft_execute(h, b.data_ptr(), a.data_ptr(), 1) == 0
    torch.cuda.synchronize()
    back = a.cpu().numpy().reshape(howmany, n) / n
    assert np.linalg.norm(back - x) / np.linalg.norm(x) <= 1e-5
    assert L.gb_fft_destroy(ctypes.byref(h)) == 0


@pytest.mark.parametrize("n,howmany", [(350, 513), (245, 77), (96, 1000), (756, 31), (125, 300), (80, 7),
                                        (1400, 40), (945, 33), (2000, 9)])
def test_two_factor_real_rows(dt, cuda, monkeypatch, n, howmany):
    """R2C / C2R rows on the two-factor kernel: even n through the n/2-point
    core (R2C pairs outputs k and n/2 - k in a third phase), odd n through the
    full-length core; against numpy FP64."""
    import torch
    monkeypatch.setenv("DTFFT_GB_F2", "1")
    L = dt.lib()
    h = ctypes.c_void_p()
    sizes = (ctypes.c_int32 * 1)(n)
    nc = n // 2 + 1
    assert L.gb_fft_create(1, 1, 0, n, nc, howmany, sizes, sizes, sizes, None, None, ctypes.byref(h)) == 0
    x = np.random.default_rng(n).standard_normal((howmany, n)).astype(np.float32)
    a = torch.from_numpy(x).to(cuda)
    b = torch.empty((howmany, nc), dtype=torch.complex64, device=cuda)
    torch.cuda.synchronize()
    L.dtfft_gb_profile_start()
    assert L.gb_fft_execute(h, a.data_ptr(), b.data_ptr(), -1) == 0
    torch.cuda.synchronize()
    fwd = b.cpu().numpy()
    c = torch.empty_like(a)
    assert L.gb_fft_execute(h, b.data_ptr(), c.data_ptr(), 1) == 0
    torch.cuda.synchronize()
    L.dtfft_gb_profile_stop()
    names = _profiled_names(L)
    assert ("fft2f_rows_r2c_m%d_f32" % (n // 2 if n % 2 == 0 else n)) in names, names
    assert ("fft2f_rows_c2r_m%d_f32" % (n // 2 if n % 2 == 0 else n)) in names, names
    ref = np.fft.rfft(x.astype(np.float64), axis=1)
    assert np.linalg.norm(fwd - ref) / np.linalg.norm(ref) <= 1e-5
    back = c.cpu().numpy() / n
    assert np.linalg.norm(back - x) / np.linalg.norm(x) <= 1e-5
    assert L.gb_fft_destroy(ctypes.byref(h)) == 0


@pytest.mark.parametrize("kind,dims,grid", [
    ("c2c", [105, 84, 60], [1, 2, 2]),     # every pass fused: X (105), Y (84) rows + transposes
    ("c2c", [378, 45, 49], [1, 2, 1]),     # 45 rows per Y pencil split over 2: ragged 8-row tiles
    ("c2c", [64, 105, 40], [1, 1, 1]),     # Z-slab plan on the generic X -> Y -> Z route
    ("c2c", [225, 288, 49], [1, 1, 1]),    # the batch's first shape
    ("r2c", [48, 175, 56], [1, 2, 2]),     # R2C: the complex Y / Z passes fuse
    ("c2c", [49, 343, 7], [1, 3, 1]),      # three ranks, a 7-point Z axis that stays unfused
    ("c2c", [1000, 60, 48], [1, 2, 2]),    # 1000 = 25 x 40
    ("c2c", [42, 729, 40], [1, 1, 1]),     # Z-slab generic route with a 729-point Y axis
])
def test_two_factor_fused_transpose(dt, orc, cuda, kind, dims, grid):
    """The two-factor kernel fused with the box-list transpose (default for
    float lengths without a tile kernel): launch list and oracle parity."""
    L = dt.lib()
    np_dtype = np.complex64 if kind == "c2c" else np.float32
    mk = dt.PlanC2C if kind == "c2c" else dt.PlanR2C
    plan = mk(dims, comm=comm_for(dt, grid), precision=dt.Precision.SINGLE, executor=dt.Executor.CUFFT)
    g = random_global(tuple(dims[::-1]), np_dtype, seed=47)
    x = orc.global_to_packed(g, 3, grid, 1)
    a = to_dev(x, plan.alloc_size, cuda)
    b = empty(plan.alloc_size, np.complex64, cuda)
    expect = orc.global_to_packed(orc.forward_values(g, kind), 3, grid, _final_layout(plan, 3))
    L.dtfft_gb_profile_start()
    plan.execute(a, b, dt.Execute.FORWARD)
    fwd = from_dev(b, expect.size, np.complex64)
    c = empty(plan.alloc_size, np_dtype, cuda)
    plan.execute(b, c, dt.Execute.BACKWARD)
    L.dtfft_gb_profile_stop()
    names = _profiled_names(L)
    assert any(nm.startswith("fft2f_xpose_m") for nm in names), names
    assert L.dtfft_gb_device_status(1) == 0
    assert orc.rel_l2(fwd, expect) <= 1e-5
    back = from_dev(c, x.size, np_dtype).astype(np.complex128) / np.prod(dims)
    assert orc.rel_l2(back, x) <= 1e-5
    plan.destroy()


@pytest.mark.parametrize("kind,dims", [("c2c", [64, 105, 40]), ("c2c", [75, 378, 49]), ("r2c", [48, 175, 56]),
                                       ("c2c", [50, 343, 40])])
def test_two_factor_columns_in_z_slab_plans(dt, orc, cuda, monkeypatch, kind, dims):
    """Z-slab plans whose Y columns (and X / Z rows) take the two-factor kernel
    (unfused: with fusion these plans take the generic X -> Y -> Z route)."""
    monkeypatch.setenv("DTFFT_GB_F2", "1")
    monkeypatch.setenv("DTFFT_GB_FUSE", "0")
    L = dt.lib()
    np_dtype = np.complex64 if kind == "c2c" else np.float32
    mk = dt.PlanC2C if kind == "c2c" else dt.PlanR2C
    plan = mk(dims, precision=dt.Precision.SINGLE, executor=dt.Executor.CUFFT)
    assert plan.z_slab_enabled
    g = random_global(tuple(dims[::-1]), np_dtype, seed=43)
    x = orc.global_to_packed(g, 3, [1, 1, 1], 1)
    a = to_dev(x, plan.alloc_size, cuda)
    b = empty(plan.alloc_size, np.complex64, cuda)
    expect = orc.global_to_packed(orc.forward_values(g, kind), 3, [1, 1, 1], _final_layout(plan, 3))
    L.dtfft_gb_profile_start()
    plan.execute(a, b, dt.Execute.FORWARD)
    fwd = from_dev(b, expect.size, np.complex64)
    c = empty(plan.alloc_size, np_dtype, cuda)
    plan.execute(b, c, dt.Execute.BACKWARD)
    L.dtfft_gb_profile_stop()
    assert ("fft2f_cols_c2c_m%d_f32" % dims[1]) in _profiled_names(L)
    assert orc.rel_l2(fwd, expect) <= 1e-5
    back = from_dev(c, x.size, np_dtype).astype(np.complex128) / np.prod(dims)
    assert orc.rel_l2(back, x) <= 1e-5
    plan.destroy()


@pytest.mark.parametrize("dims,grid,np_dtype", [
    ([512, 64, 32], [1, 2, 2], np.complex64),
    ([256, 48, 256], [1, 1, 2], np.complex128),
])
def test_exhaustive_tuned_fused_pass(dt, orc, cuda, dims, grid, np_dtype):
    """EXHAUSTIVE plans time every compiled warp split of the fused tile pass
    (and the transpose tiles) and keep the fastest; results stay correct."""
    nd = len(dims)
    plan = dt.PlanC2C(dims, comm=comm_for(dt, grid), precision=_prec(dt, np_dtype), executor=dt.Executor.CUFFT,
                      effort=dt.Effort.EXHAUSTIVE)
    g = random_global(tuple(dims[::-1]), np_dtype, seed=17)
    x = orc.global_to_packed(g, nd, grid, 1)
    a = to_dev(x, plan.alloc_size, cuda)
    b = empty(plan.alloc_size, np_dtype, cuda)
    plan.execute(a, b, dt.Execute.FORWARD)
    expect = orc.global_to_packed(orc.forward_values(g, "c2c"), nd, grid, _final_layout(plan, nd))
    assert orc.rel_l2(from_dev(b, expect.size, np_dtype), expect) <= TOL[np_dtype]
    c = empty(plan.alloc_size, np_dtype, cuda)
    plan.execute(b, c, dt.Execute.BACKWARD)
    back = from_dev(c, x.size, np_dtype).astype(np.complex128) / np.prod(dims)
    assert orc.rel_l2(back, x) <= TOL[np_dtype]
    plan.destroy()


def test_c2c_schedules_agree(dt, orc, cuda):
    """Z-slab, Y-slab and the generic 3-pencil schedule give the same spectrum."""
    dims = [64, 64, 64]
    g = random_global(tuple(dims[::-1]), np.complex64, seed=3)
    expect = orc.forward_values(g, "c2c")
    for zs, ys in ((True, False), (False, True), (False, False)):
        cfg = dt.Config(enable_z_slab=zs, enable_y_slab=ys)
        plan = dt.PlanC2C(dims, precision=dt.Precision.SINGLE, executor=dt.Executor.VKFFT, config=cfg)
        assert plan.z_slab_enabled == zs and plan.y_slab_enabled == (ys and not zs)
        x = orc.global_to_packed(g, 3, [1, 1, 1], 1)
        a = to_dev(x, plan.alloc_size, cuda)
        b = empty(plan.alloc_size, np.complex64, cuda)
        plan.execute(a, b, dt.Execute.FORWARD)
        lay = _final_layout(plan, 3)
        out = from_dev(b, x.size, np.complex64)
        assert orc.rel_l2(out, orc.global_to_packed(expect, 3, [1, 1, 1], lay)) <= 1e-5
        plan.destroy()
    dt.set_config(dt.Config())


R2C_CASES = [
    ([32, 24, 40], [1, 1, 1], np.float32),
    ([16, 32, 70], [1, 1, 1], np.float64),           # tests/c/test_r2c_3d_c.c sizes
    ([33, 20, 12], [1, 2, 2], np.float32),           # odd nx
    ([64, 32, 36], [1, 4, 4], np.float64),           # 4x4 grid, 33 complex split unevenly
    ([30, 26], [1, 1], np.float32),
    ([21, 16], [1, 2], np.float64),
    ([100, 96, 160], [1, 1, 1], np.float32),         # Z-slab plan on the fused generic route
    ([96, 64, 48], [1, 1, 2], np.float32),
]


@pytest.mark.parametrize("dims,grid,np_dtype", R2C_CASES)
def test_r2c_forward_backward(dt, orc, cuda, dims, grid, np_dtype):
    nd = len(dims)
    cdt = np.complex64 if np_dtype == np.float32 else np.complex128
    plan = dt.PlanR2C(dims, comm=comm_for(dt, grid), precision=_prec(dt, np_dtype), executor=dt.Executor.CUFFT)
    g = random_global(tuple(dims[::-1]), np_dtype, seed=sum(dims), dist="normal")
    x = orc.global_to_packed(g, nd, grid, 1)
    n_real = plan.alloc_size
    a = to_dev(x, n_real, cuda)
    b = empty(n_real // 2 + 1, cdt, cuda)
    plan.execute(a, b, dt.Execute.FORWARD)
    lay = _final_layout(plan, nd)
    G = orc.forward_values(g, "r2c")
    expect = orc.global_to_packed(G, nd, grid, lay)
    out = from_dev(b, expect.size, cdt)
    assert orc.rel_l2(out, expect) <= TOL[np_dtype]
    c = empty(n_real, np_dtype, cuda)
    plan.execute(b, c, dt.Execute.BACKWARD)
    back = from_dev(c, x.size, np_dtype).astype(np.float64) / np.prod(dims)
    assert orc.rel_l2(back, x) <= TOL[np_dtype]
    plan.destroy()


KINDS = [(5, 5), (4, 4), (3, 3), (6, 6), (7, 7), (9, 9), (8, 8), (10, 10)]


@pytest.mark.parametrize("kinds", KINDS)
@pytest.mark.parametrize("np_dtype", [np.float64, np.float32])
def test_r2r_kinds_roundtrip_17x23(dt, orc, cuda, kinds, np_dtype):
    """tests/python/test_r2r_kinds_py.py: 17 x 23, every kind, FFTW scale conventions."""
    nx, ny = 17, 23
    plan = dt.PlanR2R([nx, ny], kinds=list(kinds), precision=_prec(dt, np_dtype), executor=dt.Executor.VKFFT)
    g = random_global((ny, nx), np_dtype, seed=kinds[0])
    x = orc.global_to_packed(g, 2, [1, 1], 1)
    a = to_dev(x, plan.alloc_size, cuda)
    b = empty(plan.alloc_size, np_dtype, cuda)
    plan.execute(a, b, dt.Execute.FORWARD)
    expect = orc.global_to_packed(orc.forward_values(g, "r2r", kinds=list(kinds)), 2, [1, 1], 2)
    out = from_dev(b, expect.size, np_dtype)
    assert orc.rel_l2(out, expect) <= TOL[np_dtype]
    plan.execute(b, a, dt.Execute.BACKWARD)
    back = from_dev(a, x.size, np_dtype).astype(np.float64) / orc.r2r_roundtrip_scale([nx, ny], kinds)
    atol = 1e-10 if np_dtype == np.float64 else 2e-5
    assert np.max(np.abs(back - x)) <= atol
    plan.destroy()


@pytest.mark.parametrize("dims,grid,kinds", [
    ([16, 24, 32], [1, 1, 1], (5, 5, 5)),           # Z-slab: 2D kinds (X, Y) then Z
    ([16, 12, 20], [1, 2, 2], (5, 4, 6)),
    ([9, 10, 12], [1, 1, 1], (3, 7, 9)),
    ([64, 32, 40], [1, 4, 4], (10, 8, 5)),
    # even lengths: DCT/DST-II and -III through the n/2-point complex FFT
    ([16, 24, 32], [1, 1, 1], (9, 9, 9)),
    ([32, 20, 24], [1, 2, 2], (5, 9, 4)),
    ([48, 40, 64], [1, 2, 1], (8, 4, 5)),
    ([8, 10, 12], [1, 1, 1], (4, 8, 9)),
])
def test_r2r_3d(dt, orc, cuda, dims, grid, kinds):
    plan = dt.PlanR2R(dims, kinds=list(kinds), comm=comm_for(dt, grid), precision=dt.Precision.DOUBLE,
                      executor=dt.Executor.VKFFT)
    g = random_global(tuple(dims[::-1]), np.float64, seed=9, dist="normal")
    x = orc.global_to_packed(g, 3, grid, 1)
    a = to_dev(x, plan.alloc_size, cuda)
    b = empty(plan.alloc_size, np.float64, cuda)
    plan.execute(a, b, dt.Execute.FORWARD)
    lay = _final_layout(plan, 3)
    expect = orc.global_to_packed(orc.forward_values(g, "r2r", kinds=list(kinds)), 3, grid, lay)
    assert orc.rel_l2(from_dev(b, expect.size, np.float64), expect) <= 1e-12
    plan.execute(b, a, dt.Execute.BACKWARD)
    back = from_dev(a, x.size, np.float64) / orc.r2r_roundtrip_scale(dims, kinds)
    assert np.max(np.abs(back - x)) <= 1e-10
    plan.destroy()


@pytest.mark.parametrize("dims,kinds", [
    ([40, 24], (5, 9)),        # DCT-II x DST-II, even: n/2-point complex FFTs
    ([64, 30], (4, 8)),        # DCT-III x DST-III
    ([24, 96], (9, 4)),
])
def test_r2r_even_single(dt, orc, cuda, dims, kinds):
    """Single-precision R2R kinds on even lengths (half-length FFT path) against
    the FP64 oracle at the single-precision tolerance."""
    plan = dt.PlanR2R(dims, kinds=list(kinds), precision=dt.Precision.SINGLE, executor=dt.Executor.VKFFT)
    g = random_global(tuple(dims[::-1]), np.float32, seed=21, dist="normal")
    x = orc.global_to_packed(g, 2, [1, 1], 1)
    a = to_dev(x, plan.alloc_size, cuda)
    b = empty(plan.alloc_size, np.float32, cuda)
    plan.execute(a, b, dt.Execute.FORWARD)
    expect = orc.global_to_packed(orc.forward_values(g, "r2r", kinds=list(kinds)), 2, [1, 1], 2)
    assert orc.rel_l2(from_dev(b, expect.size, np.float32), expect) <= 1e-5
    plan.execute(b, a, dt.Execute.BACKWARD)
    back = from_dev(a, x.size, np.float32).astype(np.float64) / orc.r2r_roundtrip_scale(dims, kinds)
    assert orc.rel_l2(back, x) <= 1e-5
    plan.destroy()


def test_r2r_with_cufft_executor_is_refused(dt):
    with pytest.raises(dt.DtfftError) as e:
        dt.PlanR2R([16, 16], kinds=[5, 5], executor=dt.Executor.CUFFT)
    assert e.value.code == 101


def test_r2c_transpose_only_execute_refused(dt, cuda):
    import torch
    plan = dt.PlanR2C([16, 16, 16], precision=dt.Precision.SINGLE)
    a = torch.zeros(plan.alloc_size, dtype=torch.float32, device=cuda)
    b = torch.zeros_like(a)
    with pytest.raises(dt.DtfftError) as e:
        plan.execute(a, b, dt.Execute.FORWARD)
    assert e.value.code == 45
    plan.destroy()


# ---- FFT plug-in (gb_fft_*), the executor seam ------------------------------

@pytest.mark.parametrize("n,howmany", [(256, 64), (768, 9), (17, 5), (1000, 3), (2048, 4)])
def test_fft_plugin_c2c(dt, cuda, n, howmany):
    import torch
    L = dt.lib()
    h = ctypes.c_void_p()
    sizes = (ctypes.c_int32 * 1)(n)
    assert L.gb_fft_create(1, 0, 0, n, n, howmany, sizes, sizes, sizes, None, None, ctypes.byref(h)) == 0
    rng = np.random.default_rng(n)
    x = (rng.uniform(-1, 1, (howmany, n)) + 1j * rng.uniform(-1, 1, (howmany, n))).astype(np.complex64)
    a = torch.from_numpy(x).to(cuda)
    b = torch.empty_like(a)
    assert L.gb_fft_execute(h, a.data_ptr(), b.data_ptr(), -1) == 0
    torch.cuda.synchronize()
    ref = np.fft.fft(x.astype(np.complex128), axis=1)
    err = np.linalg.norm(b.cpu().numpy() - ref) / np.linalg.norm(ref)
    assert err <= 1e-5
    assert L.gb_fft_execute(h, b.data_ptr(), b.data_ptr(), 1) == 0   # in place, backward
    torch.cuda.synchronize()
    back = b.cpu().numpy() / n
    assert np.linalg.norm(back - x) / np.linalg.norm(x) <= 1e-5
    assert L.gb_fft_destroy(ctypes.byref(h)) == 0


@pytest.mark.parametrize("n", [64, 30, 31])
def test_fft_plugin_r2c(dt, cuda, n):
    import torch
    L = dt.lib()
    h = ctypes.c_void_p()
    sizes = (ctypes.c_int32 * 1)(n)
    onembed = (ctypes.c_int32 * 1)(n // 2 + 1)
    howmany = 7
    assert L.gb_fft_create(1, 1, 1, n, n // 2 + 1, howmany, sizes, sizes, onembed, None, None, ctypes.byref(h)) == 0
    x = np.random.default_rng(n).standard_normal((howmany, n))
    a = torch.from_numpy(x).to(cuda)
    b = torch.empty((howmany, n // 2 + 1), dtype=torch.complex128, device=cuda)
    assert L.gb_fft_execute(h, a.data_ptr(), b.data_ptr(), -1) == 0
    torch.cuda.synchronize()
    ref = np.fft.rfft(x, axis=1)
    assert np.linalg.norm(b.cpu().numpy() - ref) / np.linalg.norm(ref) <= 1e-12
    c = torch.empty_like(a)
    assert L.gb_fft_execute(h, b.data_ptr(), c.data_ptr(), 1) == 0
    torch.cuda.synchronize()
    assert np.linalg.norm(c.cpu().numpy() / n - x) / np.linalg.norm(x) <= 1e-12
    L.gb_fft_destroy(ctypes.byref(h))


def test_device_status_clean_after_runs(dt, cuda):
    """No bounded wait of the pipelined kernels gave up during the GPU tests."""
    import torch
    torch.cuda.synchronize()
    dt.lib().dtfft_gb_device_status.restype = ctypes.c_int32
    assert dt.lib().dtfft_gb_device_status(0) == 0


@pytest.mark.parametrize("dims,grid,np_dtype", [
    ([1, 16, 12], [1, 1, 1], np.complex64),          # axes of length 1
    ([16, 1, 12], [1, 1, 1], np.complex64),
    ([16, 12, 1], [1, 1, 1], np.complex128),
    ([1, 1, 1], [1, 1, 1], np.complex64),
    ([4, 1, 6], [1, 2, 2], np.complex64),            # length-1 axis split over ranks (empty ranks)
    ([2, 3], [1, 1], np.complex128),
    ([1, 7], [1, 2], np.complex64),
])
def test_c2c_degenerate_dims(dt, orc, cuda, dims, grid, np_dtype):
    nd = len(dims)
    plan = dt.PlanC2C(dims, comm=comm_for(dt, grid), precision=_prec(dt, np_dtype), executor=dt.Executor.CUFFT)
    g = random_global(tuple(dims[::-1]), np_dtype, seed=23)
    x = orc.global_to_packed(g, nd, grid, 1)
    a = to_dev(x, plan.alloc_size, cuda)
    b = empty(plan.alloc_size, np_dtype, cuda)
    plan.execute(a, b, dt.Execute.FORWARD)
    expect = orc.global_to_packed(orc.forward_values(g, "c2c"), nd, grid, _final_layout(plan, nd))
    assert orc.rel_l2(from_dev(b, expect.size, np_dtype), expect) <= TOL[np_dtype]
    c = empty(plan.alloc_size, np_dtype, cuda)
    plan.execute(b, c, dt.Execute.BACKWARD)
    back = from_dev(c, x.size, np_dtype).astype(np.complex128) / np.prod(dims)
    assert orc.rel_l2(back, x) <= TOL[np_dtype]
    plan.destroy()


@pytest.mark.parametrize("dims,kind", [([16, 12, 2], "r2c"), ([2, 8, 6], "r2c"), ([8, 1, 4], "r2c")])
def test_r2c_degenerate_dims(dt, orc, cuda, dims, kind):
    plan = dt.PlanR2C(dims, precision=dt.Precision.DOUBLE, executor=dt.Executor.CUFFT)
    g = random_global(tuple(dims[::-1]), np.float64, seed=29, dist="normal")
    x = orc.global_to_packed(g, 3, [1, 1, 1], 1)
    a = to_dev(x, plan.alloc_size, cuda)
    b = empty(plan.alloc_size // 2 + 1, np.complex128, cuda)
    plan.execute(a, b, dt.Execute.FORWARD)
    expect = orc.global_to_packed(orc.forward_values(g, "r2c"), 3, [1, 1, 1], _final_layout(plan, 3))
    assert orc.rel_l2(from_dev(b, expect.size, np.complex128), expect) <= 1e-12
    c = empty(plan.alloc_size, np.float64, cuda)
    plan.execute(b, c, dt.Execute.BACKWARD)
    back = from_dev(c, x.size, np.float64) / np.prod(dims)
    assert orc.rel_l2(back, x) <= 1e-12
    plan.destroy()


@pytest.mark.parametrize("dims,grid,np_dtype", [
    ([131, 12, 10], [1, 1, 1], np.complex64),        # prime rows above the direct butterflies
    ([16, 131, 12], [1, 1, 1], np.complex64),        # prime columns of the Z-slab 2D pass
    ([20, 18, 257], [1, 2, 2], np.complex128),       # prime Z on a 2x2 grid
    ([262, 9], [1, 1], np.complex64),                # 2 x 131
    ([139, 130], [1, 2], np.complex128),
])
def test_c2c_bluestein_lengths(dt, orc, cuda, dims, grid, np_dtype):
    """Lengths with a prime factor above 127 take Bluestein's chirp-z form
    (two power-of-two FFTs per row); the reference's executors accept them too."""
    nd = len(dims)
    plan = dt.PlanC2C(dims, comm=comm_for(dt, grid), precision=_prec(dt, np_dtype), executor=dt.Executor.CUFFT)
    g = random_global(tuple(dims[::-1]), np_dtype, seed=31)
    x = orc.global_to_packed(g, nd, grid, 1)
    a = to_dev(x, plan.alloc_size, cuda)
    b = empty(plan.alloc_size, np_dtype, cuda)
    plan.execute(a, b, dt.Execute.FORWARD)
    expect = orc.global_to_packed(orc.forward_values(g, "c2c"), nd, grid, _final_layout(plan, nd))
    assert orc.rel_l2(from_dev(b, expect.size, np_dtype), expect) <= TOL[np_dtype]
    c = empty(plan.alloc_size, np_dtype, cuda)
    plan.execute(b, c, dt.Execute.BACKWARD)
    back = from_dev(c, x.size, np_dtype).astype(np.complex128) / np.prod(dims)
    assert orc.rel_l2(back, x) <= TOL[np_dtype]
    plan.destroy()


@pytest.mark.parametrize("dims,grid,np_dtype", [
    ([131, 12, 10], [1, 1, 1], np.float32),          # odd prime real axis: full-length complex core
    ([24, 139, 8], [1, 1, 2], np.float64),
    ([263, 16], [1, 1], np.float64),
])
def test_r2c_bluestein_lengths(dt, orc, cuda, dims, grid, np_dtype):
    nd = len(dims)
    cdt = np.complex64 if np_dtype == np.float32 else np.complex128
    plan = dt.PlanR2C(dims, comm=comm_for(dt, grid), precision=_prec(dt, np_dtype), executor=dt.Executor.CUFFT)
    g = random_global(tuple(dims[::-1]), np_dtype, seed=37, dist="normal")
    x = orc.global_to_packed(g, nd, grid, 1)
    a = to_dev(x, plan.alloc_size, cuda)
    b = empty(plan.alloc_size // 2 + 1, cdt, cuda)
    plan.execute(a, b, dt.Execute.FORWARD)
    expect = orc.global_to_packed(orc.forward_values(g, "r2c"), nd, grid, _final_layout(plan, nd))
    assert orc.rel_l2(from_dev(b, expect.size, cdt), expect) <= TOL[np_dtype]
    c = empty(plan.alloc_size, np_dtype, cuda)
    plan.execute(b, c, dt.Execute.BACKWARD)
    back = from_dev(c, x.size, np_dtype) / np.prod(dims)
    assert orc.rel_l2(back, x) <= TOL[np_dtype]
    plan.destroy()


@pytest.mark.parametrize("dims,grid,kinds,np_dtype", [
    ([132, 12, 10], [1, 1, 1], (3, 4, 5), np.float64),     # DCT-I: core 2(n-1) = 2 x 131
    ([130, 10, 12], [1, 1, 1], (7, 8, 9), np.float64),     # DST-I: core 2(n+1) = 2 x 131
    ([131, 12, 10], [1, 1, 1], (4, 5, 6), np.float32),     # DCT-II of prime length 131
    ([10, 131, 12], [1, 1, 1], (8, 9, 10), np.float64),    # DST-II along columns (Y of the Z-slab pass)
    ([12, 10, 139], [1, 2, 2], (5, 6, 9), np.float64),     # DST-III on Z of a 2x2 grid
    ([131, 8], [1, 1], (6, 10), np.float32),               # DCT-IV: core 2n = 262
    ([8, 131], [1, 1], (3, 10), np.float64),               # DST-IV on Y
    ([262, 8], [1, 1], (5, 4), np.float64),                # even DCT-III whose half length (131) has no schedule
    ([20, 131, 18], [1, 2, 2], (4, 9, 6), np.float64),
])
def test_r2r_bluestein_lengths(dt, orc, cuda, dims, grid, kinds, np_dtype):
    """R2R kinds whose complex core length has a prime factor above 127 run
    the core through Bluestein's chirp-z form (the reference's VkFFT and FFTW
    executors take every length)."""
    nd = len(dims)
    plan = dt.PlanR2R(dims, kinds=list(kinds), comm=comm_for(dt, grid), precision=_prec(dt, np_dtype),
                      executor=dt.Executor.VKFFT)
    g = random_global(tuple(dims[::-1]), np_dtype, seed=41, dist="normal")
    x = orc.global_to_packed(g, nd, grid, 1)
    a = to_dev(x, plan.alloc_size, cuda)
    b = empty(plan.alloc_size, np_dtype, cuda)
    plan.execute(a, b, dt.Execute.FORWARD)
    expect = orc.global_to_packed(orc.forward_values(g, "r2r", kinds=list(kinds)), nd, grid, _final_layout(plan, nd))
    assert orc.rel_l2(from_dev(b, expect.size, np_dtype), expect) <= TOL[np_dtype]
    plan.execute(b, a, dt.Execute.BACKWARD)
    back = from_dev(a, x.size, np_dtype).astype(np.float64) / orc.r2r_roundtrip_scale(dims, kinds)
    assert orc.rel_l2(back, x) <= TOL[np_dtype]
    plan.destroy()


def test_plans_release_device_memory(dt, cuda):
    """Creating and destroying plans of every kind (fused tile passes, TMA
    transposes with cached tensor maps, Bluestein scratch, autotuned splits)
    returns the device memory they took."""
    import torch
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    free0, _ = torch.cuda.mem_get_info()
    for it in range(3):
        plans = [
            dt.PlanC2C([512, 64, 32], comm=comm_for(dt, [1, 2, 2]), precision=dt.Precision.SINGLE,
                       executor=dt.Executor.CUFFT, effort=dt.Effort.EXHAUSTIVE),
            dt.PlanC2C([131, 12, 10], precision=dt.Precision.SINGLE, executor=dt.Executor.CUFFT),
            dt.PlanR2C([64, 32, 36], comm=comm_for(dt, [1, 4, 4]), precision=dt.Precision.DOUBLE,
                       executor=dt.Executor.CUFFT),
            dt.PlanR2R([16, 24, 32], kinds=[5, 5, 5], precision=dt.Precision.DOUBLE, executor=dt.Executor.VKFFT),
        ]
        for p in plans:
            n = p.alloc_size
            a = torch.zeros(n, dtype=torch.float64, device=cuda)
            b = torch.zeros(n, dtype=torch.float64, device=cuda)
            torch.cuda.synchronize()
            if isinstance(p, dt.PlanR2R) or isinstance(p, dt.PlanR2C):
                p.execute(a, b, dt.Execute.FORWARD)
            else:
                p.transpose(a, b, dt.Transpose.X_TO_Y) if p.grid_dims[1] * p.grid_dims[2] > 1 else None
                p.execute(a, b, dt.Execute.FORWARD)
            torch.cuda.synchronize()
            del a, b
        for p in plans:
            p.destroy()
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
    free1, _ = torch.cuda.mem_get_info()
    assert free0 - free1 < 64 << 20, f"{(free0 - free1) >> 20} MiB not returned"


@pytest.mark.parametrize("kind,dims,np_dtype", [
    ("c2c", [70, 48, 105], np.complex64),
    ("r2c", [60, 42, 35], np.float32),
    ("c2c", [512, 24, 40], np.complex128),
    ("r2r", [40, 36, 30], np.float64),
])
def test_exhaustive_fft_step_autotune(dt, orc, cuda, kind, dims, np_dtype):
    """EXHAUSTIVE plans time every candidate kernel / tile shape / radix
    schedule of each FFT step (dtfft_gb_tune_records lists the choices) and
    still compute the oracle's spectrum."""
    import ctypes
    prec = dt.Precision.SINGLE if np_dtype in (np.complex64, np.float32) else dt.Precision.DOUBLE
    L = dt.lib()
    L.dtfft_gb_tune_records.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
    n0 = ctypes.c_size_t()
    assert L.dtfft_gb_tune_records(None, 0, ctypes.byref(n0)) == 0
    kinds = None
    if kind == "c2c":
        plan = dt.PlanC2C(dims, precision=prec, executor=dt.Executor.CUFFT, effort=dt.Effort.EXHAUSTIVE)
        cdt = np_dtype
    elif kind == "r2c":
        plan = dt.PlanR2C(dims, precision=prec, executor=dt.Executor.CUFFT, effort=dt.Effort.EXHAUSTIVE)
        cdt = np.complex64
    else:
        kinds = [dt.R2RKind.DCT_2, dt.R2RKind.DST_4, dt.R2RKind.DCT_1]
        plan = dt.PlanR2R(dims, kinds, precision=prec, executor=dt.Executor.VKFFT, effort=dt.Effort.EXHAUSTIVE)
        cdt = np_dtype
    n1 = ctypes.c_size_t()
    assert L.dtfft_gb_tune_records(None, 0, ctypes.byref(n1)) == 0
    buf = ctypes.create_string_buffer(n1.value)
    assert L.dtfft_gb_tune_records(buf, n1.value, ctypes.byref(n1)) == 0
    import json
    recs = json.loads(buf.value.decode())
    assert recs and all(r["chosen_ms"] > 0 for r in recs)
    g = random_global(tuple(dims[::-1]), np_dtype, seed=23, dist="normal")
    x = orc.global_to_packed(g, 3, [1, 1, 1], 1)
    a = to_dev(x, plan.alloc_size, cuda)
    b = empty(plan.alloc_size, cdt, cuda)
    plan.execute(a, b, dt.Execute.FORWARD)
    ok = [int(k) for k in kinds] if kinds else None
    expect = orc.global_to_packed(orc.forward_values(g, kind, ok), 3, [1, 1, 1], _final_layout(plan, 3))
    assert orc.rel_l2(from_dev(b, expect.size, cdt), expect) <= TOL[np_dtype]
    plan.destroy()
