"""Parity at the full sizes of the benchmark configurations.

The other GPU tests compare with the oracle at sizes it finishes in
milliseconds; these run the benchmarked plans themselves:

- 512^3 complex64 on the 2x4 virtual grid: the four grid transposes
  X->Y->Z->Y->X bit-exact against the oracle's restatement of the reference's
  pack -> all-to-all-v -> unpack (1 GiB per buffer), and the forward spectrum
  of the fused execute against a full FP64 FFT (rel-L2 <= 1e-5);
- R2C float64 1024x1024x512 on the 4x4 grid and the DCT-II R2R plan of the
  same grid: lines of the forward spectrum along X, Y and Z (edges and
  interior frequencies) against the FP64 line oracle (rel-L2 <= 1e-12);
- complex64 768^3 and 1024^3 (uniform[-1,1) plus 1e3 spikes at 0.1 % of the
  points), FP32 Stockham and tensor-core forms: sampled lines against FP64
  (rel-L2 <= 1e-5);
- the first C2C and the first R2C member of the 64-transform batch, run
  through one batch graph, against the full FP64 transform.
"""
import os

import numpy as np
import pytest

from gpu_util import from_dev, to_dev

pytestmark = pytest.mark.gpu

WORKERS = os.cpu_count() or 1


def _uniform_c64(shape, seed):
    rng = np.random.default_rng(seed)
    g = np.empty(shape, np.complex64)
    flat = g.reshape(-1)
    step = 1 << 24
    for i in range(0, flat.size, step):
        n = min(step, flat.size - i)
        flat[i:i + n].real = rng.uniform(-1, 1, n)
        flat[i:i + n].imag = rng.uniform(-1, 1, n)
    return g


def _normal_f64(shape, seed):
    return np.random.default_rng(seed).standard_normal(shape)


def _gather(buf, idx, cuda):
    """Values of a device buffer at host-computed positions."""
    import torch
    t = torch.from_numpy(np.ascontiguousarray(idx)).to(cuda)
    return buf.index_select(0, t).cpu().numpy()


def _lines_points(n):
    """Sampled fixed-index pairs: the zero and last indices and interior ones."""
    nx, ny, nz = n
    return {0: [(0, 0), (ny - 1, nz // 2), (ny // 3, 1), (7, nz - 1)],        # X lines at (ky, kz)
            1: [(0, 0), (nx - 1, nz // 3), (nx // 2, 5), (3, nz - 1)],        # Y lines at (kx, kz)
            2: [(0, 0), (nx - 1, ny - 1), (nx // 2, ny // 5), (11, 1)]}       # Z lines at (kx, ky)


def _check_lines(orc, g, kind, kinds, out_dev, gdims_out, grid, layout, cuda, tol):
    """rel-L2 of the device's forward spectrum over the sampled lines."""
    got_all, ref_all = [], []
    for axis, pts in _lines_points(gdims_out).items():
        ref = orc.sampled_lines(g, kind, axis, pts, kinds)
        for i, p in enumerate(pts):
            co = orc.line_coords(axis, p, gdims_out[axis])
            idx = orc.packed_index(3, gdims_out, grid, layout, co)
            got_all.append(_gather(out_dev, idx, cuda))
            ref_all.append(ref[i])
    err = orc.rel_l2(np.concatenate(got_all), np.concatenate(ref_all))
    assert err <= tol, err
    return err


def test_c2c_512cube_grid2x4_transposes_bit_exact(dt, orc, cuda):
    import torch
    dims, grid = [512, 512, 512], [1, 2, 4]
    plan = dt.PlanC2C(dims, comm=dt.cart_comm(grid), precision=dt.Precision.SINGLE, executor=dt.Executor.CUFFT)
    g = _uniform_c64(tuple(dims[::-1]), seed=2)
    x = orc.global_to_packed(g, 3, grid, 1)
    del g
    cur = x
    a = to_dev(x, plan.alloc_size, cuda)
    b = torch.empty_like(a)
    for t in (1, 2, -2, -1):
        expect = orc.vgrid_transpose(3, dims, grid, t, cur)
        b.fill_(float("nan"))
        torch.cuda.synchronize()
        plan.transpose(a, b, dt.Transpose(t))
        got = from_dev(b, expect.size, np.complex64)
        assert got.view(np.uint64).tobytes() == expect.view(np.uint64).tobytes(), f"transpose {t}"
        cur = expect
        a, b = b, a
    assert np.array_equal(cur, x)
    plan.destroy()


def test_c2c_512cube_grid2x4_forward_spectrum(dt, orc, cuda):
    import scipy.fft as sf
    import torch
    dims, grid = [512, 512, 512], [1, 2, 4]
    plan = dt.PlanC2C(dims, comm=dt.cart_comm(grid), precision=dt.Precision.SINGLE, executor=dt.Executor.CUFFT)
    g = _uniform_c64(tuple(dims[::-1]), seed=2)
    x = orc.global_to_packed(g, 3, grid, 1)
    a = to_dev(x, plan.alloc_size, cuda)
    b = torch.empty_like(a)
    plan.execute(a, b, dt.Execute.FORWARD)
    got = orc.packed_to_global(from_dev(b, x.size, np.complex64), 3, dims, grid, 3)
    ref = sf.fftn(g.astype(np.complex128), workers=WORKERS)
    del g
    err = float(np.linalg.norm((got - ref).ravel()) / np.linalg.norm(ref.ravel()))
    assert err <= 1e-5, err
    del got, ref
    # backward returns the input (scaled by N)
    plan.execute(b, a, dt.Execute.BACKWARD)
    back = from_dev(a, x.size, np.complex64)
    err_rt = orc.rel_l2(back.astype(np.complex128) / np.prod(dims), x)
    assert err_rt <= 1e-5, err_rt
    plan.destroy()


@pytest.mark.parametrize("kind", ["r2c", "r2r_dct2"])
def test_f64_1024x1024x512_grid4x4_lines(dt, orc, cuda, kind):
    import torch
    dims, grid = [1024, 1024, 512], [1, 4, 4]
    comm = dt.cart_comm(grid)
    g = _normal_f64(tuple(dims[::-1]), seed=3)
    x = orc.global_to_packed(g, 3, grid, 1)
    if kind == "r2c":
        plan = dt.PlanR2C(dims, comm=comm, precision=dt.Precision.DOUBLE, executor=dt.Executor.CUFFT)
        out_dims, okind, kinds = [dims[0] // 2 + 1, dims[1], dims[2]], "r2c", None
        b = torch.empty(plan.alloc_size // 2, dtype=torch.complex128, device=cuda)
    else:
        kinds = [dt.R2RKind.DCT_2] * 3
        plan = dt.PlanR2R(dims, kinds=kinds, comm=comm, precision=dt.Precision.DOUBLE, executor=dt.Executor.VKFFT)
        out_dims, okind, kinds = list(dims), "r2r", [int(k) for k in kinds]
        b = torch.empty(plan.alloc_size, dtype=torch.float64, device=cuda)
    a = to_dev(x, plan.alloc_size, cuda)
    del x
    plan.execute(a, b, dt.Execute.FORWARD)
    torch.cuda.synchronize()
    _check_lines(orc, g, okind, kinds, b, out_dims, grid, 3, cuda, 1e-12)
    plan.destroy()


@pytest.mark.parametrize("n", [768, 1024])
def test_c2c_cube_with_spikes_fp32_and_tensor_core_lines(dt, orc, cuda, n):
    import ctypes
    import torch
    L = dt.lib()
    L.dtfft_gb_set_fft_form.argtypes = [ctypes.c_int32]
    dims = [n, n, n]
    gen = torch.Generator(device=cuda)
    gen.manual_seed(4)
    npts = n ** 3
    x0 = torch.complex(torch.rand(npts, device=cuda, generator=gen) * 2 - 1,
                       torch.rand(npts, device=cuda, generator=gen) * 2 - 1)
    spikes = torch.randint(0, npts, (npts // 1000,), device=cuda, generator=gen)
    x0[spikes] *= 1e3
    g = x0.cpu().numpy().reshape(n, n, n)            # one process: the X pencil is the global array
    errs = {}
    try:
        for form in (0, 1):
            L.dtfft_gb_set_fft_form(form)
            plan = dt.PlanC2C(dims, precision=dt.Precision.SINGLE, executor=dt.Executor.CUFFT)
            L.dtfft_gb_set_fft_form(0)
            assert plan.z_slab_enabled
            a = x0.clone()
            b = torch.empty_like(a)
            torch.cuda.synchronize()
            plan.execute(a, b, dt.Execute.FORWARD)
            torch.cuda.synchronize()
            errs[form] = _check_lines(orc, g, "c2c", None, b, dims, [1, 1, 1], 3, cuda, 1e-5)
            del a, b
            plan.destroy()
    finally:
        L.dtfft_gb_set_fft_form(0)
    assert errs[0] < 1e-6


def _batch_shapes():
    """The batch workload's shapes (7-smooth edges in 48..384, PCG64 seed 5,
    alternating C2C / R2C)."""
    edges = [m for m in range(48, 385) if _smooth(m)]
    rng = np.random.default_rng(5)
    return [("c2c" if i % 2 == 0 else "r2c", [int(rng.choice(edges)) for _ in range(3)]) for i in range(64)]


def _smooth(m):
    for q in (2, 3, 5, 7):
        while m % q == 0:
            m //= q
    return m == 1


def test_batch_members_against_fp64(dt, orc, cuda):
    import torch
    shapes = _batch_shapes()
    picks = [shapes[0], shapes[1]]               # first C2C and first R2C member
    plans, ins, outs, gs = [], [], [], []
    for i, (kind, dims) in enumerate(picks):
        mk = dt.PlanC2C if kind == "c2c" else dt.PlanR2C
        p = mk(dims, precision=dt.Precision.SINGLE, executor=dt.Executor.CUFFT, effort=dt.Effort.EXHAUSTIVE)
        rng = np.random.default_rng(100 + i)
        shape = tuple(dims[::-1])
        if kind == "c2c":
            g = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
            o = torch.empty(p.alloc_size, dtype=torch.complex64, device=cuda)
        else:
            g = rng.standard_normal(shape).astype(np.float32)
            o = torch.empty(p.alloc_size // 2, dtype=torch.complex64, device=cuda)
        ins.append(to_dev(g.ravel(), p.alloc_size, cuda))
        outs.append(o)
        plans.append(p)
        gs.append(g)
    batch = dt.Batch(plans, lanes=2)
    batch.execute(ins, outs, dt.Execute.FORWARD)
    torch.cuda.synchronize()
    for (kind, dims), p, o, g in zip(picks, plans, outs, gs):
        ref = orc.forward_values(g, kind)
        expect = orc.global_to_packed(ref, 3, [1, 1, 1], 3)   # forward ends in Z pencils
        err = orc.rel_l2(from_dev(o, expect.size, np.complex64), expect)
        assert err <= 1e-5, (kind, dims, err)
    batch.destroy()
    for p in plans:
        p.destroy()
