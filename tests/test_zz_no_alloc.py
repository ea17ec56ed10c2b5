"""dtfft_execute_noalloc through the C ABI.

dtfft_execute_noalloc serves callers that cannot allocate device memory (their
memory belongs to another allocator, or they cannot take a first-use
cudaMalloc): it runs the execute schedule with scratch taken from a fixed
16 MiB buffer compiled into the library.  Both entry points run the same
kernels on the same inputs, so the output must equal dtfft_execute's bit for
bit, on two calls in a row.  Before every call the shared buffer is filled
with NaNs (a 16 MiB plan runs on NaN input through the same entry point), so
a schedule that read scratch it had not written would show it.  Plans needing
more scratch than the buffer are refused.

Cases: out-of-place and in-place generic C2C, a plan whose X and Y passes run
the fused tile FFT + transpose kernel, a transpose-only plan (TMA transposes),
R2C, R2R, a Z-slab plan and a plan on the fused two-factor passes.

This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lib(dt):
    L = dt.lib()
    L.dtfft_execute_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    L.dtfft_execute_noalloc.restype = ctypes.c_int
    L.dtfft_execute_noalloc_max_bytes.restype = ctypes.c_size_t
    return L


def _poison_scratch(dt, L, cuda):
    """Leave NaNs in every byte of the shared 16 MiB buffer: a plan whose aux
    is the whole buffer, run on NaN input through dtfft_execute_noalloc."""
    import torch
    plan = dt.PlanC2C([256, 128, 64], comm=dt.cart_comm([1, 2, 2]), precision=dt.Precision.SINGLE,
                      executor=dt.Executor.CUFFT)
    assert plan.aux_bytes == L.dtfft_execute_noalloc_max_bytes()
    a = torch.full((plan.alloc_size,), float("nan"), dtype=torch.complex64, device=cuda)
    b = torch.empty_like(a)
    torch.cuda.synchronize()
    assert L.dtfft_execute_noalloc(plan._h, a.data_ptr(), b.data_ptr(), int(dt.Execute.FORWARD)) == 0
    torch.cuda.synchronize()
    plan.destroy()


def _make(dt, case):
    S = dt.Precision.SINGLE
    g22 = dt.cart_comm([1, 2, 2])
    if case in ("c2c", "c2c_inplace"):
        return dt.PlanC2C([48, 40, 36], comm=g22, precision=S, executor=dt.Executor.CUFFT), np.complex64, np.complex64
    if case == "c2c_fused_tile":
        return dt.PlanC2C([256, 256, 16], comm=g22, precision=S, executor=dt.Executor.CUFFT), np.complex64, np.complex64
    if case == "transpose_only":
        return dt.PlanC2C([128, 96, 64], comm=g22, precision=S, executor=dt.Executor.NONE), np.complex64, np.complex64
    if case == "r2c":
        return dt.PlanR2C([64, 40, 36], comm=g22, precision=S, executor=dt.Executor.CUFFT), np.float32, np.complex64
    if case == "r2r":
        kinds = [dt.R2RKind.DCT_2, dt.R2RKind.DST_3, dt.R2RKind.DCT_4]
        return (dt.PlanR2R([40, 36, 30], kinds, comm=g22, precision=dt.Precision.DOUBLE,
                           executor=dt.Executor.VKFFT), np.float64, np.float64)
    if case == "z_slab":
        return dt.PlanC2C([64, 48, 40], precision=S, executor=dt.Executor.CUFFT), np.complex64, np.complex64
    if case == "two_factor_fused":
        return dt.PlanC2C([105, 42, 36], comm=g22, precision=S, executor=dt.Executor.CUFFT), np.complex64, np.complex64
    raise ValueError(case)


def _random(n, np_dtype, seed):
    rng = np.random.default_rng(seed)
    if np.issubdtype(np_dtype, np.complexfloating):
        return (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np_dtype)
    return rng.uniform(-1, 1, n).astype(np_dtype)


@pytest.mark.parametrize("case", ["c2c", "c2c_inplace", "c2c_fused_tile", "transpose_only", "r2c", "r2r", "z_slab",
                                  "two_factor_fused"])
def test_noalloc_matches_execute_bit_for_bit(dt, cuda, case):
    import torch
    from tests.gpu_util import torch_dtype
    L = _lib(dt)
    assert L.dtfft_execute_noalloc_max_bytes() == 16 << 20
    plan, in_dt, out_dt = _make(dt, case)
    if case == "z_slab":
        assert plan.z_slab_enabled
    assert plan.aux_bytes <= L.dtfft_execute_noalloc_max_bytes()
    inplace = case == "c2c_inplace"
    # buffers of alloc_size elements of each type (R2C: real in, complex out)
    n_in = plan.alloc_size
    n_out = plan.alloc_size // 2 if case == "r2c" else plan.alloc_size
    x = _random(n_in, in_dt, 4)
    src = torch.from_numpy(x).to(cuda)
    for direction in (dt.Execute.FORWARD, dt.Execute.BACKWARD):
        if direction == dt.Execute.BACKWARD:
            if case == "r2c":
                # backward of an R2C plan: complex in, real out
                src = torch.from_numpy(_random(n_out, out_dt, 5)).to(cuda)
                in_t, out_t, n_o = out_dt, in_dt, n_in
            else:
                src = torch.from_numpy(_random(n_in, in_dt, 5)).to(cuda)
                in_t, out_t, n_o = in_dt, out_dt, n_out
        else:
            in_t, out_t, n_o = in_dt, out_dt, n_out
        a = src.clone()
        if inplace:
            ref = a
        else:
            ref = torch.full((n_o,), float("nan"), dtype=torch_dtype(out_t), device=cuda)
        torch.cuda.synchronize()
        plan.execute(a, ref, direction)                 # existing entry point, plan-owned aux
        torch.cuda.synchronize()
        ref_h = ref.cpu().numpy()
        # the layout the direction ends in is finite; buffer space past it stays NaN in both runs
        _, in_counts, _, out_counts, _ = plan.local_sizes
        n_valid = int(np.prod(out_counts if direction == dt.Execute.FORWARD else in_counts))
        assert np.isfinite(ref_h[:n_valid]).all()
        for call in range(2):
            _poison_scratch(dt, L, cuda)
            a = src.clone()
            out = a if inplace else torch.full((n_o,), float("nan"), dtype=torch_dtype(out_t), device=cuda)
            torch.cuda.synchronize()
            rc = L.dtfft_execute_noalloc(plan._h, a.data_ptr(), out.data_ptr(), int(direction))
            assert rc == 0, rc
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            np.testing.assert_array_equal(got, ref_h, err_msg=f"{case} {direction} call {call}")
    plan.destroy()


def test_noalloc_refuses_plans_larger_than_its_buffer(dt, cuda):
    import torch
    L = _lib(dt)
    plan = dt.PlanC2C([256, 256, 256], precision=dt.Precision.SINGLE, executor=dt.Executor.CUFFT)
    assert plan.aux_bytes > L.dtfft_execute_noalloc_max_bytes()
    a = torch.zeros(8, dtype=torch.complex64, device=cuda)
    b = torch.zeros_like(a)
    assert L.dtfft_execute_noalloc(plan._h, a.data_ptr(), b.data_ptr(), int(dt.Execute.FORWARD)) == 602
    plan.destroy()
