"""dtfft_execute_noalloc through the C ABI.

dtfft_execute_noalloc serves callers that cannot allocate device memory (their
memory belongs to another allocator, or they cannot take a first-use
cudaMalloc): it runs the execute schedule with scratch taken from a fixed
16 MiB buffer compiled into the library.  Its output must match
dtfft_execute's on the same input, on two calls in a row (the buffer keeps the
previous call's contents), and plans needing more scratch are refused.

This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_SINGLE = 1e-5


def _lib(dt):
    L = dt.lib()
    L.dtfft_execute_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    L.dtfft_execute_noalloc.restype = ctypes.c_int
    L.dtfft_execute_noalloc_max_bytes.restype = ctypes.c_size_t
    return L


def test_noalloc_matches_execute_twice(dt, cuda):
    import torch
    L = _lib(dt)
    assert L.dtfft_execute_noalloc_max_bytes() == 16 << 20
    dims = [48, 40, 36]
    plan = dt.PlanC2C(dims, comm=dt.cart_comm([1, 2, 2]), precision=dt.Precision.SINGLE,
                      executor=dt.Executor.CUFFT)
    assert plan.aux_bytes <= L.dtfft_execute_noalloc_max_bytes()
    n = plan.alloc_size
    rng = np.random.default_rng(4)
    x = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex64)
    src = torch.from_numpy(x).to(cuda)
    a = src.clone()
    ref = torch.empty_like(src)
    torch.cuda.synchronize()
    plan.execute(a, ref, dt.Execute.FORWARD)          # existing entry point, plan-owned aux
    torch.cuda.synchronize()
    ref_h = ref.cpu().numpy()
    for call in range(2):
        a = src.clone()
        out = torch.full_like(src, float("nan"))
        torch.cuda.synchronize()
        rc = L.dtfft_execute_noalloc(plan._h, a.data_ptr(), out.data_ptr(), int(dt.Execute.FORWARD))
        assert rc == 0, rc
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        err = np.linalg.norm(got - ref_h) / np.linalg.norm(ref_h)
        assert err <= TOL_SINGLE, (call, err)
    # the backward direction through the same buffer returns the input (scaled)
    back = torch.empty_like(src)
    torch.cuda.synchronize()
    assert L.dtfft_execute_noalloc(plan._h, out.data_ptr(), back.data_ptr(), int(dt.Execute.BACKWARD)) == 0
    torch.cuda.synchronize()
    rt = back.cpu().numpy() / np.prod(dims)
    assert np.linalg.norm(rt - x) / np.linalg.norm(x) <= TOL_SINGLE
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
