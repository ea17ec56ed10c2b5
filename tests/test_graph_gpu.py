"""dtfft_execute inside a CUDA graph: after one warm-up execute (which makes the
plan's aux buffer, as the reference's first execute does), a forward + backward
pair captured on the plan's stream replays with the same results as eager
execution, and each replay reads the buffers' current contents.

The reference leaves capture to the caller (one stream per plan,
src/dtfft_plan.F90:599-693); the library keeps every allocation and attribute
call out of execute so that the stream-ordered work is all there is."""
import numpy as np
import pytest

from gpu_util import random_global

pytestmark = pytest.mark.gpu

CASES = [([64, 48, 40], [1, 2, 2], "c2c", "single"),
         ([256, 256], [1, 1], "c2c", "double"),          # 2D c128 256x256, one process
         ([96, 64, 512], [1, 2, 4], "r2c", "single"),
         ([48, 40, 36], [1, 1, 4], "c2c", "double")]     # Z-slab grid


@pytest.mark.parametrize("dims,grid,kind,prec", CASES)
def test_captured_execute_matches_eager(dt, orc, cuda, dims, grid, kind, prec):
    import torch
    s = torch.cuda.Stream(device=cuda)
    comm = dt.COMM_WORLD if all(g == 1 for g in grid) else dt.cart_comm(grid)
    p = dt.Precision.SINGLE if prec == "single" else dt.Precision.DOUBLE
    cfg = dt.Config(stream=s, enable_z_slab=True)
    if kind == "c2c":
        plan = dt.PlanC2C(dims, comm=comm, precision=p, executor=dt.Executor.CUFFT, config=cfg)
    else:
        plan = dt.PlanR2C(dims, comm=comm, precision=p, executor=dt.Executor.CUFFT, config=cfg)
    cdt = torch.complex64 if prec == "single" else torch.complex128
    rdt = torch.float32 if prec == "single" else torch.float64
    n = plan.alloc_size
    in_t = cdt if kind == "c2c" else rdt
    nd = len(dims)
    x0 = random_global(tuple(dims[::-1]), np.complex128 if kind == "c2c" else np.float64, seed=5)
    x1 = random_global(tuple(dims[::-1]), np.complex128 if kind == "c2c" else np.float64, seed=6)
    lay = 1
    pin0 = orc.global_to_packed(x0, nd, grid, lay)
    pin1 = orc.global_to_packed(x1, nd, grid, lay)
    a = torch.zeros(n, dtype=in_t, device=cuda)
    b = torch.zeros(n if kind == "c2c" else n // 2, dtype=cdt, device=cuda)
    c = torch.zeros(n, dtype=in_t, device=cuda)
    src = torch.zeros(n, dtype=in_t, device=cuda)

    def load(pin):
        src.zero_()
        src[: pin.size] = torch.from_numpy(pin).to(device=cuda, dtype=in_t)
        a.copy_(src)
        torch.cuda.synchronize()

    # eager reference results
    eager = []
    for pin in (pin0, pin1):
        load(pin)
        plan.execute(a, b, dt.Execute.FORWARD)
        plan.execute(b, c, dt.Execute.BACKWARD)
        torch.cuda.synchronize()
        eager.append((b.cpu().numpy().copy(), c.cpu().numpy().copy()))

    launches0 = dt.kernel_launches()
    g = torch.cuda.CUDAGraph()
    load(pin0)
    with torch.cuda.graph(g, stream=s):
        plan.execute(a, b, dt.Execute.FORWARD)
        plan.execute(b, c, dt.Execute.BACKWARD)
    per_pair = dt.kernel_launches() - launches0
    assert per_pair > 0
    for k, pin in enumerate((pin0, pin1, pin0)):
        load(pin)
        b.zero_()
        c.zero_()
        torch.cuda.synchronize()
        g.replay()
        torch.cuda.synchronize()
        eb, ec = eager[k % 2]
        # the same kernels on the same data: bit-identical to eager execution
        assert np.array_equal(b.cpu().numpy(), eb)
        assert np.array_equal(c.cpu().numpy(), ec)
    # and the eager result is the transform (round trip within tolerance)
    tol = 1e-5 if prec == "single" else 1e-12
    back = eager[1][1][: pin1.size] / float(np.prod(dims))
    assert orc.rel_l2(back, pin1) <= tol
    assert dt.kernel_launches() - launches0 == per_pair   # replays launch nothing through the library
    del g
    plan.destroy()
