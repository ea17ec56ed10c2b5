"""dtfft_gb_batch_*: plans of mixed kinds, shapes, precisions and grids run as
one CUDA graph give the same bytes as one dtfft_execute per plan, replays
follow the buffers' contents, and new buffers are picked up by a new capture."""
import numpy as np
import pytest

from gpu_util import random_global

pytestmark = pytest.mark.gpu


def _plans(dt):
    mk = []
    sp, dp = dt.Precision.SINGLE, dt.Precision.DOUBLE
    cu = dt.Executor.CUFFT
    mk.append(("c2c", np.complex64, dt.PlanC2C([48, 40, 36], precision=sp, executor=cu)))
    mk.append(("r2c", np.float32, dt.PlanR2C([60, 42, 50], precision=sp, executor=cu)))
    mk.append(("c2c", np.complex128, dt.PlanC2C([256, 256], precision=dp, executor=cu)))
    mk.append(("c2c", np.complex64, dt.PlanC2C([64, 48, 40], comm=dt.cart_comm([1, 2, 2]), precision=sp,
                                               executor=cu)))
    mk.append(("r2r", np.float64, dt.PlanR2R([30, 28, 40], kinds=[dt.R2RKind.DCT_2] * 3, precision=dp,
                                             executor=dt.Executor.VKFFT)))
    mk.append(("c2c", np.complex64, dt.PlanC2C([50, 54, 56], precision=sp)))           # transpose only
    return mk


def test_batch_matches_per_plan_execute(dt, cuda):
    import torch
    tdt = {np.complex64: torch.complex64, np.complex128: torch.complex128, np.float32: torch.float32,
           np.float64: torch.float64}
    cplx = {np.float32: torch.complex64, np.float64: torch.complex128}
    plans = _plans(dt)
    ins, outs, backs, refs = [], [], [], []
    for k, (kind, npd, p) in enumerate(plans):
        n = p.alloc_size
        x = random_global((n,), npd, seed=k)
        ins.append(torch.from_numpy(x).to(cuda))
        odt = cplx[npd] if kind == "r2c" else tdt[npd]
        outs.append(torch.zeros(n // 2 if kind == "r2c" else n, dtype=odt, device=cuda))
        backs.append(torch.zeros(n, dtype=tdt[npd], device=cuda))
    torch.cuda.synchronize()
    # eager reference, one plan after the other (the inputs are kept: execute may clobber them)
    for (kind, npd, p), a, b, c in zip(plans, ins, outs, backs):
        a2 = a.clone()
        torch.cuda.synchronize()
        p.execute(a2, b, dt.Execute.FORWARD)
        torch.cuda.synchronize()
        b2 = b.clone()
        torch.cuda.synchronize()
        p.execute(b2, c, dt.Execute.BACKWARD)
        torch.cuda.synchronize()
        refs.append((b.cpu().numpy().copy(), c.cpu().numpy().copy()))

    batch = dt.Batch([p for _, _, p in plans], lanes=3)
    work = [a.clone() for a in ins]
    for rep in range(3):
        for w, a in zip(work, ins):
            w.copy_(a)
        for b, c in zip(outs, backs):
            b.zero_()
            c.zero_()
        torch.cuda.synchronize()
        batch.execute(work, outs, dt.Execute.FORWARD)
        torch.cuda.synchronize()
        for (rb, _), b in zip(refs, outs):
            assert np.array_equal(b.cpu().numpy(), rb)
        work_b = [b.clone() for b in outs]
        torch.cuda.synchronize()
        batch.execute(work_b, backs, dt.Execute.BACKWARD)      # new buffers: captured again
        torch.cuda.synchronize()
        for (_, rc), c in zip(refs, backs):
            assert np.array_equal(c.cpu().numpy(), rc)
    assert batch.graph_nodes > len(plans)
    batch.destroy()
    for _, _, p in plans:
        p.destroy()


def test_batch_replay_follows_contents(dt, cuda):
    import torch
    p = dt.PlanC2C([40, 36, 32], precision=dt.Precision.DOUBLE, executor=dt.Executor.CUFFT)
    n = p.alloc_size
    a = torch.zeros(n, dtype=torch.complex128, device=cuda)
    b = torch.zeros_like(a)
    batch = dt.Batch([p])
    outs = []
    for seed in (1, 2):
        x = random_global((n,), np.complex128, seed=seed)
        a.copy_(torch.from_numpy(x).to(cuda))
        torch.cuda.synchronize()
        batch.execute([a], [b], dt.Execute.FORWARD)
        torch.cuda.synchronize()
        outs.append(b.cpu().numpy().copy())
        # Z-slab plan: output in Z pencils (Z, X, Y)
        ref = np.fft.fftn(x.reshape(32, 36, 40)).transpose(1, 2, 0).ravel()
        assert np.linalg.norm(outs[-1] - ref) / np.linalg.norm(ref) <= 1e-12
    assert not np.array_equal(outs[0], outs[1])
    batch.destroy()
    p.destroy()


def test_plans_sharing_a_kernel_keep_their_smem_limits(dt, cuda):
    """Two plans whose column FFTs use the same kernel with different shared
    memory: the second plan's creation must not lower the first one's limit."""
    import torch
    big = dt.PlanC2C([48, 384, 64], precision=dt.Precision.SINGLE, executor=dt.Executor.CUFFT)
    small = dt.PlanC2C([48, 98, 64], precision=dt.Precision.SINGLE, executor=dt.Executor.CUFFT)
    for p, dims in ((big, [48, 384, 64]), (small, [48, 98, 64]), (big, [48, 384, 64])):
        n = p.alloc_size
        x = random_global((n,), np.complex64, seed=n)
        a = torch.from_numpy(x).to(cuda)
        b = torch.zeros_like(a)
        torch.cuda.synchronize()
        p.execute(a, b, dt.Execute.FORWARD)
        torch.cuda.synchronize()
        g = x[: int(np.prod(dims))].astype(np.complex128).reshape(dims[::-1])
        ref = np.fft.fftn(g).transpose(1, 2, 0).ravel()
        got = b.cpu().numpy()[: ref.size]
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= 1e-5
    big.destroy()
    small.destroy()
