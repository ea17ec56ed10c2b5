"""Tensor-core form of the complex FP32 row FFT (dtfft_gb_set_fft_form(1)):
rows of 256 / 512 / 768 / 1024 points as two DFT-matrix GEMM stages on
tcgen05 with FP16 hi + lo operands.  Each case states its error against the
FP64 oracle (numpy) and must stay within the FP32 bar (rel-L2 <= 1e-5), on
inputs uniform[-1,1) plus 1e3-amplitude spikes at 0.1% of the points."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _signal(shape, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)
    n = x.size
    idx = rng.choice(n, max(1, n // 1000), replace=False)
    x.ravel()[idx] *= 1e3
    return x.astype(np.complex64)


@pytest.fixture
def tc_form(dt):
    L = dt.lib()
    L.dtfft_gb_set_fft_form.argtypes = [ctypes.c_int32]
    old = L.dtfft_gb_get_fft_form()
    assert L.dtfft_gb_set_fft_form(1) == 0
    yield L
    L.dtfft_gb_set_fft_form(old)


def _kernel_names(L):
    names = []
    for i in range(L.dtfft_gb_profile_count()):
        buf = ctypes.create_string_buffer(128)
        n = ctypes.c_int64()
        ms = ctypes.c_double()
        L.dtfft_gb_profile_get(i, buf, 128, ctypes.byref(n), ctypes.byref(ms))
        names.append(buf.value.decode())
    return names


# (256, 7301) and (1024, 3651): about three tiles per CTA of the 304-CTA grid
# with a ragged last tile (each CTA loads its next tile while the current one
# multiplies)
@pytest.mark.parametrize("n,howmany", [(256, 1000), (512, 333), (768, 130), (1024, 67), (512, 3),
                                       (256, 7301), (1024, 3651)])
def test_tc_rows_match_fp64(dt, cuda, tc_form, n, howmany):
    import torch
    L = tc_form
    L.dtfft_gb_profile_count.restype = ctypes.c_int32
    h = ctypes.c_void_p()
    sizes = (ctypes.c_int32 * 1)(n)
    assert L.gb_fft_create(1, 0, 0, n, n, howmany, sizes, sizes, sizes, None, None, ctypes.byref(h)) == 0
    x = _signal((howmany, n), seed=n + howmany)
    a = torch.from_numpy(x).to(cuda)
    b = torch.empty_like(a)
    torch.cuda.synchronize()
    L.dtfft_gb_profile_start()
    assert L.gb_fft_execute(h, a.data_ptr(), b.data_ptr(), -1) == 0
    torch.cuda.synchronize()
    L.dtfft_gb_profile_stop()
    assert any(nm.startswith("ffttc_rows_c2c_m%d" % n) for nm in _kernel_names(L))
    assert L.dtfft_gb_device_status(1) == 0
    ref = np.fft.fft(x.astype(np.complex128), axis=1)
    err = np.linalg.norm(b.cpu().numpy() - ref) / np.linalg.norm(ref)
    print(f"tensor-core rows m={n}: forward rel-L2 vs FP64 = {err:.3e}")
    assert err <= TOL
    assert L.gb_fft_execute(h, b.data_ptr(), b.data_ptr(), 1) == 0     # in place, backward
    torch.cuda.synchronize()
    back = b.cpu().numpy() / n
    rt = np.linalg.norm(back - x) / np.linalg.norm(x)
    print(f"tensor-core rows m={n}: round trip rel-L2 = {rt:.3e}")
    assert rt <= TOL
    assert L.dtfft_gb_device_status(1) == 0
    assert L.gb_fft_destroy(ctypes.byref(h)) == 0


# The fused FFT + transpose passes stay on the FP32 kernels; the plain row
# passes left over (the forward Z rows of these one-process Z-slab plans) run
# on tensor cores where Z has a tensor-core length.
@pytest.mark.parametrize("dims", [[512, 40, 48], [768, 36, 32], [1024, 24, 20],
                                  [40, 48, 512], [36, 32, 768], [24, 20, 1024]])
def test_tc_plan_forward_matches_fp64(dt, cuda, tc_form, dims):
    import torch
    L = tc_form
    L.dtfft_gb_profile_count.restype = ctypes.c_int32
    plan = dt.PlanC2C(dims, precision=dt.Precision.SINGLE, executor=dt.Executor.CUFFT)
    n = plan.alloc_size
    g = _signal(tuple(dims[::-1]), seed=sum(dims))
    a = torch.zeros(n, dtype=torch.complex64, device=cuda)
    a[: g.size] = torch.from_numpy(g.ravel()).to(cuda)
    b = torch.zeros_like(a)
    torch.cuda.synchronize()
    L.dtfft_gb_profile_start()
    plan.execute(a, b, dt.Execute.FORWARD)
    torch.cuda.synchronize()
    L.dtfft_gb_profile_stop()
    if dims[2] in (256, 512, 768, 1024):
        assert any(nm.startswith("ffttc_rows_c2c_m%d" % dims[2]) for nm in _kernel_names(L))
    assert L.dtfft_gb_device_status(1) == 0
    ref = np.fft.fftn(g.astype(np.complex128))
    # Z pencils of a one-process plan: (Z, X, Y) with Z fastest
    ref = ref.transpose(1, 2, 0).ravel()
    got = b.cpu().numpy()[: ref.size]
    err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    print(f"tensor-core plan {dims}: forward rel-L2 vs FP64 = {err:.3e}")
    assert err <= TOL
    plan.destroy()
