"""Every 7-smooth transform length in 24..384 (the edges of the batched
workload and their R2C half lengths) through the FFT plug-in, rows and
columns, single and double precision, against the FP64 oracle (numpy):
rel-L2 <= 1e-5 single, <= 1e-12 double."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def smooth(lo, hi):
    out = []
    for n in range(lo, hi + 1):
        m = n
        for p in (2, 3, 5, 7):
            while m % p == 0:
                m //= p
        if m == 1:
            out.append(n)
    return out


LENGTHS = smooth(24, 384)
TOL = {0: 1e-5, 1: 1e-12}


def _run(dt, cuda, n_fast, n_slow, howmany, prec):
    import torch
    L = dt.lib()
    h = ctypes.c_void_p()
    rank = 1 if n_slow == 1 else 2
    sizes = (ctypes.c_int32 * 2)(*([n_fast, 0] if rank == 1 else [n_slow, n_fast]))
    per = n_fast * n_slow
    assert L.gb_fft_create(rank, 0, prec, per, per, howmany, sizes, sizes, sizes, None, None, ctypes.byref(h)) == 0
    rng = np.random.default_rng(n_fast * 7 + n_slow)
    shape = (howmany, n_slow, n_fast) if rank == 2 else (howmany, n_fast)
    x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    x = x.astype(np.complex64 if prec == 0 else np.complex128)
    a = torch.from_numpy(x).to(cuda)
    b = torch.empty_like(a)
    torch.cuda.synchronize()
    assert L.gb_fft_execute(h, a.data_ptr(), b.data_ptr(), -1) == 0
    torch.cuda.synchronize()
    axes = (1, 2) if rank == 2 else (1,)
    ref = np.fft.fftn(x.astype(np.complex128), axes=axes)
    err = np.linalg.norm(b.cpu().numpy() - ref) / np.linalg.norm(ref)
    assert err <= TOL[prec], (n_fast, n_slow, err)
    assert L.gb_fft_destroy(ctypes.byref(h)) == 0


@pytest.mark.parametrize("n", LENGTHS)
@pytest.mark.parametrize("prec", [0, 1])
def test_rows(dt, cuda, n, prec):
    _run(dt, cuda, n, 1, 37, prec)


@pytest.mark.parametrize("n", LENGTHS)
def test_columns(dt, cuda, n):
    # rank-2: rows of 6 points, then the in-place column pass of length n
    _run(dt, cuda, 6, n, 5, 0)
