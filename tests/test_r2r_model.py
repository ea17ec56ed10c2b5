"""CPU model of the R2R kinds as a length-m complex core FFT
(dtfft_gb300/csrc/fft_kernels.cuh r2r_pre / r2r_post_src / r2r_post) and of
the Bluestein chirp-z evaluation of that core (fft_bluestein.cu), against
scipy.fft's DCT/DST types I-IV in FFTW's unnormalised conventions (the
reference's executors: src/interfaces/fft/fftw/dtfft_executor_fftw_m.F90 and
src/interfaces/fft/vkfft/dtfft_executor_vkfft_m.F90 accept every R2R kind at
every length).  Core lengths with a prime factor above 127 are the ones the
device runs through Bluestein."""
import numpy as np
import pytest
import scipy.fft as sf

# FFTW kind numbers: REDFT00 .. RODFT11
DCT1, DCT2, DCT3, DCT4, DST1, DST2, DST3, DST4 = 3, 4, 5, 6, 7, 8, 9, 10


def core_geometry(kind, n):
    """(m, sign) of the complex core (fft_host.cu mode_geometry)."""
    return {DCT1: (2 * (n - 1), -1), DST1: (2 * (n + 1), -1), DCT2: (n, -1), DST2: (n, -1),
            DCT3: (n, 1), DST3: (n, 1), DCT4: (2 * n, -1), DST4: (2 * n, -1)}[kind]


def tables(n):
    k = np.arange(n)
    ta = np.exp(-2j * np.pi * k / (4 * n))                 # W_4n^k
    tb = np.exp(-2j * np.pi * (2 * k + 1) / (8 * n))       # W_8n^(2k+1)
    return ta, tb


def r2r_pre(kind, n, m, k, x, ta):
    if kind == DCT1:
        return complex(x[k if k < n else m - k])
    if kind == DST1:
        if 1 <= k <= n:
            return complex(x[k - 1])
        return complex(-x[m - k - 1]) if k >= n + 2 else 0j
    if kind in (DCT2, DST2):
        j = 2 * k if 2 * k < n else 2 * (n - 1 - k) + 1
        t = x[j]
        return complex(-t if (kind == DST2 and j & 1) else t)
    if kind in (DCT3, DST3):
        if kind == DCT3:
            a, b = x[k], (x[n - k] if k > 0 else 0.0)
        else:
            a, b = x[n - 1 - k], (x[k - 1] if k > 0 else 0.0)
        return complex(a, -b) * np.conj(ta[k])
    if k < n:
        return complex(x[k if kind == DCT4 else n - 1 - k]) * ta[k]
    return 0j


def r2r_post_src(kind, n, k):
    if kind == DST1:
        return k + 1
    if kind == DST2:
        return n - 1 - k
    if kind in (DCT3, DST3):
        return n - 1 - (k >> 1) if k & 1 else k >> 1
    return k


def r2r_post(kind, n, k, f, ta, tb):
    if kind == DCT1:
        return f.real
    if kind == DST1:
        return -f.imag
    if kind in (DCT2, DST2):
        p = k if kind == DCT2 else n - 1 - k
        return 2 * (ta[p] * f).real
    if kind == DCT3:
        return f.real
    if kind == DST3:
        return -f.real if k & 1 else f.real
    y = 2 * (tb[k] * f).real
    return -y if (kind == DST4 and k & 1) else y


def core_fft(v, sign):
    return np.fft.fft(v) if sign < 0 else np.fft.ifft(v) * len(v)


def bluestein(v, sign):
    """fft_bluestein.cu: X[k] = w[k] sum_j (v[j] w[j]) conj(w[k-j]),
    w[j] = exp(s pi i j^2 / m), as a circular convolution of power-of-two length L."""
    m = len(v)
    L = 1
    while L < 2 * m - 1:
        L <<= 1
    j = np.arange(m)
    w = np.exp(sign * 1j * np.pi * ((j * j) % (2 * m)) / m)
    c = np.zeros(L, complex)
    c[0] = np.conj(w[0])
    c[1:m] = np.conj(w[1:])
    c[L - m + 1:] = np.conj(w[1:])[::-1]
    a = np.zeros(L, complex)
    a[:m] = v * w
    a = np.fft.ifft(np.fft.fft(a) * np.fft.fft(c))
    return w * a[:m]


def reference(kind, x):
    t = {DCT1: 1, DCT2: 2, DCT3: 3, DCT4: 4, DST1: 1, DST2: 2, DST3: 3, DST4: 4}[kind]
    f = sf.dct if kind <= DCT4 else sf.dst
    return f(x, type=t)


def model(kind, x, chirp):
    n = len(x)
    m, sign = core_geometry(kind, n)
    ta, tb = tables(n)
    v = np.array([r2r_pre(kind, n, m, k, x, ta) for k in range(m)])
    F = bluestein(v, sign) if chirp else core_fft(v, sign)
    return np.array([r2r_post(kind, n, k, F[r2r_post_src(kind, n, k)], ta, tb) for k in range(n)])


@pytest.mark.parametrize("kind", [DCT1, DCT2, DCT3, DCT4, DST1, DST2, DST3, DST4])
@pytest.mark.parametrize("n", [5, 8, 17, 24])
def test_pre_post_around_the_core_fft_is_the_kind(kind, n):
    x = np.random.default_rng(n + kind).standard_normal(n)
    ref = reference(kind, x)
    got = model(kind, x, chirp=False)
    assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref)


@pytest.mark.parametrize("kind,n", [(DCT1, 132), (DST1, 130), (DCT2, 131), (DST2, 131), (DCT3, 139),
                                    (DST3, 131), (DCT4, 131), (DST4, 131), (DCT3, 262)])
def test_bluestein_core_gives_the_kind(kind, n):
    """Core lengths with a prime factor above 127 (131, 139, 262 = 2 x 131)."""
    m, _ = core_geometry(kind, n)
    p = m
    for q in range(2, 128):
        while p % q == 0:
            p //= q
    assert p > 127
    x = np.random.default_rng(n * kind).standard_normal(n)
    ref = reference(kind, x)
    got = model(kind, x, chirp=True)
    assert np.linalg.norm(got - ref) <= 1e-11 * np.linalg.norm(ref)
