"""CPU model of the two-factor FFT kernel (dtfft_gb300/csrc/fft_2f.cuh): the
in-register codelets (recursive Cooley-Tukey with the split rule of
codelet_split), the four-step decomposition of a length m = M1 * M2 across
phases A and B, the intermediate's shared-memory layouts, and the
compile-time twiddle constants of ktrig.h (compiled with g++ and compared
with libm)."""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "dtfft_gb300", "csrc")
DIRECT = (2, 3, 4, 5, 7, 8, 16)


def codelet_split(n):
    for p in (16, 8, 7, 5, 4, 3, 2):
        if n % p == 0 and n > p:
            return p
    return n


def dftc(v, s):
    """dftc<R, N>: natural order in and out, v[k] = sum_j v[j] exp(s 2 pi i j k / N)."""
    n = len(v)
    if n == 1:
        return v.copy()
    if n in DIRECT:
        k = np.arange(n)
        return np.exp(s * 2j * np.pi * np.outer(k, k) / n) @ v
    p = codelet_split(n)
    q = n // p
    a = np.empty((q, p), complex)
    for qq in range(q):
        a[qq] = dftc(v[qq + q * np.arange(p)], s)
        a[qq] *= np.exp(s * 2j * np.pi * qq * np.arange(p) / n)
    out = np.empty(n, complex)
    for k1 in range(p):
        b = dftc(a[:, k1].copy(), s)
        out[k1 + p * np.arange(q)] = b
    return out


def two_factor(x, m1, m2, s):
    """Phases A and B of fft2f_kernel for one signal."""
    m = m1 * m2
    y = np.empty((m1, m2), complex)
    for j2 in range(m2):
        v = dftc(x[j2 + m2 * np.arange(m1)], s)
        e = (j2 * np.arange(m1)) % m
        y[:, j2] = v * np.exp(s * 2j * np.pi * e / m)
    out = np.empty(m, complex)
    for k1 in range(m1):
        out[k1 + m1 * np.arange(m2)] = dftc(y[k1].copy(), s)
    return out


SPLITS = [(40, 5, 8), (105, 7, 15), (175, 7, 25), (225, 15, 15), (243, 9, 27), (245, 7, 35), (343, 7, 49),
          (378, 18, 21), (392, 14, 28), (400, 20, 20)]


def _compiled_splits():
    out = {}
    for f in sorted(os.listdir(CSRC)):
        if f.startswith("fft_2f_f32_") and f.endswith(".cu"):
            for m, a, b in re.findall(r"GB_F2\((\d+), (\d+), (\d+)\)", open(os.path.join(CSRC, f)).read()):
                out[int(m)] = (int(a), int(b))
    return out


@pytest.mark.parametrize("n", sorted({a for _, a, b in SPLITS} | {b for _, a, b in SPLITS} | {6, 9, 12, 24, 32}))
@pytest.mark.parametrize("s", [-1, 1])
def test_codelet_is_the_dft(n, s):
    x = np.random.default_rng(n).standard_normal(n) + 1j * np.random.default_rng(n + 1).standard_normal(n)
    ref = np.fft.fft(x) if s < 0 else np.fft.ifft(x) * n
    assert np.allclose(dftc(x, s), ref, rtol=0, atol=1e-10 * np.abs(ref).max())


@pytest.mark.parametrize("m,m1,m2", SPLITS)
@pytest.mark.parametrize("s", [-1, 1])
def test_two_phases_give_the_dft(m, m1, m2, s):
    x = np.random.default_rng(m).standard_normal(m) + 1j * np.random.default_rng(m + 7).standard_normal(m)
    ref = np.fft.fft(x) if s < 0 else np.fft.ifft(x) * m
    assert np.allclose(two_factor(x, m1, m2, s), ref, rtol=0, atol=1e-10 * np.abs(ref).max())


def test_compiled_splits_are_balanced_7_smooth_factorisations():
    comp = _compiled_splits()
    assert len(comp) >= 60
    for m, (a, b) in comp.items():
        assert a * b == m and 2 <= a <= b <= 49
        for f in (a, b):
            r = f
            for p in (2, 3, 5, 7):
                while r % p == 0:
                    r //= p
            assert r == 1
            # every codelet decomposes into the direct butterflies
            stack = [f]
            while stack:
                n = stack.pop()
                if n in DIRECT or n == 1:
                    continue
                p = codelet_split(n)
                assert p in DIRECT and n % p == 0
                stack.append(n // p)


@pytest.mark.parametrize("m1,m2", [(7, 15), (18, 21), (14, 28), (20, 20)])
def test_intermediate_layouts(m1, m2):
    """Rows: (sl*M1 + k1)*PR + j2 with PR = M2 | 1 (odd), a bijection whose
    phase-B reads (lanes on consecutive k1, 8-byte elements) touch each
    4-byte bank pair at most twice per 32 lanes; columns: (k1*M2 + j2)*per + sl."""
    pr = m2 | 1
    per = 5
    idx = {(sl, k1, j2): (sl * m1 + k1) * pr + j2 for sl in range(per) for k1 in range(m1) for j2 in range(m2)}
    assert len(set(idx.values())) == len(idx)
    lanes = [(sl, k1) for sl in range(per) for k1 in range(m1)][:32]
    for j2 in range(m2):
        words = [2 * idx[(sl, k1, j2)] % 32 for sl, k1 in lanes]
        assert max(words.count(w) for w in set(words)) <= 2
    cper = 32
    cidx = {(sl, k1, j2): (k1 * m2 + j2) * cper + sl for sl in range(cper) for k1 in range(m1) for j2 in range(m2)}
    assert sorted(cidx.values()) == list(range(m1 * m2 * cper))


def test_constexpr_twiddles_match_libm(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not found")
    src = tmp_path / "kt.cpp"
    src.write_text(r'''
#include "ktrig.h"
#include <cmath>
#include <cstdio>
int main() {
    double worst = 0;
    for (int n = 1; n <= 512; ++n)
        for (int e = -n; e < 2 * n; ++e) {
            const double a = 2.0 * M_PI * (double)e / n;
            worst = std::fmax(worst, std::fabs(gb::ktrig::cos2pi(e, n) - std::cos(a)));
            worst = std::fmax(worst, std::fabs(gb::ktrig::sin2pi(e, n) - std::sin(a)));
        }
    static_assert(gb::ktrig::cos2pi(0, 7) == 1.0, "exact at zero");
    constexpr double c17 = gb::ktrig::cos2pi(1, 7);
    printf("%.3e %.17g\n", worst, c17);
}
''')
    exe = tmp_path / "kt"
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    worst, c17 = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert float(worst) < 1e-14
    assert abs(float(c17) - np.cos(2 * np.pi / 7)) < 1e-15
