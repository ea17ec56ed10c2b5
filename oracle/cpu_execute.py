"""CPU port of dtFFT's execute path -- the timed CPU baseline.

TEST INFRASTRUCTURE ONLY: imported by bench.py's CPU-baseline leg and by the
`--impl reference` arm, never by the product.

The reference's own CPU path (dtFFT + FFTW3 + MPI + OpenMP host kernels) cannot
be built on either machine of this project (no gfortran, MPI or FFTW3), so the
baseline is this port of it: the execute schedule of src/dtfft_plan.F90:1057-1101
(execute_generic) run rank by rank, the transposes by the C restatement of the
reference's host kernels and generic reshape handle (dtfft_oracle.c, OpenMP),
the per-rank batched 1D FFTs by scipy.fft (pocketfft, all host threads) in place
of FFTW's plan_many_dft.  Results are the oracle's; the point here is time.
"""
from __future__ import annotations

import os
import time

import numpy as np

from . import oracle as O


def _threads() -> int:
    return os.cpu_count() or 1


def _fft_layout(buf: np.ndarray, ndims, gdims, grid, layout, sign, workers):
    """Batched 1D C2C along the aligned axis of every rank's block (in place)."""
    import scipy.fft as sf
    n = gdims[layout - 1]
    # every block of this layout has the full aligned axis, so the whole packed
    # buffer is a batch of rows of length n
    rows = buf.reshape(-1, n)
    if sign < 0:
        rows[...] = sf.fft(rows, axis=1, workers=workers)
    else:
        rows[...] = sf.ifft(rows, axis=1, workers=workers, norm="forward")


class CpuC2C:
    """C2C plan of the CPU port on a virtual P1 x P2 grid (generic schedule)."""

    def __init__(self, dims, grid, dtype=np.complex64):
        self.dims = list(dims)
        self.grid = O.norm_grid(3, grid)
        self.dtype = np.dtype(dtype)
        self.n = int(np.prod(dims))
        self.workers = _threads()
        O.lib()

    def forward(self, x: np.ndarray) -> np.ndarray:
        d, g = self.dims, self.grid
        aux = x.copy()
        _fft_layout(aux, 3, d, g, 1, -1, self.workers)                 # fft(1): in -> aux
        out = O.vgrid_transpose(3, d, g, O.X_TO_Y, aux)                # X -> Y: aux -> out
        _fft_layout(out, 3, d, g, 2, -1, self.workers)                 # fft(2) in place
        aux = O.vgrid_transpose(3, d, g, O.Y_TO_Z, out)                # Y -> Z: out -> aux
        _fft_layout(aux, 3, d, g, 3, -1, self.workers)                 # fft(3): aux -> out
        return aux

    def backward(self, x: np.ndarray) -> np.ndarray:
        d, g = self.dims, self.grid
        aux = x.copy()
        _fft_layout(aux, 3, d, g, 3, +1, self.workers)
        y = O.vgrid_transpose(3, d, g, O.Z_TO_Y, aux)
        _fft_layout(y, 3, d, g, 2, +1, self.workers)
        aux = O.vgrid_transpose(3, d, g, O.Y_TO_X, y)
        _fft_layout(aux, 3, d, g, 1, +1, self.workers)
        return aux


def time_cycles(dims, grid, dtype=np.complex64, min_seconds=10.0, max_cycles=3, seed=2):
    """Time fwd+bwd cycles of the CPU port; returns (seconds per cycle, cycles, threads)."""
    rng = np.random.default_rng(seed)
    n = int(np.prod(dims))
    x = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(dtype)
    plan = CpuC2C(dims, grid, dtype)
    t0 = time.perf_counter()
    cycles = 0
    while True:
        y = plan.forward(x)
        x = plan.backward(y)
        x *= np.asarray(1.0 / n, dtype=x.real.dtype)
        cycles += 1
        el = time.perf_counter() - t0
        if el >= min_seconds or cycles >= max_cycles:
            break
    return el / cycles, cycles, plan.workers
