"""Batched 1D transforms through the executor plug-in (gb_fft_create /
gb_fft_execute), timed with CUDA events: the row kernels alone, for
measurements and profiles.

Usage:  python -m dtfft_gb300.rowbench --n 270 --rows 66150 [--kind c2c|r2c] [--reps 20]

Prints one line per run: microseconds per launch and the GB/s of one read and
one write of the batch.
"""
from __future__ import annotations

import argparse
import ctypes


def run(n: int, rows: int, kind: str = "c2c", reps: int = 20) -> float:
    import torch
    import dtfft_gb300 as dt
    L = dt.lib()
    dev = torch.device("cuda:0")
    h = ctypes.c_void_p()
    sizes = (ctypes.c_int32 * 1)(n)
    if kind == "c2c":
        rc = L.gb_fft_create(1, 0, 0, n, n, rows, sizes, sizes, sizes, None, None, ctypes.byref(h))
        a = torch.randn(rows, n, dtype=torch.complex64, device=dev)
        b = torch.empty_like(a)
    else:
        rc = L.gb_fft_create(1, 1, 0, n, n // 2 + 1, rows, sizes, sizes, sizes, None, None, ctypes.byref(h))
        a = torch.randn(rows, n, dtype=torch.float32, device=dev)
        b = torch.empty(rows, n // 2 + 1, dtype=torch.complex64, device=dev)
    if rc != 0:
        raise RuntimeError(f"gb_fft_create failed: {rc}")
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    for i in range(reps + 1):
        if i == 1:
            e0.record()
        if L.gb_fft_execute(h, a.data_ptr(), b.data_ptr(), -1) != 0:
            raise RuntimeError("gb_fft_execute failed")
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / max(reps, 1)
    nbytes = a.numel() * a.element_size() + b.numel() * b.element_size()
    print(f"{kind} n={n} rows={rows}: {ms * 1e3:.1f} us/launch, {nbytes / ms / 1e6:.0f} GB/s", flush=True)
    L.gb_fft_destroy(ctypes.byref(h))
    return ms


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, required=True)
    ap.add_argument("--rows", type=int, required=True)
    ap.add_argument("--kind", choices=["c2c", "r2c"], default="c2c")
    ap.add_argument("--reps", type=int, default=20)
    a = ap.parse_args()
    run(a.n, a.rows, a.kind, a.reps)


if __name__ == "__main__":
    main()
