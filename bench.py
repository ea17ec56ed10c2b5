"""Benchmark of dtFFT's execute path on GB300.

Workload (headline): 3D C2C complex64 512 x 512 x 512 on a 2 x 4 virtual rank
grid (8 pencil ranks held in one HBM allocation, 1 GiB per buffer), inputs
uniform[-1,1) re/im.  One step = one forward + one backward dtfft_execute
(X -> Y -> Z and back: 3 FFT passes + 2 transposes each way).

JSON line (rank 0): metric / value (fwd+bwd cycles per second, whole job),
roofline of the dominant kernel (live CUDA-event timing inside the timed
region), e2e (same metric through the C ABI with host buffers and the
host<->device copies inside the timed region), cpu_baseline (the CPU port of
the reference path on the host cores), clocks sampled during the timed region.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 runs N independent replicas of the workload (one per GPU); the path is
a single-GPU path with no inter-GPU exchange, so scaling is weak.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "3D fwd+bwd cycles/s & HBM TB/s; batched/TC vs plain on 1 GB300 at stated rel err"
DIMS = [512, 512, 512]
GRID = [1, 2, 4]
WORKLOAD = "c2c_c64_512x512x512_grid2x4_fwd+bwd"
FALLBACK_HBM = 6800.0


def _env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def max_over_ranks(values, world, device):
    """Element-wise maximum of per-rank values over all ranks (the slowest
    rank's time); the values themselves for a single rank."""
    values = [float(v) for v in values]
    if world <= 1:
        return values
    import torch
    import torch.distributed as dist
    t = torch.tensor(values, dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def _peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sms, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sms.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sms) if sms else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sms)}


def _profile_results(L):
    out = []
    n = L.dtfft_gb_profile_count()
    for i in range(n):
        name = ctypes.create_string_buffer(128)
        launches = ctypes.c_int64()
        ms = ctypes.c_double()
        L.dtfft_gb_profile_get(i, name, 128, ctypes.byref(launches), ctypes.byref(ms))
        out.append((name.value.decode(), int(launches.value), float(ms.value)))
    return out


def _traffic_for(kernel: str):
    """dram read+write bytes per launch of `kernel` from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            t = json.load(f)
        return t.get(WORKLOAD, {}).get(kernel)
    except Exception:
        return None


def cpu_baseline(sample_seconds=12.0):
    """The CPU port of the reference path, timed on this host (rank 0, N=1 only)."""
    from oracle import cpu_execute
    spc, cycles, threads = cpu_execute.time_cycles(DIMS, GRID, min_seconds=sample_seconds, max_cycles=2)
    return {"value": 1.0 / spc, "unit": "cycles/s", "cores": threads, "kind": "port",
            "sample": f"{cycles} full fwd+bwd cycle(s) of the {WORKLOAD} workload; C restatement of the "
                      f"reference host kernels (OpenMP) + scipy.fft (pocketfft) for the FFTW executor"}


def bench_config():
    """The workload description shared by both arms of the benchmark."""
    return {"workload": WORKLOAD, "dims": DIMS, "grid": "1x" + "x".join(map(str, GRID[1:])) + " virtual ranks",
            "precision": "single", "l2": "inputs larger than L2 (1 GiB per buffer)", "parallelism": "single GPU"}


def run_reference(args):
    """The reference path on the host cores: the CPU port (the oracle's C
    restatement of the reference's host kernels with OpenMP, scipy.fft for the
    FFTW executor) on this arm's workload.  Each step is one full forward +
    backward cycle; --steps and --warmup are honoured."""
    rank, world, _ = _env_rank()
    if rank != 0:
        return 0
    from oracle import cpu_execute
    if args.warmup:
        cpu_execute.time_cycles(DIMS, GRID, min_seconds=1e9, max_cycles=args.warmup)
    spc, cycles, threads = cpu_execute.time_cycles(DIMS, GRID, min_seconds=1e9, max_cycles=args.steps)
    v = 1.0 / spc
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "cycles/s", "n_gpus": args.gpus,
            "steps": cycles, "warmup": args.warmup, "ms_per_step": spc * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": bench_config(),
            "implementation": "CPU port of the reference path (oracle C kernels with OpenMP + scipy.fft)",
            "cpu_baseline": {"value": v, "unit": "cycles/s", "cores": threads, "kind": "port",
                             "sample": f"{cycles} full fwd+bwd cycle(s) of the workload, {threads} host threads"},
            "e2e": {"value": v, "unit": "cycles/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def seven_smooth(lo, hi):
    out = []
    for n in range(lo, hi + 1):
        m = n
        for q in (2, 3, 5, 7):
            while m % q == 0:
                m //= q
        if m == 1:
            out.append(n)
    return out


def batch_shapes(count=64, seed=5):
    """64 independent 3D transforms: edges drawn (PCG64, seed 5) from the
    7-smooth sizes in 48..384, alternating C2C complex64 / R2C float32."""
    import numpy as np
    rng = np.random.default_rng(seed)
    edges = seven_smooth(48, 384)
    return [("c2c" if i % 2 == 0 else "r2c", [int(rng.choice(edges)) for _ in range(3)]) for i in range(count)]


def _tune_records(dt):
    """Summary of the FFT step autotuner's choices (EXHAUSTIVE plans): steps
    tuned, chosen kernel kinds, and the chosen and runner-up candidates with
    their times for the steps where the choice mattered most."""
    L = dt.lib()
    L.dtfft_gb_tune_records.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
    n = ctypes.c_size_t()
    if L.dtfft_gb_tune_records(None, 0, ctypes.byref(n)) != 0:
        return None
    buf = ctypes.create_string_buffer(n.value)
    if L.dtfft_gb_tune_records(buf, n.value, ctypes.byref(n)) != 0:
        return None
    recs = json.loads(buf.value.decode())
    kinds = {}
    for r in recs:
        k = r["chosen"].split(":")[0]
        kinds[k] = kinds.get(k, 0) + 1
    gain = sorted(recs, key=lambda r: -(r["runner_up_ms"] - r["chosen_ms"]) if r["runner_up"] else 0)
    fused = [r for r in gain if r["step"].startswith("fused")]
    return {"steps_tuned": len(recs), "candidates_timed": sum(r["candidates"] for r in recs),
            "chosen_kinds": kinds, "largest_margins": gain[:12],
            "fused_passes_tuned": len(fused), "fused_passes": fused[:12]}


def batched_section(args, dt, dev, stream, peak):
    """64 mixed transforms, fwd+bwd each: 64 sequential plain plans (default
    effort, one dtfft_execute per plan and direction) against the same
    transforms as tuned plans (EXHAUSTIVE: measured transpose tiles) replayed
    as one CUDA graph per direction (dtfft_gb_batch_execute)."""
    import torch
    shapes = batch_shapes(count=args.batch_count)
    cfg = dt.Config(stream=stream.cuda_stream)
    plain, tuned, bufs = [], [], []
    pass_bytes = 0
    for i, (kind, dims) in enumerate(shapes):
        mk = dt.PlanC2C if kind == "c2c" else dt.PlanR2C
        plain.append(mk(dims, precision=dt.Precision.SINGLE, executor=dt.Executor.CUFFT, config=cfg))
        tuned.append(mk(dims, precision=dt.Precision.SINGLE, executor=dt.Executor.CUFFT,
                        effort=dt.Effort.EXHAUSTIVE, config=cfg))
        n = plain[-1].alloc_size
        g = torch.Generator(device=dev)
        g.manual_seed(1000 + i)
        if kind == "c2c":
            x = torch.complex(torch.randn(n, device=dev, generator=g), torch.randn(n, device=dev, generator=g))
            o = torch.empty_like(x)
            cbytes = n * 8
        else:
            x = torch.randn(n, device=dev, generator=g)
            o = torch.empty(n // 2, dtype=torch.complex64, device=dev)
            cbytes = (n // 2) * 8
        aux = torch.empty(max(n * x.element_size(), 16) // 4, dtype=torch.float32, device=dev)
        bufs.append((x, o, aux))
        # unfused passes per direction: Z-slab 2D FFT (2) + X->Z + FFT Z, generic 3 FFT + 2 transposes
        passes = 4 if plain[-1].z_slab_enabled else 5
        pass_bytes += 2 * passes * 2 * cbytes
    dt.set_config(dt.Config())
    torch.cuda.synchronize()
    tune = _tune_records(dt)
    ins = [b[0] for b in bufs]
    outs = [b[1] for b in bufs]
    auxs = [b[2] for b in bufs]

    def seq_step():
        for p, (x, o, a) in zip(plain, bufs):
            p.execute(x, o, dt.Execute.FORWARD, a)
        for p, (x, o, a) in zip(plain, bufs):
            p.execute(o, x, dt.Execute.BACKWARD, a)

    batch = dt.Batch(tuned, lanes=4)

    def batch_step():
        batch.execute(ins, outs, dt.Execute.FORWARD, auxs, stream)
        batch.execute(outs, ins, dt.Execute.BACKWARD, auxs, stream)

    def timed(fn):
        for _ in range(max(args.warmup, 3)):
            fn()
        torch.cuda.synchronize()
        k = max(3, min(args.steps, 10))
        l0 = dt.kernel_launches()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / k, (dt.kernel_launches() - l0) / k

    seq_ms, seq_launch = timed(seq_step)
    # where the sequential cycle's time goes, per kernel class (live event timing)
    L = dt.lib()
    L.dtfft_gb_profile_start()
    seq_step()
    torch.cuda.synchronize()
    L.dtfft_gb_profile_stop()
    classes = {}
    for name, cnt, tms in _profile_results(L):
        cls = name.split("_m")[0] if "_m" in name else name
        c = classes.setdefault(cls, [0, 0.0])
        c[0] += cnt
        c[1] += tms
    kernel_classes = [{"class": k, "launches": v[0], "total_ms": v[1]}
                      for k, v in sorted(classes.items(), key=lambda kv: -kv[1][1])]
    fwd_nodes = bwd_nodes = 0
    batch_ms, _ = timed(batch_step)
    batch.execute(ins, outs, dt.Execute.FORWARD, auxs, stream)
    fwd_nodes = batch.graph_nodes
    batch.execute(outs, ins, dt.Execute.BACKWARD, auxs, stream)
    bwd_nodes = batch.graph_nodes
    torch.cuda.synchronize()
    batch.destroy()
    # forward spectra of the first C2C and the first R2C member, five Z-lines
    # each against numpy FP64 (inputs regenerated from their seeds)
    member_err = {}
    for i in range(2):
        kind, dims = shapes[i]
        p = plain[i]
        x, o, aux = bufs[i]
        gen = torch.Generator(device=dev)
        gen.manual_seed(1000 + i)
        n = p.alloc_size
        if kind == "c2c":
            x.copy_(torch.complex(torch.randn(n, device=dev, generator=gen), torch.randn(n, device=dev, generator=gen)))
        else:
            x.copy_(torch.randn(n, device=dev, generator=gen))
        nx, ny, nz = dims
        glob = x[:nx * ny * nz].cpu().numpy().reshape(nz, ny, nx)
        p.execute(x, o, dt.Execute.FORWARD, aux)
        torch.cuda.synchronize()
        pts = _z_line_points(nx // 2 + 1 if kind == "r2c" else nx, ny)
        member_err[f"{kind}_{nx}x{ny}x{nz}"] = _rel_l2(_device_z_lines(dt, p, o, pts, nz), _fp64_z_lines(glob, pts, kind))
    for p in plain + tuned:
        p.destroy()
    n_c2c = sum(1 for k, _ in shapes if k == "c2c")
    return {"workload": "64 3D transforms, edges 7-smooth in 48..384 (PCG64 seed 5), 32 C2C c64 + 32 R2C f32, "
                        "N(0,1), fwd+bwd each, one process per transform",
            "transforms": len(shapes), "c2c": n_c2c, "r2c": len(shapes) - n_c2c,
            "sequential_plain": {"cycles_per_s": 1000.0 / seq_ms, "ms_per_cycle": seq_ms,
                                 "kernel_launches_per_cycle": seq_launch},
            "batched_graph": {"cycles_per_s": 1000.0 / batch_ms, "ms_per_cycle": batch_ms,
                              "graph_launches_per_cycle": 2, "graph_nodes_per_cycle": fwd_nodes + bwd_nodes},
            "speedup": seq_ms / batch_ms,
            "fwd_rel_l2_vs_numpy_fp64_z_lines": member_err,
            "sequential_kernel_classes": kernel_classes,
            "unfused_pass_bytes_per_cycle": pass_bytes,
            "fft_autotune": tune,
            "effective_tbs": {"sequential_plain": pass_bytes / (seq_ms * 1e-3) / 1e12,
                              "batched_graph": pass_bytes / (batch_ms * 1e-3) / 1e12}}


def _z_line_points(nx, ny):
    """(kx, ky) of the sampled Z-lines: the zero and last frequencies, the
    middle and two interior points."""
    return [(0, 0), (nx - 1, ny - 1), (nx // 2, ny // 5), (11 % nx, 1 % ny), (nx // 3, ny - 1)]


def _fp64_z_lines(g, pts, kind="c2c"):
    """FP64 values along Z of the forward 3D transform of g (numpy, C order
    [z][y][x]) at the fixed (kx, ky) frequencies `pts`, computed with numpy
    as the contraction of g with the two basis vectors followed by the 1D
    transform along Z (the transform is separable), reading g in chunks of
    z-planes.  kind: "c2c" / "r2c" (exp(-2 pi i j k / n) along X and Y, FFT
    along Z) or "dct2" (FFTW's REDFT10 2 cos(pi k (2j + 1) / (2n)) on every axis)."""
    import numpy as np
    nz, ny, nx = g.shape
    kx = np.array([p[0] for p in pts])
    ky = np.array([p[1] for p in pts])
    if kind == "dct2":
        bx = 2 * np.cos(np.pi * np.outer(2 * np.arange(nx) + 1, kx) / (2 * nx))
        by = 2 * np.cos(np.pi * np.outer(2 * np.arange(ny) + 1, ky) / (2 * ny))
        acc = np.zeros((len(pts), nz))
    else:
        bx = np.exp(-2j * np.pi * np.outer(np.arange(nx), kx) / nx)
        by = np.exp(-2j * np.pi * np.outer(np.arange(ny), ky) / ny)
        acc = np.zeros((len(pts), nz), dtype=np.complex128)
    for z0 in range(0, nz, 16):
        G = np.asarray(g[z0:z0 + 16], dtype=acc.dtype)
        t = (G.reshape(-1, nx) @ bx).reshape(G.shape[0], ny, len(pts))
        acc[:, z0:z0 + G.shape[0]] = np.einsum("zyk,yk->kz", t, by)
    if kind == "dct2":
        import scipy.fft as sf
        return sf.dct(acc, type=2, axis=1, norm=None)
    return np.fft.fft(acc, axis=1)


def _device_z_lines(dt, plan, buf, pts, nz):
    """The same Z-lines from a plan's forward output (Z pencils of every
    virtual rank, packed; a rank's block stores (z, x, y) with z fastest),
    located through the library's own per-rank pencils and offsets."""
    import numpy as np
    out = []
    for kx, ky in pts:
        for r in range(plan.nranks):
            pen, off = plan.vrank_pencil(dt.Layout.Z_PENCILS, r)
            sz, sx, sy = pen.starts
            cz, cx, cy = pen.counts
            if sx <= kx < sx + cx and sy <= ky < sy + cy:
                base = off + cz * ((kx - sx) + cx * (ky - sy))
                out.append(buf[base:base + cz].cpu().numpy().astype(np.complex128 if buf.is_complex() else np.float64))
                break
    return np.stack(out)


def _rel_l2(a, b):
    import numpy as np
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def tensor_core_section(args, dt, dev, stream, sizes=(768, 1024)):
    """C2C complex64 N^3 (one process, Z-slab plan), inputs uniform[-1,1) re/im
    plus 1e3-amplitude spikes at 0.1% of the points: FP32 Stockham row passes
    against the tensor-core form (DFT-matrix GEMMs on tcgen05, FP16 hi + lo,
    FP32 accumulate) of the plain row passes (both plans keep the fused FFT +
    transpose passes on the FP32 kernels; `row_pass_ms` compares the two row
    kernels alone), fwd+bwd cycles/s, forward error against an FP64
    (complex128) plan of the same transform, and against numpy FP64 values of
    five Z-lines of the spectrum."""
    import torch
    L = dt.lib()
    L.dtfft_gb_set_fft_form.argtypes = [ctypes.c_int32]
    out = []
    for N in sizes:
        dims = [N, N, N]
        cfg = dt.Config(stream=stream.cuda_stream)
        plans = {}
        for form in (0, 1):
            L.dtfft_gb_set_fft_form(form)
            plans[form] = dt.PlanC2C(dims, precision=dt.Precision.SINGLE, executor=dt.Executor.CUFFT, config=cfg)
        L.dtfft_gb_set_fft_form(0)
        p64 = dt.PlanC2C(dims, precision=dt.Precision.DOUBLE, executor=dt.Executor.CUFFT, config=cfg)
        dt.set_config(dt.Config())
        n = plans[0].alloc_size
        g = torch.Generator(device=dev)
        g.manual_seed(4)
        x0 = torch.complex(torch.rand(n, device=dev, generator=g) * 2 - 1,
                           torch.rand(n, device=dev, generator=g) * 2 - 1)
        spikes = torch.randint(0, n, (max(1, n // 1000),), device=dev, generator=g)
        x0[spikes] *= 1e3
        # FP64 reference spectrum
        a64 = x0.to(torch.complex128)
        b64 = torch.empty_like(a64)
        aux64 = torch.empty_like(a64)
        torch.cuda.synchronize()
        p64.execute(a64, b64, dt.Execute.FORWARD, aux64)
        torch.cuda.synchronize()
        del a64, aux64
        ref_norm = float(torch.linalg.vector_norm(b64))
        pts = _z_line_points(N, N)
        lines_ref = _fp64_z_lines(x0.cpu().numpy().reshape(N, N, N), pts)
        a = torch.empty_like(x0)
        b = torch.empty_like(x0)
        aux = torch.empty_like(x0)
        row = {"dims": dims, "points": n}
        for form, name in ((0, "fp32_stockham"), (1, "tensor_core_fp16x3")):
            p = plans[form]
            a.copy_(x0)
            torch.cuda.synchronize()
            p.execute(a, b, dt.Execute.FORWARD, aux)
            torch.cuda.synchronize()
            err = float(torch.linalg.vector_norm(b.to(torch.complex128) - b64)) / ref_norm
            err_lines = _rel_l2(_device_z_lines(dt, p, b, pts, N), lines_ref)
            p.execute(b, a, dt.Execute.BACKWARD, aux)
            torch.cuda.synchronize()
            rt = float(torch.linalg.vector_norm(a / n - x0) / torch.linalg.vector_norm(x0))

            def step():
                p.execute(a, b, dt.Execute.FORWARD, aux)
                p.execute(b, a, dt.Execute.BACKWARD, aux)

            for _ in range(max(args.warmup, 3)):
                a.copy_(x0)
                step()
            torch.cuda.synchronize()
            k = max(3, min(args.steps, 10))
            L.dtfft_gb_profile_start()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(k):
                step()
            e1.record(stream)
            torch.cuda.synchronize()
            L.dtfft_gb_profile_stop()
            ms = e0.elapsed_time(e1) / k
            prof = sorted(_profile_results(L), key=lambda r: -r[2])
            rows = [r for r in prof if "rows_c2c" in r[0]]
            row[name] = {"cycles_per_s": 1000.0 / ms, "ms_per_cycle": ms, "fwd_rel_l2_vs_fp64": err,
                         "fwd_rel_l2_vs_numpy_fp64_z_lines": err_lines,
                         "roundtrip_rel_l2": rt,
                         "row_pass_kernel": rows[0][0] if rows else None,
                         "row_pass_ms": rows[0][2] / max(rows[0][1], 1) if rows else None,
                         "kernels": [{"name": r[0], "launches": r[1], "total_ms": r[2]} for r in prof]}
        row["speedup_tc_vs_fp32"] = row["fp32_stockham"]["ms_per_cycle"] / row["tensor_core_fp16x3"]["ms_per_cycle"]
        out.append(row)
        for p in list(plans.values()) + [p64]:
            p.destroy()
        del x0, a, b, aux, b64
        torch.cuda.empty_cache()
    return out


def config1_section(args, dt, dev, stream):
    """2D C2C complex128 256x256 in one process (execute_2d: FFT X, X->Y, FFT Y
    and back), inputs uniform[-1,1) re/im: fwd+bwd cycles/s with one
    dtfft_execute per direction, and the same cycle replayed as one CUDA graph
    per direction (dtfft_gb_batch_execute of this one plan).  1 MiB per buffer:
    the cycle is launch- and L2-bound, not HBM-bound."""
    import torch
    dims = [256, 256]
    plan = dt.PlanC2C(dims, precision=dt.Precision.DOUBLE, executor=dt.Executor.CUFFT,
                      config=dt.Config(stream=stream.cuda_stream))
    dt.set_config(dt.Config())
    n = plan.alloc_size
    g = torch.Generator(device=dev)
    g.manual_seed(1)
    x0 = torch.complex(torch.rand(n, device=dev, generator=g, dtype=torch.float64) * 2 - 1,
                       torch.rand(n, device=dev, generator=g, dtype=torch.float64) * 2 - 1)
    a = x0.clone()
    b = torch.empty_like(a)
    aux = torch.empty_like(a)
    torch.cuda.synchronize()
    plan.execute(a, b, dt.Execute.FORWARD, aux)
    plan.execute(b, a, dt.Execute.BACKWARD, aux)
    torch.cuda.synchronize()
    rt = float(torch.linalg.vector_norm(a / n - x0) / torch.linalg.vector_norm(x0))
    batch = dt.Batch([plan])

    def plain():
        plan.execute(a, b, dt.Execute.FORWARD, aux)
        plan.execute(b, a, dt.Execute.BACKWARD, aux)

    def graph():
        batch.execute([a], [b], dt.Execute.FORWARD, [aux], stream)
        batch.execute([b], [a], dt.Execute.BACKWARD, [aux], stream)

    out = {"workload": "2D C2C complex128 256x256, one process, fwd+bwd", "roundtrip_rel_l2": rt}
    for name, fn in (("execute", plain), ("graph", graph)):
        for _ in range(max(args.warmup, 3)):
            fn()
        torch.cuda.synchronize()
        k = 200
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / k
        out[name] = {"cycles_per_s": 1000.0 / ms, "ms_per_cycle": ms}
    l0 = dt.kernel_launches()
    plain()
    torch.cuda.synchronize()
    out["kernels_per_cycle"] = dt.kernel_launches() - l0
    batch.destroy()
    plan.destroy()
    return out


def config3_section(args, dt, dev, stream):
    """3D R2C float64 1024x1024x512 (real input N(0,1)) on a 4x4 virtual grid,
    and the R2R plan of the same grid with DCT-II on every axis: fwd+bwd
    cycles/s, the round trip, and the forward spectrum on five Z-lines against
    numpy FP64."""
    import numpy as np
    import torch
    dims = [1024, 1024, 512]
    comm = dt.cart_comm([1, 4, 4])
    L = dt.lib()
    L.dtfft_gb_measure_fp64_fma.argtypes = [ctypes.POINTER(ctypes.c_double)]
    t = ctypes.c_double()
    fp64_peak = t.value if L.dtfft_gb_measure_fp64_fma(ctypes.byref(t)) == 0 else None
    hbm_peak, hbm_kind = _peaks()
    out = {"dims": dims, "grid": "1x4x4 virtual ranks", "precision": "double",
           "fp64_fma_peak_tflops": fp64_peak, "fp64_peak_kind": "measured (FMA chains on every SM)",
           "hbm_peak_gbs": hbm_peak, "hbm_peak_kind": hbm_kind}
    cfg = dt.Config(stream=stream.cuda_stream)
    for kind in ("r2c", "r2r_dct2"):
        if kind == "r2c":
            plan = dt.PlanR2C(dims, comm=comm, precision=dt.Precision.DOUBLE, executor=dt.Executor.CUFFT, config=cfg)
            n_in = plan.alloc_size                     # real elements
            n_out = n_in // 2                          # complex elements
        else:
            plan = dt.PlanR2R(dims, kinds=[dt.R2RKind.DCT_2] * 3, comm=comm, precision=dt.Precision.DOUBLE,
                              executor=dt.Executor.VKFFT, config=cfg)
            n_in = n_out = plan.alloc_size
        dt.set_config(dt.Config())
        g = torch.Generator(device=dev)
        g.manual_seed(3)
        x0 = torch.randn(n_in, device=dev, generator=g, dtype=torch.float64)
        a = x0.clone()
        b = (torch.empty(n_out, dtype=torch.complex128, device=dev) if kind == "r2c"
             else torch.empty(n_out, dtype=torch.float64, device=dev))
        aux = torch.empty_like(b)
        torch.cuda.synchronize()

        def step():
            plan.execute(a, b, dt.Execute.FORWARD, aux)
            plan.execute(b, a, dt.Execute.BACKWARD, aux)

        # forward spectrum: five Z-lines against numpy FP64 (the global real
        # array is assembled from every virtual rank's X pencil block)
        plan.execute(a, b, dt.Execute.FORWARD, aux)
        torch.cuda.synchronize()
        gx = x0.cpu().numpy()
        glob = np.empty((dims[2], dims[1], dims[0]))
        for r in range(plan.nranks):
            pen, off = plan.vrank_pencil(dt.Layout.X_PENCILS, r)
            sx, sy, sz = pen.starts
            cx, cy, cz = pen.counts
            glob[sz:sz + cz, sy:sy + cy, sx:sx + cx] = gx[off:off + cx * cy * cz].reshape(cz, cy, cx)
        del gx
        nxo = dims[0] // 2 + 1 if kind == "r2c" else dims[0]
        pts = _z_line_points(nxo, dims[1])
        err_lines = _rel_l2(_device_z_lines(dt, plan, b, pts, dims[2]),
                            _fp64_z_lines(glob, pts, "r2c" if kind == "r2c" else "dct2"))
        del glob
        a.copy_(x0)
        step()
        torch.cuda.synchronize()
        # unnormalised round trip: R2C scales by N, DCT-II/III by prod(2 n)
        # the real grid is the first prod(dims) elements (an R2C buffer is sized for the complex layouts)
        nreal = dims[0] * dims[1] * dims[2]
        scale = float(nreal) * (8.0 if kind != "r2c" else 1.0)
        rt = float(torch.linalg.vector_norm(a[:nreal] / scale - x0[:nreal]) / torch.linalg.vector_norm(x0[:nreal]))
        for _ in range(max(1, min(args.warmup, 2))):
            step()
        torch.cuda.synchronize()
        k = 3
        L = dt.lib()
        L.dtfft_gb_profile_start()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        L.dtfft_gb_profile_stop()
        ms = e0.elapsed_time(e1) / k
        prof = sorted(_profile_results(L), key=lambda r: -r[2])
        # rooflines: conventional FFT flops (2.5 N log2 N per real-data
        # direction) against the measured FP64 FMA rate, and each kernel's
        # one-read-one-write of the larger buffer against HBM
        flops = 2 * 2.5 * nreal * math.log2(nreal)
        big = max(n_in * 8, n_out * (16 if kind == "r2c" else 8))
        out[kind] = {"cycles_per_s": 1000.0 / ms, "ms_per_cycle": ms, "roundtrip_rel_l2": rt,
                     "fwd_rel_l2_vs_numpy_fp64_z_lines": err_lines,
                     "fft_tflops_conventional": flops / (ms * 1e-3) / 1e12,
                     "frac_of_fp64_fma_peak": (flops / (ms * 1e-3) / 1e12) / fp64_peak if fp64_peak else None,
                     "kernels": [{"name": r[0], "launches": r[1], "total_ms": r[2],
                                  "hbm_frac_at_2B": (2 * big / (r[2] / max(r[1], 1) * 1e-3) / 1e9) / hbm_peak}
                                 for r in prof]}
        plan.destroy()
        del a, b, aux, x0
        torch.cuda.empty_cache()
    return out


def run_ours(args):
    import numpy as np
    import torch
    import torch.distributed as dist

    import dtfft_gb300 as dt

    rank, world, local = _env_rank()
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    L = dt.lib()

    global DIMS, GRID, WORKLOAD
    if args.dims:
        DIMS = list(args.dims)
        GRID = [1] + list(args.grid)
        WORKLOAD = f"c2c_c64_{'x'.join(map(str, DIMS))}_grid{'x'.join(map(str, GRID[1:]))}_fwd+bwd"
    comm = dt.cart_comm(GRID)
    # one stream for torch's copies and the plan's kernels
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    cfg = dt.Config(stream=stream.cuda_stream)
    plan = dt.PlanC2C(DIMS, comm=comm, precision=dt.Precision.SINGLE, executor=dt.Executor.CUFFT,
                      effort=dt.Effort(args.effort), config=cfg)
    dt.set_config(dt.Config())
    n = plan.alloc_size
    nbytes = n * 8
    g = torch.Generator(device=dev)
    g.manual_seed(2)
    x0 = torch.complex(torch.rand(n, device=dev, generator=g) * 2 - 1,
                       torch.rand(n, device=dev, generator=g) * 2 - 1).to(torch.complex64)
    a = x0.clone()
    b = torch.empty_like(a)
    aux = torch.empty_like(a)
    torch.cuda.synchronize()

    def step():
        plan.execute(a, b, dt.Execute.FORWARD, aux)
        plan.execute(b, a, dt.Execute.BACKWARD, aux)

    # forward spectrum on five Z-lines against numpy FP64 (outside the timed region)
    plan.execute(a, b, dt.Execute.FORWARD, aux)
    torch.cuda.synchronize()
    gx = x0.cpu().numpy()
    glob = np.empty((DIMS[2], DIMS[1], DIMS[0]), dtype=np.complex64)
    for r in range(plan.nranks):
        pen, off = plan.vrank_pencil(dt.Layout.X_PENCILS, r)
        sx, sy, sz = pen.starts
        cx, cy, cz = pen.counts
        glob[sz:sz + cz, sy:sy + cy, sx:sx + cx] = gx[off:off + cx * cy * cz].reshape(cz, cy, cx)
    del gx
    zpts = _z_line_points(DIMS[0], DIMS[1])
    fwd_lines_err = _rel_l2(_device_z_lines(dt, plan, b, zpts, DIMS[2]), _fp64_z_lines(glob, zpts))
    del glob
    a.copy_(x0)
    # round-trip error (outside the timed region): fwd, bwd, scale
    step()
    torch.cuda.synchronize()
    rt = float(torch.linalg.vector_norm(a / (DIMS[0] * DIMS[1] * DIMS[2]) - x0) / torch.linalg.vector_norm(x0))

    # Every timed step starts from the same finite input: the unnormalised
    # forward + backward multiplies the data by N = 1.3e8, so a chain of
    # cycles would overflow complex64 after four of them.  Between steps, and
    # outside each step's event pair, the input is copied back and a 256 MiB
    # buffer is written so that no part of it is left in the 129 MB L2.
    flush = torch.empty(64 << 20, dtype=torch.float32, device=dev)

    def refresh():
        a.copy_(x0)
        flush.fill_(1.0)

    for _ in range(args.warmup):
        refresh()
        step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    launches0 = dt.kernel_launches()
    L.dtfft_gb_profile_start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    torch.cuda.synchronize()
    for e0, e1 in ev:
        refresh()
        e0.record(stream)
        step()
        e1.record(stream)
    torch.cuda.synchronize()
    L.dtfft_gb_profile_stop()
    launches = dt.kernel_launches() - launches0
    ms = sum(e0.elapsed_time(e1) for e0, e1 in ev)
    finite = bool(torch.isfinite(torch.view_as_real(a)).all())
    clk = clocks.stop()
    prof = _profile_results(L)
    ms = max_over_ranks([ms], world, dev)[0]
    ms_step = ms / args.steps
    value = world * 1000.0 / ms_step

    # dominant kernel of the timed region
    top = max(prof, key=lambda r: r[2]) if prof else ("none", 1, 0.0)
    per_launch_ms = top[2] / max(top[1], 1)
    algo_bytes = 2 * nbytes          # one read + one write of the whole buffer per launch
    achieved = algo_bytes / (per_launch_ms * 1e-3) / 1e9 if per_launch_ms > 0 else 0.0
    peak, peak_kind = _peaks()
    # unfused pass count of the generic schedule: 2 x (3 FFT + 2 transposes), each one read + one write
    step_bytes = 2 * (3 + 2) * 2 * nbytes
    eff_tbs = step_bytes / (ms_step * 1e-3) / 1e12

    # e2e: host buffers through the C ABI.  Every step copies its input from
    # pinned host memory, runs forward + backward, and copies the result back;
    # consecutive steps are pipelined over three device buffer sets and three
    # streams (host->device, compute on the plan's stream, device->host), so the
    # copies of one step overlap the transforms of its neighbours and the other
    # direction's copies.  The timed region spans the first copy-in to the last
    # copy-out.
    e2e_ms = link_ms = None
    e2e_windows = []
    link_windows = []
    if not args.no_e2e:
        host_in = torch.empty(n, dtype=torch.complex64, pin_memory=True)
        host_in.copy_(x0.cpu())
        NSETS = 3
        host_out = [torch.empty(n, dtype=torch.complex64, pin_memory=True) for _ in range(NSETS)]
        sets = [(a, b)] + [(torch.empty_like(a), torch.empty_like(a)) for _ in range(NSETS - 1)]
        s_in = torch.cuda.Stream(dev)
        s_out = torch.cuda.Stream(dev)
        e2e_steps = max(2, min(args.steps, 10))
        ev = {k: [torch.cuda.Event() for _ in range(NSETS)] for k in ("in", "comp", "out")}
        for e in ev["out"]:
            e.record(s_out)

        def e2e_step(k):
            i = k % NSETS
            da, db = sets[i]
            s_in.wait_event(ev["out"][i])            # the copy-out NSETS steps back has read this set
            with torch.cuda.stream(s_in):
                da.copy_(host_in, non_blocking=True)
            ev["in"][i].record(s_in)
            stream.wait_event(ev["in"][i])
            plan.execute(da, db, dt.Execute.FORWARD, aux)
            plan.execute(db, da, dt.Execute.BACKWARD, aux)
            ev["comp"][i].record(stream)
            s_out.wait_event(ev["comp"][i])
            with torch.cuda.stream(s_out):
                host_out[i].copy_(da, non_blocking=True)
            ev["out"][i].record(s_out)

        for k in range(NSETS):
            e2e_step(k)
        torch.cuda.synchronize()
        # three windows of e2e_steps steps; the median window is reported (the
        # device->host rate into pinned host memory varies between windows on
        # shared hosts), every window is listed
        e2e_windows = []
        for _ in range(3):
            f0 = torch.cuda.Event(enable_timing=True)
            f1 = torch.cuda.Event(enable_timing=True)
            f0.record(s_in)
            for k in range(e2e_steps):
                e2e_step(k)
            f1.record(s_out)
            torch.cuda.synchronize()
            e2e_windows.append(f0.elapsed_time(f1) / e2e_steps)
        e2e_ms = sorted(e2e_windows)[1]
        # the round trip survived the pipeline: last result == input (scaled)
        e2e_rt = float(torch.linalg.vector_norm(host_out[(e2e_steps - 1) % NSETS] / (DIMS[0] * DIMS[1] * DIMS[2])
                                                - host_in) / torch.linalg.vector_norm(host_in))
        # the host link alone: the same two copies per step, both directions
        # at once, no transforms - the bound the end-to-end figure runs into
        # (three windows, median, as for the end-to-end figure)
        link_windows = []
        for _ in range(3):
            lk0 = torch.cuda.Event(enable_timing=True)
            lk1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            lk0.record(s_in)
            s_out.wait_event(lk0)
            for k in range(e2e_steps):
                ca, cb = sets[k % NSETS]
                with torch.cuda.stream(s_in):
                    ca.copy_(host_in, non_blocking=True)
                with torch.cuda.stream(s_out):
                    host_out[(k + 1) % NSETS].copy_(sets[(k + 1) % NSETS][1], non_blocking=True)
            lk_in = torch.cuda.Event()
            lk_in.record(s_in)
            s_out.wait_event(lk_in)
            lk1.record(s_out)
            torch.cuda.synchronize()
            link_windows.append(lk0.elapsed_time(lk1) / e2e_steps)
        link_ms = sorted(link_windows)[1]
        e2e_ms, link_ms = max_over_ranks([e2e_ms, link_ms], world, dev)
        del sets

    # transpose-only cycle of the same grid (X->Y->Z->Y->X, executor NONE):
    # 4 grid transposes per cycle, each one read + one write of the buffer
    tonly = None
    if not args.no_transpose_only:
        tplan = dt.PlanC2C(DIMS, comm=comm, precision=dt.Precision.SINGLE, executor=dt.Executor.NONE,
                           effort=dt.Effort(args.effort), config=dt.Config(stream=stream.cuda_stream))
        dt.set_config(dt.Config())

        def tstep():
            tplan.execute(a, b, dt.Execute.FORWARD, aux)
            tplan.execute(b, a, dt.Execute.BACKWARD, aux)

        for _ in range(args.warmup):
            tstep()
        torch.cuda.synchronize()
        L.dtfft_gb_profile_start()
        g0 = torch.cuda.Event(enable_timing=True)
        g1 = torch.cuda.Event(enable_timing=True)
        g0.record(stream)
        for _ in range(args.steps):
            tstep()
        g1.record(stream)
        torch.cuda.synchronize()
        L.dtfft_gb_profile_stop()
        tprof = _profile_results(L)
        t_ms = g0.elapsed_time(g1) / args.steps
        tk = max(tprof, key=lambda r: r[2]) if tprof else ("none", 1, 0.0)
        t_launch = tk[2] / max(tk[1], 1)
        tonly = {"cycles_per_s": 1000.0 / t_ms, "ms_per_cycle": t_ms, "kernel": tk[0], "launch_ms": t_launch,
                 "achieved_gbs": algo_bytes / (t_launch * 1e-3) / 1e9 if t_launch > 0 else 0.0,
                 "frac": (algo_bytes / (t_launch * 1e-3) / 1e9) / peak if t_launch > 0 else 0.0,
                 "effective_tbs": 4 * algo_bytes / (t_ms * 1e-3) / 1e12}
        tplan.destroy()

    tensor_core = None
    if not args.no_tc:
        tensor_core = tensor_core_section(args, dt, dev, stream, sizes=tuple(args.tc_sizes))

    cfg1 = cfg3 = None
    if not args.no_configs:
        cfg1 = config1_section(args, dt, dev, stream)
        cfg3 = config3_section(args, dt, dev, stream)

    batched = None
    if not args.no_batch:
        batched = batched_section(args, dt, dev, stream, peak)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            cpu = cpu_baseline()
        except Exception as ex:  # report, never fake
            cpu = {"value": None, "unit": "cycles/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"failed: {ex}"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "cycles/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(bench_config(), **({"parallelism": "replicas"} if world > 1 else {})),
            "implementation": "own Stockham tile kernels, fused FFT + grid transpose passes",
            "timing": "per-step CUDA event pairs on the plan's stream; the input is restored and L2 flushed "
                      "between steps, outside the pairs",
            "data_finite_after_timed_steps": finite,
            "pass_equivalent_tbs": {"value": eff_tbs, "what": "unfused pass count 2 x (3 FFT + 2 transposes) x "
                                    "2 B per cycle / time; fusion makes it exceed the DRAM traffic"},
            "roundtrip_rel_l2": rt,
            "fwd_rel_l2_vs_numpy_fp64_z_lines": fwd_lines_err,
            "roofline": {"bound": "hbm", "kernel": top[0], "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": _traffic_for(top[0]), "algorithmic_bytes": algo_bytes,
                         "launch_ms": per_launch_ms},
            "kernels": [{"name": k, "launches": c, "total_ms": t} for k, c, t in sorted(prof, key=lambda r: -r[2])],
            "e2e": ({"value": world * 1000.0 / e2e_ms, "unit": "cycles/s", "h2d_bytes_per_step": nbytes,
                     "d2h_bytes_per_step": nbytes, "ms_per_step": e2e_ms, "roundtrip_rel_l2": e2e_rt,
                     "pipelined": "3 buffer sets; copy-in, compute, copy-out streams",
                     "windows_ms_per_step": e2e_windows, "reported": "median of 3 windows",
                     "host_link_bound": {"value": world * 1000.0 / link_ms, "unit": "cycles/s", "ms_per_step": link_ms,
                                         "what": "the step's H2D and D2H copies alone, concurrently",
                                         "windows_ms_per_step": link_windows, "reported": "median of 3 windows"}}
                    if e2e_ms else None),
            "gpu_launches": launches,
            "autotune": _tune_records(dt) if args.effort == 3 else None,
            "cpu_baseline": cpu,
            "clocks": clk,
            "transpose_only": tonly,
            "batched": batched,
            "tensor_core": tensor_core,
            "config_2d_c128_256x256": cfg1,
            "config_r2c_f64_1024x1024x512_grid4x4": cfg3,
        }
        print(json.dumps(line), flush=True)
    plan.destroy()
    if world > 1:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--effort", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-transpose-only", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-transform batched section")
    ap.add_argument("--no-tc", action="store_true", help="skip the tensor-core 768^3 / 1024^3 section")
    ap.add_argument("--batch-count", type=int, default=64,
                    help="transforms of the batch section (fewer for profiling; the workload is 64)")
    ap.add_argument("--tc-sizes", type=int, nargs="+", default=[768, 1024],
                    help="cube edges of the tensor-core section (smaller ones for profiling)")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the 2D c128 256x256 and R2C/R2R f64 1024x1024x512 sections")
    ap.add_argument("--dims", type=int, nargs=3, default=None,
                    help="smaller C2C case for profiling (default: the 512^3 headline workload)")
    ap.add_argument("--grid", type=int, nargs=2, default=[2, 4])
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
