"""Build libdtfft_gb300.so (CUDA kernels + C ABI) in-tree with nvcc for sm_103a.

Usage:  python -m dtfft_gb300.build [--force]
Output: dtfft_gb300/_build/libdtfft_gb300.so
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "csrc")
INC = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libdtfft_gb300.so")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=default",
          "-I", INC, "-I", SRC]
CU_FLAGS = ARCH + ["-lineinfo", "--expt-relaxed-constexpr"]


def sources():
    out = []
    for f in sorted(os.listdir(SRC)):
        if f.endswith((".cu", ".cpp")):
            out.append(os.path.join(SRC, f))
    return out


def _deps_mtime():
    t = 0.0
    for d in (SRC, INC):
        for f in os.listdir(d):
            t = max(t, os.path.getmtime(os.path.join(d, f)))
    return max(t, os.path.getmtime(__file__))


def _compile(src: str) -> str:
    obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
    flags = COMMON + (CU_FLAGS if src.endswith(".cu") else [])
    cmd = [NVCC, "-c", src, "-o", obj] + flags
    if src.endswith(".cpp"):
        cmd = [NVCC, "-x", "cu", "-c", src, "-o", obj] + COMMON + CU_FLAGS
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, srcs))
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [NVCC, "-shared", "-o", tmp] + objs + ARCH + ["-cudart", "static", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
