"""Build recipe for C and C++ programs that call libdtfft_gb300 as dtFFT's
own C/C++ callers do: include/dtfft.h (+ dtfft.hpp), the single-process
include/single_process_mpi/mpi.h, the helper functions of dtfft_test_helpers.c
and the library itself.  Used by tests/test_ref_callers.py (the reference's
integration programs, compiled and linked here where its sources are present)
and tests/test_ref_callers_gpu.py (this directory's programs, built and run on
a GPU).  Test infrastructure.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
INCLUDE = os.path.join(ROOT, "include")
MPI_INCLUDE = os.path.join(INCLUDE, "single_process_mpi")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def lib_dir() -> str:
    return os.path.join(ROOT, "dtfft_gb300", "_build")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    return r.returncode, (r.stdout + r.stderr)


def _includes(extra=()):
    out = []
    # `extra` first (a caller's own headers win over this library's dtfft.hpp),
    # then the single-process mpi.h, so <mpi.h> resolves to it
    for d in tuple(extra) + (MPI_INCLUDE, INCLUDE, HERE, os.path.join(CUDA, "include")):
        out += ["-I", d]
    return out


def compile_source(src: str, outdir: str, extra_includes=()) -> tuple[int, str, str]:
    """Compile one C or C++ source to an object in outdir."""
    os.makedirs(outdir, exist_ok=True)
    obj = os.path.join(outdir, os.path.basename(src) + ".o")
    if src.endswith((".cpp", ".cc", ".cxx")):
        cmd = ["g++", "-std=c++17", "-O1", "-c", src, "-o", obj]
    else:
        cmd = ["gcc", "-std=gnu11", "-O1", "-c", src, "-o", obj]
    rc, log = _run(cmd + _includes(extra_includes))
    return rc, log, obj


def link(objs, exe: str) -> tuple[int, str]:
    cuda_lib = os.path.join(CUDA, "lib64")
    cmd = (["g++", "-o", exe] + list(objs) +
           ["-L", lib_dir(), "-ldtfft_gb300", "-Wl,-rpath," + lib_dir(),
            "-L", cuda_lib, "-lcudart", "-Wl,-rpath," + cuda_lib, "-lm"])
    return _run(cmd)


def build_program(srcs, outdir: str, name: str, extra_includes=()) -> tuple[int, str, str]:
    """Compile `srcs` plus the helpers and link them into outdir/name."""
    objs, logs = [], []
    for s in list(srcs) + [os.path.join(HERE, "dtfft_test_helpers.c")]:
        rc, log, obj = compile_source(s, outdir, extra_includes)
        logs.append(log)
        if rc != 0:
            return rc, "\n".join(logs), ""
        objs.append(obj)
    exe = os.path.join(outdir, name)
    rc, log = link(objs, exe)
    logs.append(log)
    return rc, "\n".join(logs), exe


def reference_program_dirs(ref_root: str, outdir: str):
    """Include directories for the reference's own integration programs: its
    tests/c (test_utils.h), and a copy of its C++ header in outdir, so that the
    header's #include "dtfft.h" resolves to this library's dtfft.h and not to
    the reference's header next to it.  Nothing of the reference is written
    outside outdir."""
    hpp_dir = os.path.join(outdir, "ref_hpp")
    os.makedirs(hpp_dir, exist_ok=True)
    shutil.copy(os.path.join(ref_root, "include", "dtfft.hpp"), hpp_dir)
    return (hpp_dir, os.path.join(ref_root, "tests", "c"))
