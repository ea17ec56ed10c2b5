"""dtfft_gb300 -- dtFFT's single-GPU execute path on GB300.

The compute lives in libdtfft_gb300.so (hand-written CUDA for sm_103a behind
dtFFT's C ABI, see include/dtfft.h).  This module is a thin ctypes host layer
whose classes mirror the reference's Python interface
(src/interfaces/python/__init__.py: PlanC2C / PlanR2C / PlanR2R, execute,
transpose, get_pencil, local_sizes ...), taking torch CUDA tensors (or raw
device pointers) instead of cupy arrays.  Dimensions are in natural Fortran
order (X fastest), as in the reference.

There is no CPU path: if the CUDA library cannot be built or loaded, import of
the library fails.
"""
from __future__ import annotations

import ctypes
import enum
import os
from typing import Optional

__all__ = [
    "lib", "pencils_comm", "Batch", "DtfftError", "Execute", "Transpose", "Layout", "Reshape", "Precision", "Effort",
    "Executor", "R2RKind", "Backend", "Platform", "Pencil", "Config", "set_config",
    "PlanC2C", "PlanR2C", "PlanR2R", "cart_comm", "world_comm", "COMM_WORLD",
    "get_backend_string", "get_precision_string", "get_executor_string",
    "is_fftw_enabled", "is_mkl_enabled", "is_cufft_enabled", "is_vkfft_enabled", "is_cuda_enabled",
    "is_transpose_only_enabled", "is_nccl_enabled", "is_nvshmem_enabled", "is_compression_enabled",
]

_LIB = None
COMM_WORLD = 0x44000000


def lib() -> ctypes.CDLL:
    """Load (building in-tree on first use) libdtfft_gb300.so."""
    global _LIB
    if _LIB is None:
        from . import build as _build
        path = _build.build()
        L = ctypes.CDLL(path, mode=ctypes.RTLD_GLOBAL)
        _declare(L)
        _LIB = L
    return _LIB


class DtfftError(RuntimeError):
    def __init__(self, code: int, where: str = ""):
        self.code = int(code)
        msg = lib().dtfft_get_error_string(self.code).decode()
        super().__init__(f"dtFFT error {self.code} in {where}: {msg}")


def _check(code: int, where: str):
    if code != 0:
        raise DtfftError(code, where)


class Execute(enum.IntEnum):
    FORWARD = 11
    BACKWARD = 12


class Transpose(enum.IntEnum):
    X_TO_Y = 1
    Y_TO_X = -1
    Y_TO_Z = 2
    Z_TO_Y = -2
    X_TO_Z = 3
    Z_TO_X = -3


class Layout(enum.IntEnum):
    X_BRICKS = 1
    X_PENCILS = 2
    X_PENCILS_FOURIER = 3
    Y_PENCILS = 4
    Z_PENCILS = 5
    Z_BRICKS = 6


class Reshape(enum.IntEnum):
    X_BRICKS_TO_PENCILS = 11
    X_PENCILS_TO_BRICKS = 12
    Z_PENCILS_TO_BRICKS = 13
    Z_BRICKS_TO_PENCILS = 14


class Precision(enum.IntEnum):
    SINGLE = 0
    DOUBLE = 1


class Effort(enum.IntEnum):
    ESTIMATE = 0
    MEASURE = 1
    PATIENT = 2
    EXHAUSTIVE = 3


class Executor(enum.IntEnum):
    NONE = 0
    FFTW3 = 1
    MKL = 2
    CUFFT = 3
    VKFFT = 4


class R2RKind(enum.IntEnum):
    DCT_1 = 3
    DCT_2 = 5
    DCT_3 = 4
    DCT_4 = 6
    DST_1 = 7
    DST_2 = 9
    DST_3 = 8
    DST_4 = 10


class Backend(enum.IntEnum):
    MPI_DATATYPE = 21
    MPI_P2P = 22
    MPI_A2A = 23
    NCCL = 24
    CUFFTMP = 25
    MPI_P2P_PIPELINED = 26
    NCCL_PIPELINED = 27
    CUFFTMP_PIPELINED = 28
    MPI_RMA = 29
    MPI_RMA_PIPELINED = 30
    MPI_P2P_SCHEDULED = 31
    MPI_P2P_FUSED = 32
    MPI_RMA_FUSED = 33
    MPI_P2P_COMPRESSED = 34
    MPI_RMA_COMPRESSED = 35
    ADAPTIVE = 36
    NCCL_COMPRESSED = 37
    NONE = -111


class Platform(enum.IntEnum):
    HOST = 1
    CUDA = 2


# Build-configuration queries of the reference's Python module
# (src/interfaces/python/__init__.py: is_*_enabled).  This library is the CUDA
# platform only; DTFFT_EXECUTOR_CUFFT and DTFFT_EXECUTOR_VKFFT both select its
# own kernels, and it has no host executors, MPI/NCCL/NVSHMEM backends or
# compression.
def is_fftw_enabled() -> bool:
    return False


def is_mkl_enabled() -> bool:
    return False


def is_cufft_enabled() -> bool:
    return True


def is_vkfft_enabled() -> bool:
    return True


def is_cuda_enabled() -> bool:
    return True


def is_transpose_only_enabled() -> bool:
    return False


def is_nccl_enabled() -> bool:
    return False


def is_nvshmem_enabled() -> bool:
    return False


def is_compression_enabled() -> bool:
    return False


def get_backend_string(backend: "Backend") -> str:
    """Name of a Backend value (dtfft_get_backend_string)."""
    return lib().dtfft_get_backend_string(int(backend)).decode()


def get_precision_string(precision: "Precision") -> str:
    """Name of a Precision value (dtfft_get_precision_string)."""
    return lib().dtfft_get_precision_string(int(precision)).decode()


def get_executor_string(executor: "Executor") -> str:
    """Name of an Executor value (dtfft_get_executor_string)."""
    return lib().dtfft_get_executor_string(int(executor)).decode()


class _CPencil(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_uint8), ("ndims", ctypes.c_uint8),
                ("starts", ctypes.c_int32 * 3), ("counts", ctypes.c_int32 * 3),
                ("size", ctypes.c_size_t)]


class _CConfig(ctypes.Structure):
    _fields_ = [("enable_log", ctypes.c_bool), ("enable_z_slab", ctypes.c_bool),
                ("enable_y_slab", ctypes.c_bool), ("n_measure_warmup_iters", ctypes.c_int32),
                ("n_measure_iters", ctypes.c_int32), ("platform", ctypes.c_int),
                ("stream", ctypes.c_void_p), ("backend", ctypes.c_int), ("reshape_backend", ctypes.c_int),
                ("enable_datatype_backend", ctypes.c_bool), ("enable_mpi_backends", ctypes.c_bool),
                ("enable_pipelined_backends", ctypes.c_bool), ("enable_rma_backends", ctypes.c_bool),
                ("enable_fused_backends", ctypes.c_bool), ("enable_nccl_backends", ctypes.c_bool),
                ("enable_nvshmem_backends", ctypes.c_bool), ("enable_kernel_autotune", ctypes.c_bool),
                ("enable_fourier_reshape", ctypes.c_bool), ("transpose_mode", ctypes.c_int),
                ("access_mode", ctypes.c_int)]


def _declare(L):
    vp, i32, i8, sz = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int8, ctypes.c_size_t
    P = ctypes.POINTER
    L.dtfft_get_error_string.restype = ctypes.c_char_p
    L.dtfft_get_error_string.argtypes = [ctypes.c_int]
    L.dtfft_get_backend_string.restype = ctypes.c_char_p
    L.dtfft_get_backend_string.argtypes = [ctypes.c_int]
    for name in ("dtfft_get_precision_string", "dtfft_get_executor_string"):
        getattr(L, name).restype = ctypes.c_char_p
        getattr(L, name).argtypes = [ctypes.c_int]
    L.dtfft_get_version.restype = i32
    for name in ("dtfft_create_plan_c2c", "dtfft_create_plan_r2c"):
        getattr(L, name).argtypes = [i8, P(i32), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, P(vp)]
    L.dtfft_create_plan_r2r.argtypes = [i8, P(i32), P(ctypes.c_int), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, P(vp)]
    for name in ("dtfft_create_plan_c2c_pencil", "dtfft_create_plan_r2c_pencil"):
        getattr(L, name).argtypes = [P(_CPencil), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, P(vp)]
    L.dtfft_create_plan_r2r_pencil.argtypes = [P(_CPencil), P(ctypes.c_int), ctypes.c_int, ctypes.c_int,
                                               ctypes.c_int, ctypes.c_int, P(vp)]
    L.dtfft_execute.argtypes = [vp, vp, vp, ctypes.c_int, vp]
    L.dtfft_transpose.argtypes = [vp, vp, vp, ctypes.c_int, vp]
    L.dtfft_transpose_start.argtypes = [vp, vp, vp, ctypes.c_int, vp, P(vp)]
    L.dtfft_transpose_end.argtypes = [vp, vp]
    L.dtfft_reshape.argtypes = [vp, vp, vp, ctypes.c_int, vp]
    L.dtfft_destroy.argtypes = [P(vp)]
    L.dtfft_get_local_sizes.argtypes = [vp, P(i32), P(i32), P(i32), P(i32), P(sz)]
    for name in ("dtfft_get_alloc_size", "dtfft_get_aux_size", "dtfft_get_aux_bytes", "dtfft_get_aux_size_reshape",
                 "dtfft_get_aux_bytes_reshape", "dtfft_get_aux_size_transpose", "dtfft_get_aux_bytes_transpose",
                 "dtfft_get_element_size", "dtfft_get_alloc_bytes"):
        getattr(L, name).argtypes = [vp, P(sz)]
    L.dtfft_get_pencil.argtypes = [vp, ctypes.c_int, P(_CPencil)]
    L.dtfft_vgrid_get_pencil.argtypes = [vp, ctypes.c_int, i32, P(_CPencil), P(sz)]
    L.dtfft_vgrid_get_nranks.argtypes = [vp, P(i32)]
    L.dtfft_vgrid_cart_create.argtypes = [i32, P(i32), P(ctypes.c_int)]
    L.dtfft_vgrid_world_create.argtypes = [i32, P(ctypes.c_int)]
    L.dtfft_vgrid_pencils_create.argtypes = [i32, i32, P(i32), P(i32), P(ctypes.c_int)]
    L.dtfft_reshape_start.argtypes = [vp, vp, vp, ctypes.c_int, vp, P(vp)]
    L.dtfft_reshape_end.argtypes = [vp, vp]
    L.dtfft_vgrid_free.argtypes = [P(ctypes.c_int)]
    L.dtfft_get_z_slab_enabled.argtypes = [vp, P(ctypes.c_bool)]
    L.dtfft_get_y_slab_enabled.argtypes = [vp, P(ctypes.c_bool)]
    L.dtfft_get_dims.argtypes = [vp, P(i8), P(P(i32))]
    L.dtfft_get_grid_dims.argtypes = [vp, P(i8), P(P(i32))]
    L.dtfft_get_stream.argtypes = [vp, P(vp)]
    L.dtfft_get_executor.argtypes = [vp, P(ctypes.c_int)]
    L.dtfft_get_precision.argtypes = [vp, P(ctypes.c_int)]
    L.dtfft_get_backend.argtypes = [vp, P(ctypes.c_int)]
    L.dtfft_get_reshape_backend.argtypes = [vp, P(ctypes.c_int)]
    L.dtfft_get_platform.argtypes = [vp, P(ctypes.c_int)]
    L.dtfft_mem_alloc.argtypes = [vp, sz, P(vp)]
    L.dtfft_mem_free.argtypes = [vp, vp]
    L.dtfft_report.argtypes = [vp]
    L.dtfft_create_config.argtypes = [P(_CConfig)]
    L.dtfft_set_config.argtypes = [P(_CConfig)]
    L.dtfft_gb_kernel_launch_count.restype = ctypes.c_int64
    L.gb_kernel_create.argtypes = [i32, P(i32), i32, i32, P(i32), i32, i32, P(vp)]
    L.gb_kernel_execute.argtypes = [vp, vp, vp, vp, i32]
    L.gb_kernel_destroy.argtypes = [P(vp)]
    L.gb_fft_create.argtypes = [i32, i32, i32, i32, i32, i32, P(i32), P(i32), P(i32), P(i32), vp, P(vp)]
    L.gb_fft_execute.argtypes = [vp, vp, vp, i32]
    L.gb_fft_destroy.argtypes = [P(vp)]
    L.dtfft_gb_batch_create.argtypes = [i32, P(vp), i32, P(vp)]
    L.dtfft_gb_batch_execute.argtypes = [vp, P(vp), P(vp), P(vp), ctypes.c_int, vp]
    L.dtfft_gb_batch_graph_nodes.argtypes = [vp, P(ctypes.c_int64)]
    L.dtfft_gb_batch_destroy.argtypes = [P(vp)]
    L.dtfft_gb_device_status.argtypes = [i32]
    L.dtfft_gb_device_status.restype = i32
    L.dtfft_gb_set_wait_limit.argtypes = [i32]
    L.dtfft_gb_set_wait_limit.restype = i32


def kernel_launches() -> int:
    return int(lib().dtfft_gb_kernel_launch_count())


def device_status(reset: bool = False) -> int:
    """Status of the bounded waits on the current device after a device
    synchronisation (0 = fine; dtfft_gb_device_status)."""
    return int(lib().dtfft_gb_device_status(1 if reset else 0))


def set_wait_limit(iterations: int) -> None:
    """Iteration limit of the tile kernels' and TMA transpose's waits for their
    bulk copies (dtfft_gb_set_wait_limit; 0 makes them give up at once)."""
    _check(lib().dtfft_gb_set_wait_limit(int(iterations)), "dtfft_gb_set_wait_limit")


WAIT_LIMIT_DEFAULT = 1 << 22


# ---------------------------------------------------------------------------
# Communicators of virtual ranks (include/dtfft_mpi_shim.h)
# ---------------------------------------------------------------------------

def cart_comm(dims) -> int:
    """Cartesian grid of virtual ranks; dims as MPI_Cart_create takes them
    (for a full-rank grid dims[0] is the X axis and must be 1)."""
    arr = (ctypes.c_int32 * len(dims))(*[int(d) for d in dims])
    h = ctypes.c_int()
    _check(lib().dtfft_vgrid_cart_create(len(dims), arr, ctypes.byref(h)), "dtfft_vgrid_cart_create")
    return h.value


def world_comm(nprocs: int) -> int:
    """`nprocs` virtual ranks without a topology: the planner picks the grid."""
    h = ctypes.c_int()
    _check(lib().dtfft_vgrid_world_create(int(nprocs), ctypes.byref(h)), "dtfft_vgrid_world_create")
    return h.value


def pencils_comm(blocks) -> int:
    """Virtual ranks that each own a block: `blocks[r] = (starts, counts)` in
    dtfft_pencil_t order (dims[0] fastest).  Create the plan with
    `Pencil(*blocks[0])` and this communicator."""
    nd = len(blocks[0][0])
    st = [int(v) for b in blocks for v in b[0]]
    ct = [int(v) for b in blocks for v in b[1]]
    h = ctypes.c_int()
    _check(lib().dtfft_vgrid_pencils_create(len(blocks), nd, _dims_arr(st), _dims_arr(ct), ctypes.byref(h)),
           "dtfft_vgrid_pencils_create")
    return h.value


# ---------------------------------------------------------------------------
# Config
# ---------------------------------------------------------------------------

class Config:
    """Mirror of dtfft_config_t (reference include/dtfft.h:1159-1395)."""

    def __init__(self, **kw):
        c = _CConfig()
        _check(lib().dtfft_create_config(ctypes.byref(c)), "dtfft_create_config")
        self._c = c
        for k, v in kw.items():
            setattr(self, k, v)

    def __setattr__(self, k, v):
        if k == "_c":
            object.__setattr__(self, k, v)
            return
        if k == "stream" and v is not None and not isinstance(v, int):
            v = int(getattr(v, "cuda_stream", v))
        setattr(self._c, k, v)

    def __getattr__(self, k):
        return getattr(object.__getattribute__(self, "_c"), k)


def set_config(cfg: Config):
    _check(lib().dtfft_set_config(ctypes.byref(cfg._c)), "dtfft_set_config")


# ---------------------------------------------------------------------------
# Plans
# ---------------------------------------------------------------------------

class Pencil:
    """Local box of one layout (starts/counts in natural Fortran order)."""

    def __init__(self, starts, counts, dim=0):
        self.starts = [int(s) for s in starts]
        self.counts = [int(c) for c in counts]
        self.ndims = len(self.counts)
        self.dim = int(dim)
        n = 1
        for c in self.counts:
            n *= c
        self.size = n

    @classmethod
    def _from_c(cls, p: _CPencil):
        return cls(list(p.starts)[:p.ndims], list(p.counts)[:p.ndims], p.dim)

    def _to_c(self) -> _CPencil:
        p = _CPencil()
        p.ndims = self.ndims
        for i in range(self.ndims):
            p.starts[i] = self.starts[i]
            p.counts[i] = self.counts[i]
        return p

    def __repr__(self):
        return f"Pencil(dim={self.dim}, starts={self.starts}, counts={self.counts})"


def _ptr(x) -> Optional[int]:
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return int(x.data_ptr())
    raise TypeError(f"expected a torch CUDA tensor or a device pointer, got {type(x)}")


class Plan:
    """Owner of a dtfft_plan_t (reference Python Plan, src/interfaces/python/__init__.py:396-720)."""

    _kind = "c2c"

    def __init__(self, handle: ctypes.c_void_p):
        self._h = handle

    # -- execution ----------------------------------------------------------
    def execute(self, input, output, execute_type: Execute, aux=None):
        _check(lib().dtfft_execute(self._h, _ptr(input), _ptr(output), int(execute_type), _ptr(aux)), "dtfft_execute")

    def transpose(self, input, output, transpose_type: Transpose, aux=None):
        _check(lib().dtfft_transpose(self._h, _ptr(input), _ptr(output), int(transpose_type), _ptr(aux)),
               "dtfft_transpose")

    def transpose_start(self, input, output, transpose_type: Transpose, aux=None):
        req = ctypes.c_void_p()
        _check(lib().dtfft_transpose_start(self._h, _ptr(input), _ptr(output), int(transpose_type), _ptr(aux),
                                           ctypes.byref(req)), "dtfft_transpose_start")
        return req

    def transpose_end(self, request):
        _check(lib().dtfft_transpose_end(self._h, request), "dtfft_transpose_end")

    def reshape(self, input, output, reshape_type: Reshape, aux=None):
        _check(lib().dtfft_reshape(self._h, _ptr(input), _ptr(output), int(reshape_type), _ptr(aux)), "dtfft_reshape")

    def reshape_start(self, input, output, reshape_type: Reshape, aux=None):
        req = ctypes.c_void_p()
        _check(lib().dtfft_reshape_start(self._h, _ptr(input), _ptr(output), int(reshape_type), _ptr(aux),
                                         ctypes.byref(req)), "dtfft_reshape_start")
        return req

    def reshape_end(self, request):
        _check(lib().dtfft_reshape_end(self._h, request), "dtfft_reshape_end")

    def report(self):
        _check(lib().dtfft_report(self._h), "dtfft_report")

    def destroy(self):
        if self._h:
            h = ctypes.c_void_p(self._h.value if isinstance(self._h, ctypes.c_void_p) else self._h)
            _check(lib().dtfft_destroy(ctypes.byref(h)), "dtfft_destroy")
            self._h = None

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                self.destroy()
        except Exception:
            pass

    # -- properties ---------------------------------------------------------
    def _size(self, fn) -> int:
        v = ctypes.c_size_t()
        _check(getattr(lib(), fn)(self._h, ctypes.byref(v)), fn)
        return int(v.value)

    alloc_size = property(lambda s: s._size("dtfft_get_alloc_size"))
    alloc_bytes = property(lambda s: s._size("dtfft_get_alloc_bytes"))
    aux_size = property(lambda s: s._size("dtfft_get_aux_size"))
    aux_bytes = property(lambda s: s._size("dtfft_get_aux_bytes"))
    aux_size_transpose = property(lambda s: s._size("dtfft_get_aux_size_transpose"))
    aux_bytes_transpose = property(lambda s: s._size("dtfft_get_aux_bytes_transpose"))
    aux_size_reshape = property(lambda s: s._size("dtfft_get_aux_size_reshape"))
    aux_bytes_reshape = property(lambda s: s._size("dtfft_get_aux_bytes_reshape"))
    element_size = property(lambda s: s._size("dtfft_get_element_size"))

    @property
    def dtype(self):
        """numpy dtype of the plan's buffers, as the reference's Python Plan
        derives it: complex for C2C plans, real for R2C and R2R plans."""
        import numpy as np
        es = self.element_size
        if isinstance(self, PlanC2C):
            return np.dtype(np.complex128 if es == 16 else np.complex64)
        return np.dtype(np.float64 if es == 8 else np.float32)

    @property
    def local_sizes(self):
        nd = self.ndims
        a = [(ctypes.c_int32 * 3)() for _ in range(4)]
        al = ctypes.c_size_t()
        _check(lib().dtfft_get_local_sizes(self._h, a[0], a[1], a[2], a[3], ctypes.byref(al)), "dtfft_get_local_sizes")
        return tuple(list(x)[:nd] for x in a) + (int(al.value),)

    @property
    def ndims(self) -> int:
        n = ctypes.c_int8()
        _check(lib().dtfft_get_dims(self._h, ctypes.byref(n), None), "dtfft_get_dims")
        return int(n.value)

    def _dims(self, fn):
        n = ctypes.c_int8()
        p = ctypes.POINTER(ctypes.c_int32)()
        _check(getattr(lib(), fn)(self._h, ctypes.byref(n), ctypes.byref(p)), fn)
        return [int(p[i]) for i in range(n.value)]

    dims = property(lambda s: s._dims("dtfft_get_dims"))
    grid_dims = property(lambda s: s._dims("dtfft_get_grid_dims"))

    def _bool(self, fn):
        v = ctypes.c_bool()
        _check(getattr(lib(), fn)(self._h, ctypes.byref(v)), fn)
        return bool(v.value)

    z_slab_enabled = property(lambda s: s._bool("dtfft_get_z_slab_enabled"))
    y_slab_enabled = property(lambda s: s._bool("dtfft_get_y_slab_enabled"))

    def _int(self, fn):
        v = ctypes.c_int()
        _check(getattr(lib(), fn)(self._h, ctypes.byref(v)), fn)
        return int(v.value)

    executor = property(lambda s: Executor(s._int("dtfft_get_executor")))
    precision = property(lambda s: Precision(s._int("dtfft_get_precision")))
    backend = property(lambda s: Backend(s._int("dtfft_get_backend")))
    reshape_backend = property(lambda s: Backend(s._int("dtfft_get_reshape_backend")))
    platform = property(lambda s: Platform(s._int("dtfft_get_platform")))

    @property
    def stream(self) -> int:
        v = ctypes.c_void_p()
        _check(lib().dtfft_get_stream(self._h, ctypes.byref(v)), "dtfft_get_stream")
        return int(v.value or 0)

    def get_pencil(self, layout: Layout) -> Pencil:
        p = _CPencil()
        _check(lib().dtfft_get_pencil(self._h, int(layout), ctypes.byref(p)), "dtfft_get_pencil")
        return Pencil._from_c(p)

    # -- virtual ranks ------------------------------------------------------
    @property
    def nranks(self) -> int:
        v = ctypes.c_int32()
        _check(lib().dtfft_vgrid_get_nranks(self._h, ctypes.byref(v)), "dtfft_vgrid_get_nranks")
        return int(v.value)

    def vrank_pencil(self, layout: Layout, rank: int):
        """(Pencil, element offset) of virtual rank `rank` in `layout`."""
        p = _CPencil()
        off = ctypes.c_size_t()
        _check(lib().dtfft_vgrid_get_pencil(self._h, int(layout), int(rank), ctypes.byref(p), ctypes.byref(off)),
               "dtfft_vgrid_get_pencil")
        return Pencil._from_c(p), int(off.value)


def _dims_arr(dims):
    return (ctypes.c_int32 * len(dims))(*[int(d) for d in dims])


def _create(fn, *args):
    h = ctypes.c_void_p()
    _check(getattr(lib(), fn)(*args, ctypes.byref(h)), fn)
    return h


class PlanC2C(Plan):
    _kind = "c2c"

    def __init__(self, dims_or_pencil, comm: int = COMM_WORLD, precision: Precision = Precision.DOUBLE,
                 effort: Effort = Effort.ESTIMATE, executor: Executor = Executor.NONE, config: Config = None):
        if config is not None:
            set_config(config)
        if isinstance(dims_or_pencil, Pencil):
            h = _create("dtfft_create_plan_c2c_pencil", ctypes.byref(dims_or_pencil._to_c()), int(comm),
                        int(precision), int(effort), int(executor))
        else:
            d = list(dims_or_pencil)
            h = _create("dtfft_create_plan_c2c", len(d), _dims_arr(d), int(comm), int(precision), int(effort),
                        int(executor))
        super().__init__(h)


class PlanR2C(Plan):
    _kind = "r2c"

    def __init__(self, dims_or_pencil, comm: int = COMM_WORLD, precision: Precision = Precision.DOUBLE,
                 effort: Effort = Effort.ESTIMATE, executor: Executor = Executor.NONE, config: Config = None):
        if config is not None:
            set_config(config)
        if isinstance(dims_or_pencil, Pencil):
            h = _create("dtfft_create_plan_r2c_pencil", ctypes.byref(dims_or_pencil._to_c()), int(comm),
                        int(precision), int(effort), int(executor))
        else:
            d = list(dims_or_pencil)
            h = _create("dtfft_create_plan_r2c", len(d), _dims_arr(d), int(comm), int(precision), int(effort),
                        int(executor))
        super().__init__(h)


class PlanR2R(Plan):
    _kind = "r2r"

    def __init__(self, dims_or_pencil, kinds=None, comm: int = COMM_WORLD, precision: Precision = Precision.DOUBLE,
                 effort: Effort = Effort.ESTIMATE, executor: Executor = Executor.NONE, config: Config = None):
        if config is not None:
            set_config(config)
        k = None
        if kinds:
            k = (ctypes.c_int * len(kinds))(*[int(x) for x in kinds])
        if isinstance(dims_or_pencil, Pencil):
            h = _create("dtfft_create_plan_r2r_pencil", ctypes.byref(dims_or_pencil._to_c()), k, int(comm),
                        int(precision), int(effort), int(executor))
        else:
            d = list(dims_or_pencil)
            h = _create("dtfft_create_plan_r2r", len(d), _dims_arr(d), k, int(comm), int(precision), int(effort),
                        int(executor))
        super().__init__(h)


class Batch:
    """Several plans executed with one CUDA graph launch (dtfft_gb_batch_*)."""

    def __init__(self, plans, lanes: int = 0):
        self._plans = list(plans)
        arr = (ctypes.c_void_p * len(self._plans))(*[p._h.value if isinstance(p._h, ctypes.c_void_p) else p._h
                                                       for p in self._plans])
        h = ctypes.c_void_p()
        _check(lib().dtfft_gb_batch_create(len(self._plans), arr, int(lanes), ctypes.byref(h)),
               "dtfft_gb_batch_create")
        self._h = h

    def execute(self, inputs, outputs, execute_type: Execute, auxs=None, stream=None):
        n = len(self._plans)
        ins = (ctypes.c_void_p * n)(*[_ptr(x) for x in inputs])
        outs = (ctypes.c_void_p * n)(*[_ptr(x) for x in outputs])
        ax = (ctypes.c_void_p * n)(*[_ptr(x) for x in auxs]) if auxs is not None else None
        s = None if stream is None else int(getattr(stream, "cuda_stream", stream))
        _check(lib().dtfft_gb_batch_execute(self._h, ins, outs, ax, int(execute_type), s), "dtfft_gb_batch_execute")

    @property
    def graph_nodes(self) -> int:
        v = ctypes.c_int64()
        _check(lib().dtfft_gb_batch_graph_nodes(self._h, ctypes.byref(v)), "dtfft_gb_batch_graph_nodes")
        return int(v.value)

    def destroy(self):
        if self._h:
            _check(lib().dtfft_gb_batch_destroy(ctypes.byref(self._h)), "dtfft_gb_batch_destroy")
            self._h = None
