"""CPU tests of the C-ABI boundary: the library loads, exports every function
declared in include/*.h, keeps the reference's enum values, and rejects bad
arguments with the reference's error codes before touching the GPU."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")


def _declared_functions():
    names = set()
    for f in os.listdir(INC):
        if not f.endswith(".h"):
            continue
        src = open(os.path.join(INC, f)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        src = re.sub(r"#define[^\n]*(\\\n[^\n]*)*", "", src)
        for m in re.finditer(r"\b((?:dtfft|gb)_[a-z0-9_]+)\s*\(", src):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_function(dt):
    L = dt.lib()
    missing = [n for n in _declared_functions() if not hasattr(L, n)]
    assert not missing, missing
    assert len(_declared_functions()) >= 58


def test_enum_values_match_reference(dt):
    # include/dtfft_config.h.in of the reference
    assert dt.Execute.FORWARD == 11 and dt.Execute.BACKWARD == 12
    assert [dt.Transpose.X_TO_Y, dt.Transpose.Y_TO_Z, dt.Transpose.X_TO_Z] == [1, 2, 3]
    assert [dt.R2RKind.DCT_1, dt.R2RKind.DCT_2, dt.R2RKind.DCT_3, dt.R2RKind.DCT_4] == [3, 5, 4, 6]
    assert [dt.R2RKind.DST_1, dt.R2RKind.DST_2, dt.R2RKind.DST_3, dt.R2RKind.DST_4] == [7, 9, 8, 10]
    assert dt.Backend.NONE == -111 and dt.Layout.Z_BRICKS == 6
    hdr = open(os.path.join(INC, "dtfft.h")).read()
    for name, val in [("DTFFT_ERROR_R2R_FFT_NOT_SUPPORTED", 101), ("DTFFT_ERROR_NOT_DEVICE_PTR", 300),
                      ("DTFFT_ERROR_INVALID_PLATFORM_EXECUTOR", 401), ("DTFFT_ERROR_INVALID_CART_COMM", 46)]:
        assert re.search(rf"{name} = {val}\b", hdr), name


def test_version(dt):
    assert dt.lib().dtfft_get_version() == 3 * 100000 + 2 * 1000 + 0


def test_error_strings(dt):
    L = dt.lib()
    assert L.dtfft_get_error_string(0) == b"DTFFT_SUCCESS"
    assert b"R2R" in L.dtfft_get_error_string(101)
    assert L.dtfft_get_backend_string(-111) == b"NONE"


def test_config_roundtrip(dt):
    c = dt.Config()
    assert c.enable_z_slab and not c.enable_y_slab
    assert c.n_measure_warmup_iters == 2 and c.n_measure_iters == 5
    assert c.platform == dt.Platform.CUDA
    bad = dt.Config(n_measure_iters=0)
    with pytest.raises(dt.DtfftError) as e:
        dt.set_config(bad)
    assert e.value.code == 34
    dt.set_config(dt.Config())


def _create(dt, ndims, dims, comm, precision=0, effort=0, executor=0):
    L = dt.lib()
    h = ctypes.c_void_p()
    arr = (ctypes.c_int32 * 3)(*(list(dims) + [0] * (3 - len(dims))))
    return L.dtfft_create_plan_c2c(ndims, arr, comm, precision, effort, executor, ctypes.byref(h))


def test_create_argument_errors(dt):
    W = dt.COMM_WORLD
    assert _create(dt, 4, [8, 8, 8], W) == 3            # INVALID_N_DIMENSIONS
    assert _create(dt, 3, [8, 0, 8], W) == 4            # INVALID_DIMENSION_SIZE
    assert _create(dt, 3, [8, 8, 8], 0x1234) == 5       # INVALID_COMM_TYPE
    assert _create(dt, 3, [8, 8, 8], W, precision=5) == 6
    assert _create(dt, 3, [8, 8, 8], W, effort=9) == 7
    assert _create(dt, 3, [8, 8, 8], W, executor=9) == 8
    assert _create(dt, 3, [8, 8, 8], W, executor=1) == 401   # FFTW3 on the CUDA platform
    assert _create(dt, 3, [8, 8, 8], dt.cart_comm([2, 2, 2])) == 10   # fast dim split
    assert _create(dt, 2, [8, 8], dt.cart_comm([1, 2, 2])) == 9       # more grid dims than plan dims


def test_r2r_kind_validation(dt):
    L = dt.lib()
    h = ctypes.c_void_p()
    dims = (ctypes.c_int32 * 2)(8, 8)
    kinds = (ctypes.c_int * 2)(5, 42)
    assert L.dtfft_create_plan_r2r(2, dims, kinds, dt.COMM_WORLD, 0, 0, 4, ctypes.byref(h)) == 12


def test_null_handles(dt):
    L = dt.lib()
    assert L.dtfft_execute(None, None, None, 11, None) == 17
    v = ctypes.c_size_t()
    assert L.dtfft_get_alloc_size(None, ctypes.byref(v)) == 1
    assert L.dtfft_destroy(None) == 17


def test_oracle_lib_loads(orc):
    assert orc.lib().orc_num_threads() >= 1


def test_module_queries_and_strings(dt):
    """Module-level queries of the reference's Python module
    (src/interfaces/python/__init__.py:25-72) and the enum-name strings."""
    assert dt.is_cuda_enabled() and dt.is_cufft_enabled() and dt.is_vkfft_enabled()
    assert not (dt.is_fftw_enabled() or dt.is_mkl_enabled() or dt.is_nccl_enabled() or dt.is_nvshmem_enabled()
                or dt.is_compression_enabled() or dt.is_transpose_only_enabled())
    names = [dt.get_backend_string(b) for b in dt.Backend]
    assert all(isinstance(x, str) and x for x in names) and len(set(names)) == len(names)
    assert dt.get_precision_string(dt.Precision.SINGLE) != dt.get_precision_string(dt.Precision.DOUBLE)
    assert dt.get_executor_string(dt.Executor.CUFFT)
