"""CPU oracle for dtFFT's single-GPU execute path.

TEST INFRASTRUCTURE ONLY.  This module is the oracle of the GPU library's parity tests
(`dtfft_gb300`).  Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg import it; the product never does.

Three parts:

* Data movement: `vgrid_transpose` drives the C restatement in
  dtfft_oracle.c of the reference's generic reshape handle
  (pack -> all-to-all-v -> unpack per virtual rank,
  src/dtfft_reshape_handle_generic.F90:174-759).  `global_to_packed` /
  `packed_to_global` give the independent "pencil semantics" view
  (each rank holds a sub-box of the global array stored aligned-axis-first,
  src/dtfft_transpose_plan.F90:1084-1131) that the tests cross-check the
  restatement against.

* FFT values: FP64 numpy/scipy transforms with FFTW's conventions as used by
  the executors (sign -1 forward, unnormalised; R2C keeps n/2+1;
  R2R kinds = FFTW r2r kinds, inverse kinds from src/dtfft_utils.F90:447-471).
  The algorithm lives in FFTW3 (un-vendored, unpinned version, used by
  src/interfaces/fft/fftw/dtfft_executor_fftw_m.F90:91-226); it is restated
  here by the published DFT/DCT/DST definitions (`dft_direct`,
  `r2r_direct`), against which scipy's pocketfft is pinned in the tests.

* Plan semantics: `execute_oracle` applies the execute schedules of
  src/dtfft_plan.F90:877-1101 at the level of global arrays and returns the
  packed per-rank output the reference would hold.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libdtfft_oracle.so")

# dtFFT enum values (include/dtfft_config.h.in)
X_TO_Y, Y_TO_X, Y_TO_Z, Z_TO_Y, X_TO_Z, Z_TO_X = 1, -1, 2, -2, 3, -3
DCT_1, DCT_2, DCT_3, DCT_4, DST_1, DST_2, DST_3, DST_4 = 3, 5, 4, 6, 7, 9, 8, 10

_lib = None


def build(force: bool = False) -> str:
    """Compile dtfft_oracle.c into oracle/_build/libdtfft_oracle.so (gcc + OpenMP)."""
    src = os.path.join(HERE, "dtfft_oracle.c")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src)):
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", src, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        i32p = ctypes.POINTER(ctypes.c_int)
        L.orc_local_size.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, i32p, i32p]
        L.orc_pencil.argtypes = [ctypes.c_int, i32p, i32p, ctypes.c_int, ctypes.c_int, i32p, i32p]
        L.orc_rank_offset.argtypes = [ctypes.c_int, i32p, i32p, ctypes.c_int, ctypes.c_int]
        L.orc_rank_offset.restype = ctypes.c_int64
        L.orc_nranks.argtypes = [ctypes.c_int, i32p]
        L.orc_vgrid_transpose.argtypes = [ctypes.c_int, i32p, i32p, ctypes.c_int,
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        L.orc_num_threads.restype = ctypes.c_int
        for name in ("orc_permute_forward",):
            getattr(L, name).argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, i32p, ctypes.c_int]
        for name in ("orc_permute_backward", "orc_permute_backward_start"):
            getattr(L, name).argtypes = [ctypes.c_void_p, ctypes.c_void_p, i32p, ctypes.c_int]
        L.orc_permute_backward_end_one.argtypes = [ctypes.c_void_p, ctypes.c_void_p, i32p, i32p, ctypes.c_int]
        for name in ("orc_unpack_one", "orc_pack_one"):
            getattr(L, name).argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, i32p, i32p, ctypes.c_int]
        _lib = L
    return _lib


def _ivec(v):
    arr = (ctypes.c_int * 3)(*([int(x) for x in v] + [0] * (3 - len(v))))
    return arr


# ----------------------------------------------------------------------------
# Pencils of a (1, g1[, g2]) grid
# ----------------------------------------------------------------------------

def norm_grid(ndims, grid):
    """Grid as (1, g1, g2) / (1, g1) in Fortran (fastest-first) order."""
    grid = list(grid)
    if len(grid) == ndims - 1:
        grid = [1] + grid
    assert len(grid) == ndims and grid[0] == 1
    return grid


def nranks(ndims, grid):
    grid = norm_grid(ndims, grid)
    return grid[1] * (grid[2] if ndims == 3 else 1)


def local_size(n, P, r):
    s, c = ctypes.c_int(), ctypes.c_int()
    lib().orc_local_size(n, P, r, ctypes.byref(s), ctypes.byref(c))
    return s.value, c.value


def pencil(ndims, gdims, grid, layout, rank):
    """(starts, counts) of `rank`'s pencil `layout` (1=X, 2=Y, 3=Z), aligned-first order."""
    grid = norm_grid(ndims, grid)
    s, c = _ivec([0, 0, 0]), _ivec([0, 0, 0])
    lib().orc_pencil(ndims, _ivec(gdims), _ivec(grid), layout, rank, s, c)
    return list(s)[:ndims], list(c)[:ndims]


def rank_offset(ndims, gdims, grid, layout, rank):
    grid = norm_grid(ndims, grid)
    return int(lib().orc_rank_offset(ndims, _ivec(gdims), _ivec(grid), layout, rank))


def layout_total(ndims, gdims, grid, layout):
    return rank_offset(ndims, gdims, grid, layout, nranks(ndims, grid))


def vgrid_transpose(ndims, gdims, grid, ttype, packed_in: np.ndarray) -> np.ndarray:
    """Reference transpose of a packed multi-rank buffer (C restatement)."""
    grid = norm_grid(ndims, grid)
    src = np.ascontiguousarray(packed_in)
    es = src.dtype.itemsize
    rl = {1: 2, -1: 1, 2: 3, -2: 2, 3: 3, -3: 1}[ttype]
    out = np.zeros(layout_total(ndims, gdims, grid, rl), dtype=src.dtype)
    rc = lib().orc_vgrid_transpose(ndims, _ivec(gdims), _ivec(grid), ttype,
                                   src.ctypes.data, out.ctypes.data, es)
    if rc != 0:
        raise RuntimeError(f"orc_vgrid_transpose failed: {rc}")
    return out


# ----------------------------------------------------------------------------
# Global <-> packed per-rank views (pencil semantics)
# ----------------------------------------------------------------------------

def _block_from_global(g, ndims, layout, s, c):
    """Local block of a pencil from the global array g (C order: [z][y][x] / [y][x]).

    Returns the block as a flat array in the pencil's Fortran order
    (aligned axis fastest)."""
    if ndims == 2:
        if layout == 1:   # (X, Y): X fastest
            blk = g[s[1]:s[1] + c[1], s[0]:s[0] + c[0]]
        else:             # (Y, X): Y fastest
            blk = g[s[0]:s[0] + c[0], s[1]:s[1] + c[1]].T
        return np.ascontiguousarray(blk).ravel()
    if layout == 1:       # (X, Y, Z)
        blk = g[s[2]:s[2] + c[2], s[1]:s[1] + c[1], s[0]:s[0] + c[0]]
    elif layout == 2:     # (Y, Z, X): C order [x][z][y]
        blk = g[s[1]:s[1] + c[1], s[0]:s[0] + c[0], s[2]:s[2] + c[2]].transpose(2, 0, 1)
    else:                 # (Z, X, Y): C order [y][x][z]
        blk = g[s[0]:s[0] + c[0], s[2]:s[2] + c[2], s[1]:s[1] + c[1]].transpose(1, 2, 0)
    return np.ascontiguousarray(blk).ravel()


def global_to_packed(g: np.ndarray, ndims, grid, layout) -> np.ndarray:
    """Pack a global array (numpy C order, x fastest) into the multi-rank layout."""
    gdims = list(g.shape[::-1])
    grid = norm_grid(ndims, grid)
    parts = []
    for r in range(nranks(ndims, grid)):
        s, c = pencil(ndims, gdims, grid, layout, r)
        parts.append(_block_from_global(g, ndims, layout, s, c))
    return np.concatenate(parts) if parts else np.zeros(0, g.dtype)


def packed_to_global(p: np.ndarray, ndims, gdims, grid, layout) -> np.ndarray:
    grid = norm_grid(ndims, grid)
    g = np.zeros(tuple(gdims[::-1]), dtype=p.dtype)
    off = 0
    for r in range(nranks(ndims, grid)):
        s, c = pencil(ndims, gdims, grid, layout, r)
        n = int(np.prod(c))
        blk = p[off:off + n]
        off += n
        if n == 0:
            continue
        if ndims == 2:
            if layout == 1:
                g[s[1]:s[1] + c[1], s[0]:s[0] + c[0]] = blk.reshape(c[1], c[0])
            else:
                g[s[0]:s[0] + c[0], s[1]:s[1] + c[1]] = blk.reshape(c[1], c[0]).T
        elif layout == 1:
            g[s[2]:s[2] + c[2], s[1]:s[1] + c[1], s[0]:s[0] + c[0]] = blk.reshape(c[2], c[1], c[0])
        elif layout == 2:
            g[s[1]:s[1] + c[1], s[0]:s[0] + c[0], s[2]:s[2] + c[2]] = \
                blk.reshape(c[2], c[1], c[0]).transpose(1, 2, 0)
        else:
            g[s[0]:s[0] + c[0], s[2]:s[2] + c[2], s[1]:s[1] + c[1]] = \
                blk.reshape(c[2], c[1], c[0]).transpose(2, 0, 1)
    return g


# ----------------------------------------------------------------------------
# FFT value oracle (FP64), FFTW conventions
# ----------------------------------------------------------------------------

INVERSE_KIND = {DCT_1: DCT_1, DCT_2: DCT_3, DCT_3: DCT_2, DCT_4: DCT_4,
                DST_1: DST_1, DST_2: DST_3, DST_3: DST_2, DST_4: DST_4}
_SCIPY_KIND = {DCT_1: ("dct", 1), DCT_2: ("dct", 2), DCT_3: ("dct", 3), DCT_4: ("dct", 4),
               DST_1: ("dst", 1), DST_2: ("dst", 2), DST_3: ("dst", 3), DST_4: ("dst", 4)}


def dft_direct(x: np.ndarray, sign: int) -> np.ndarray:
    """Unnormalised DFT by definition, Y_k = sum_j X_j exp(sign*2*pi*i*j*k/n), along the last axis."""
    n = x.shape[-1]
    j = np.arange(n)
    w = np.exp(sign * 2j * np.pi * np.outer(j, j) / n)
    return x.astype(np.complex128) @ w


def r2r_direct(x: np.ndarray, kind: int) -> np.ndarray:
    """FFTW r2r definitions (REDFT00..RODFT11), along the last axis, by direct sums."""
    x = x.astype(np.float64)
    n = x.shape[-1]
    j = np.arange(n)[:, None]
    k = np.arange(n)[None, :]
    if kind == DCT_1:      # REDFT00
        m = 2 * np.cos(np.pi * j * k / (n - 1))
        m[0, :] = 1.0
        m[n - 1, :] = (-1.0) ** np.arange(n)
    elif kind == DCT_2:    # REDFT10
        m = 2 * np.cos(np.pi * (j + 0.5) * k / n)
    elif kind == DCT_3:    # REDFT01
        m = 2 * np.cos(np.pi * j * (k + 0.5) / n)
        m[0, :] = 1.0
    elif kind == DCT_4:    # REDFT11
        m = 2 * np.cos(np.pi * (j + 0.5) * (k + 0.5) / n)
    elif kind == DST_1:    # RODFT00
        m = 2 * np.sin(np.pi * (j + 1) * (k + 1) / (n + 1))
    elif kind == DST_2:    # RODFT10
        m = 2 * np.sin(np.pi * (j + 0.5) * (k + 1) / n)
    elif kind == DST_3:    # RODFT01
        m = 2 * np.sin(np.pi * (j + 1) * (k + 0.5) / n)
        m[n - 1, :] = (-1.0) ** np.arange(n)
    elif kind == DST_4:    # RODFT11
        m = 2 * np.sin(np.pi * (j + 0.5) * (k + 0.5) / n)
    else:
        raise ValueError(kind)
    return x @ m


def r2r(x: np.ndarray, kind: int, axis: int) -> np.ndarray:
    import scipy.fft as sf
    fam, t = _SCIPY_KIND[kind]
    f = sf.dct if fam == "dct" else sf.dst
    return f(np.asarray(x, dtype=np.float64), type=t, axis=axis, norm=None)


def _axes_c(ndims):
    """numpy axis of Fortran dim d (0 = X fastest)."""
    return [ndims - 1 - d for d in range(ndims)]


def forward_values(g: np.ndarray, kind: str, kinds=None) -> np.ndarray:
    """Forward transform of a global array with FFTW conventions (FP64)."""
    nd = g.ndim
    ax = _axes_c(nd)
    if kind == "c2c":
        return np.fft.fftn(g.astype(np.complex128), axes=ax[::-1])
    if kind == "r2c":
        # R2C along X (last numpy axis) then C2C along the others
        return np.fft.rfftn(g.astype(np.float64), axes=ax[::-1])
    if kind == "r2r":
        y = g.astype(np.float64)
        for d in range(nd):
            y = r2r(y, kinds[d], ax[d])
        return y
    raise ValueError(kind)


def backward_values(G: np.ndarray, kind: str, real_dims=None, kinds=None) -> np.ndarray:
    """Unnormalised backward transform (FFTW conventions)."""
    nd = G.ndim
    ax = _axes_c(nd)
    if kind == "c2c":
        n = int(np.prod(G.shape))
        return np.fft.ifftn(G, axes=ax[::-1]) * n
    if kind == "r2c":
        shape = tuple(real_dims[::-1])
        n = int(np.prod(shape))
        return np.fft.irfftn(G, s=shape, axes=ax[::-1]) * n
    if kind == "r2r":
        y = G.astype(np.float64)
        for d in range(nd):
            y = r2r(y, INVERSE_KIND[kinds[d]], ax[d])
        return y
    raise ValueError(kind)


def r2r_roundtrip_scale(dims, kinds) -> float:
    """FFTW round-trip factor for r2r kinds (tests/python/test_r2r_kinds_py.py:1-16)."""
    s = 1.0
    for n, k in zip(dims, kinds):
        if k == DCT_1:
            s *= 2 * (n - 1)
        elif k == DST_1:
            s *= 2 * (n + 1)
        else:
            s *= 2 * n
    return s


def roundtrip_threshold(n_global: int, single: bool) -> float:
    """Max-abs round-trip threshold 5*log2(N)*eps of tests/test_utils.F90:89-109."""
    if single:
        eps = float(np.nextafter(np.float32(1), np.float32(2)) - np.nextafter(np.float32(1), np.float32(0)))
    else:
        eps = float(np.nextafter(1.0, 2.0) - np.nextafter(1.0, 0.0))
    return 5.0 * math.log2(n_global) * eps


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.complex128 if np.iscomplexobj(a) or np.iscomplexobj(b) else np.float64)
    b = np.asarray(b, dtype=a.dtype)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))


# ----------------------------------------------------------------------------
# Plan semantics: layouts the execute schedules start and end in
# ----------------------------------------------------------------------------

def final_layout(ndims: int, z_slab: bool, y_slab: bool) -> int:
    """Aligned layout after a forward execute (src/dtfft_plan.F90:877-1101;
    get_local_sizes out_dim rule src/dtfft_pencil.F90:438-463)."""
    if ndims == 2 or y_slab:
        return 2
    return 3


def choose_grid(ndims, gdims, nprocs=1, z_slab=True, y_slab=False, cart=None):
    """Grid choice of src/dtfft_transpose_plan.F90:58-209 for the CUDA platform.

    Returns (grid, is_z_slab, is_y_slab).  With `cart` (user cartesian dims in
    Fortran order, fastest first) the grid is taken from it."""
    tile = 32  # DEF_TILE_SIZE, src/dtfft_parameters.F90:555
    if cart is not None:
        grid = list(cart)
        if len(grid) == ndims - 1:
            grid = [1] + grid
        elif len(grid) == ndims - 2:
            grid = [1, 1] + grid
        zs = ys = False
        if ndims == 3:
            if grid[1] == 1 and z_slab:
                zs = True
            elif grid[2] == 1 and y_slab:
                ys = True
        return grid, zs, ys
    if ndims == 2:
        return [1, nprocs], False, False
    cond1 = tile <= gdims[2] // nprocs
    cond2 = tile <= gdims[0] // nprocs and tile <= gdims[1] // nprocs
    if cond1 and z_slab:
        return [1, 1, nprocs], True, False
    if cond2 and y_slab:
        return [1, nprocs, 1], False, True
    if cond1:
        return [1, 1, nprocs], False, False
    if cond2:
        return [1, nprocs, 1], False, False
    # MPI_Dims_create of the remaining dims (balanced factorisation)
    best = None
    for a in range(1, nprocs + 1):
        if nprocs % a == 0:
            b = nprocs // a
            if a >= b and (best is None or a - b < best[0] - best[1]):
                best = (a, b)
    return [1, best[0], best[1]], False, False


# ----------------------------------------------------------------------------
# Full-size checks: packed positions and sampled spectrum lines (FP64)
# ----------------------------------------------------------------------------

def packed_index(ndims, gdims, grid, layout, coords) -> np.ndarray:
    """Positions in the packed multi-rank buffer of layout `layout` of the
    global points `coords` (array (n, ndims) of (x, y[, z]) indices): rank r's
    block starts at rank_offset and stores its pencil aligned-axis-first
    (src/dtfft_transpose_plan.F90:1084-1131)."""
    coords = np.asarray(coords, dtype=np.int64).reshape(-1, ndims)
    grid = norm_grid(ndims, grid)
    # global axis held by pencil dim d of this layout
    if ndims == 2:
        axes = [0, 1] if layout == 1 else [1, 0]
    else:
        axes = {1: [0, 1, 2], 2: [1, 2, 0], 3: [2, 0, 1]}[layout]
    out = np.full(len(coords), -1, dtype=np.int64)
    for r in range(nranks(ndims, grid)):
        s, c = pencil(ndims, gdims, grid, layout, r)
        loc = np.stack([coords[:, axes[d]] - s[d] for d in range(ndims)], axis=1)
        inside = np.all((loc >= 0) & (loc < np.asarray(c)[None, :]), axis=1)
        if not inside.any():
            continue
        lin = np.zeros(int(inside.sum()), dtype=np.int64)
        stride = 1
        for d in range(ndims):
            lin += loc[inside, d] * stride
            stride *= c[d]
        out[inside] = rank_offset(ndims, gdims, grid, layout, r) + lin
    if (out < 0).any():
        raise ValueError("a point lies outside every rank's block")
    return out


def _basis(n, k, kind, axis_kind):
    """Column k of the forward transform of length n along one axis:
    exp(-2 pi i j k / n) for C2C and R2C axes, FFTW's r2r kernels otherwise."""
    if axis_kind == "dft":
        return np.exp(-2j * np.pi * np.arange(n) * k / n)
    m = r2r_direct(np.eye(n), kind)
    return m[:, k]


def _line_transform(v, n_out, axis_kind, kind):
    if axis_kind == "dft":
        return np.fft.fft(v)[:n_out]
    return r2r(np.real(v), kind, axis=-1)


def sampled_lines(g: np.ndarray, kind: str, axis: int, points, kinds=None, chunk=16):
    """FP64 values of the forward 3D transform of `g` (numpy C order [z][y][x],
    FFTW conventions as forward_values) along `axis` (0 = X, 1 = Y, 2 = Z) at
    the fixed output indices `points` of the two other axes, in X, Y, Z order
    ((ky, kz) for X lines, (kx, kz) for Y lines, (kx, ky) for Z lines).

    The transform is separable, so each line is the contraction of g with the
    basis vectors of the two fixed indices followed by the 1D transform along
    `axis`; g is read once per call in chunks of `chunk` z-planes, which keeps
    inputs of several GiB within host memory.  R2C: X is the halved axis
    (n/2 + 1 outputs), the others are C2C.  Returns (len(points), n_axis_out)."""
    nz, ny, nx = g.shape
    n = [nx, ny, nz]
    other = [a for a in range(3) if a != axis]
    pts = [tuple(int(v) for v in p) for p in points]
    K = len(pts)

    def axis_kind(a):
        return "r2r" if kind == "r2r" else "dft"

    def kind_of(a):
        return kinds[a] if kind == "r2r" else None

    dt_acc = np.float64 if kind == "r2r" else np.complex128
    bases = {a: np.stack([_basis(n[a], p[i], kind_of(a), axis_kind(a)) for p in pts], axis=1).astype(dt_acc)
             for i, a in enumerate(other)}
    acc = np.zeros((K, n[axis]), dtype=dt_acc)
    for z0 in range(0, nz, chunk):
        G = np.asarray(g[z0:z0 + chunk]).astype(dt_acc)          # (cz, ny, nx)
        cz = G.shape[0]
        if axis == 2:          # contract x, then y
            T = (G.reshape(-1, nx) @ bases[0]).reshape(cz, ny, K)
            acc[:, z0:z0 + cz] = np.einsum("zyk,yk->kz", T, bases[1])
        elif axis == 1:        # contract x, then z
            T = (G.reshape(-1, nx) @ bases[0]).reshape(cz, ny, K)
            acc += np.einsum("zyk,zk->ky", T, bases[2][z0:z0 + cz])
        else:                  # contract y, then z
            T = np.matmul(G.transpose(0, 2, 1), bases[1])      # (cz, nx, K)
            acc += np.einsum("zxk,zk->kx", T, bases[2][z0:z0 + cz])
    n_out = n[axis] // 2 + 1 if (kind == "r2c" and axis == 0) else n[axis]
    return np.stack([_line_transform(acc[i], n_out, axis_kind(axis), kind_of(axis)) for i in range(K)])


def line_coords(axis: int, point, n_axis: int) -> np.ndarray:
    """Global (x, y, z) indices of one sampled line (see sampled_lines)."""
    other = [a for a in range(3) if a != axis]
    c = np.zeros((n_axis, 3), dtype=np.int64)
    c[:, axis] = np.arange(n_axis)
    c[:, other[0]] = point[0]
    c[:, other[1]] = point[1]
    return c
