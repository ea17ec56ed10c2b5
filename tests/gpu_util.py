"""Helpers shared by the GPU parity tests: run a plan through the C ABI on
torch CUDA buffers and compare with the oracle."""
import numpy as np

_TORCH_DT = {}


def torch_dtype(np_dtype):
    import torch
    return {np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64,
            np.dtype(np.complex64): torch.complex64, np.dtype(np.complex128): torch.complex128}[np.dtype(np_dtype)]


def to_dev(a: np.ndarray, n_alloc: int, dev):
    """Copy a numpy vector into a zero-padded device buffer of n_alloc elements."""
    import torch
    t = torch.zeros(max(n_alloc, a.size), dtype=torch_dtype(a.dtype), device=dev)
    if a.size:
        t[: a.size] = torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    # plans run on their own stream: finish torch's work before handing buffers over
    torch.cuda.synchronize()
    return t


def from_dev(t, n: int, np_dtype) -> np.ndarray:
    import torch
    torch.cuda.synchronize()
    return t[:n].cpu().numpy().astype(np_dtype, copy=False)


def empty(n_alloc: int, np_dtype, dev, fill=np.nan):
    import torch
    t = torch.empty(max(n_alloc, 1), dtype=torch_dtype(np_dtype), device=dev)
    if np.issubdtype(np_dtype, np.complexfloating):
        t.real.fill_(fill)
        t.imag.fill_(fill)
    else:
        t.fill_(fill)
    torch.cuda.synchronize()
    return t


def random_global(shape, np_dtype, seed, dist="uniform"):
    rng = np.random.default_rng(seed)
    if dist == "uniform":
        re = rng.uniform(-1, 1, shape)
        im = rng.uniform(-1, 1, shape)
    else:
        re = rng.standard_normal(shape)
        im = rng.standard_normal(shape)
    if np.issubdtype(np_dtype, np.complexfloating):
        return (re + 1j * im).astype(np_dtype)
    return re.astype(np_dtype)


def comm_for(dt, grid):
    """Virtual communicator for a (1, g1[, g2]) grid; COMM_WORLD for one rank."""
    if all(g == 1 for g in grid):
        return dt.COMM_WORLD
    return dt.cart_comm(grid)
