"""Oracle (test infrastructure only): decomposition of plans built from
user-defined blocks, restated in plain Python from the reference.

Only tests/ use this module, as the oracle of the library's own geometry
(dtfft_vgrid_get_pencil) and data movement.  Parity is pinned by the
reference's own test of this path, tests/c/test_c2c_3d_c.c:105-136 (2, 4 and 8
processes on 96x64x512, expected grids 1x1x2, 1x2x2, 1x2x4; in_starts equal
to the user's block when X is not split) and by the round trip it checks.

Reference procedures restated (file:line in the dtFFT source tree):
  create_pencil_init       src/dtfft_pencil.F90:777-908
  create_1d_comm           src/dtfft_pencil.F90:1034-1081
  from_bricks              src/dtfft_pencil.F90:520-775 (non-cartesian branch)
  pencil%create            src/dtfft_pencil.F90:109-227
  get_local_size           src/dtfft_pencil.F90:237-279
  create_pencils_and_comm  src/dtfft_transpose_plan.F90:1084-1131
  reshape_plan%create      src/dtfft_reshape_plan.F90:98-260

A communicator is a dict rank -> tuple of member ranks (in communicator rank
order).  Boxes are (starts, counts) in the layout's own dim order.
"""
from __future__ import annotations

import numpy as np

TILE = 32   # DEF_TILE_SIZE, src/dtfft_parameters.F90:555


class PencilError(Exception):
    def __init__(self, code):
        super().__init__(code)
        self.code = code


# error codes of include/dtfft.h
E_STARTS, E_COUNTS, E_SHAPE, E_OVERLAP, E_CONT = 28, 27, 29, 30, 31


def _self(P):
    return {r: (r,) for r in range(P)}


def _split(parent, color, key):
    """MPI_Comm_split inside every group of `parent`: by color, ordered by
    (key, rank in parent)."""
    out = {}
    for r, grp in parent.items():
        mates = [q for q in grp if color[q] == color[r]]
        mates.sort(key=lambda q: (key[q], grp.index(q)))
        out[r] = tuple(mates)
    return out


def _local(n, comm, r, keep=None):
    """get_local_size: (start, count) of rank r; `keep` = (start, count) kept."""
    grp = comm[r]
    P = len(grp)
    if P == 1:
        return 0, n
    me = grp.index(r)
    base, res = divmod(n, P)
    counts = [base + (1 if i >= P - res else 0) for i in range(P)]
    if keep is not None:
        return keep
    return sum(counts[:me]), counts[me]


def pencil_init(starts, counts):
    nd = len(starts[0])
    P = len(starts)
    s = [list(map(int, v)) for v in starts]
    c = [list(map(int, v)) for v in counts]
    if any(v < 0 for b in s for v in b):
        raise PencilError(E_STARTS)
    if any(v < 0 for b in c for v in b):
        raise PencilError(E_COUNTS)
    dims = [max(s[r][d] + c[r][d] for r in range(P)) for d in range(nd)]
    zero = [any(v == 0 for v in c[r]) for r in range(P)]
    for p1 in range(P):
        for p2 in range(p1 + 1, P):
            if zero[p1] or zero[p2]:
                continue
            for d1 in range(nd):
                for d2 in range(d1 + 1, nd):
                    if s[p1][d1] == s[p2][d1] and s[p1][d2] == s[p2][d2] and \
                            (c[p1][d1] != c[p2][d1] or c[p1][d2] != c[p2][d2]):
                        raise PencilError(E_SHAPE)
    for i in range(P):
        for j in range(i + 1, P):
            if zero[i] or zero[j]:
                continue
            if all(s[i][d] < s[j][d] + c[j][d] and s[j][d] < s[i][d] + c[i][d] for d in range(nd)):
                raise PencilError(E_OVERLAP)
    vol = sum(int(np.prod(c[r])) for r in range(P) if not zero[r])
    if vol != int(np.prod(dims)):
        raise PencilError(E_CONT)
    comms = []
    for var in range(nd):
        comm = {}
        for r in range(P):
            nb = []
            for i in range(P):
                matched = all(s[i][j] == s[r][j] and c[i][j] == c[r][j] for j in range(nd) if j != var)
                same = s[i][var] == s[r][var]
                if (matched and not same) or i == r or (matched and same and (c[i][var] == 0 or c[r][var] == 0)):
                    nb.append(i)
            nb.sort(key=lambda q: s[q][var])   # stable, like sort_by_varying_dim
            comm[r] = tuple(nb)
        comms.append(comm)
    return {"nd": nd, "P": P, "dims": dims, "s": s, "c": c, "comms": comms}


def _dims_create2(n):
    best = (n, 1)
    q = 1
    while q * q <= n:
        if n % q == 0:
            best = (n // q, q)
        q += 1
    return best


def from_bricks(b):
    nd, P, dims, s, c = b["nd"], b["P"], b["dims"], b["s"], b["c"]
    B1 = b["comms"][0]
    fast = len(B1[0])
    c0 = c[0]
    if nd == 3 and c0[2] > TILE * fast:
        ys, zs = 1, fast
    elif c0[1] > TILE * fast or nd == 2:
        ys, zs = fast, 1
    else:
        for i in range(2, fast + 1):
            if fast % i or c0[nd - 1] < TILE * i or c0[nd - 1] % i or c0[1] < TILE * i or c0[1] % i:
                continue
            ys, zs = min(i, fast // i), max(i, fast // i)
            break
        else:
            ys, zs = _dims_create2(fast)
    me = {r: B1[r].index(r) for r in range(P)}
    if ys == 1:
        pc2, pc3 = _self(P), B1
        ay, az = {r: 0 for r in range(P)}, dict(me)
    elif zs == 1:
        pc2, pc3 = B1, _self(P)
        ay, az = dict(me), {r: 0 for r in range(P)}
    else:
        ay = {r: me[r] // zs for r in range(P)}
        az = {r: me[r] % zs for r in range(P)}
        pc2 = {r: tuple(sorted((q for q in B1[r] if az[q] == az[r]), key=lambda q: ay[q])) for r in range(P)}
        pc3 = {r: tuple(sorted((q for q in B1[r] if ay[q] == ay[r]), key=lambda q: az[q])) for r in range(P)}
    os_, oc = [], []
    for r in range(P):
        st, ct = [0] * nd, [0] * nd
        ct[0] = dims[0]
        a, n = _local(c[r][1], pc2, r)
        st[1], ct[1] = a + min(s[q][1] for q in pc2[r]), n
        if nd == 3:
            a, n = _local(c[r][2], pc3, r)
            st[2], ct[2] = a + min(s[q][2] for q in pc3[r]), n
        os_.append(st)
        oc.append(ct)
    world = {r: tuple(range(P)) for r in range(P)}
    comms = [_self(P)]
    if nd == 2:
        comms.append(_split(world, {r: 0 for r in range(P)}, {r: os_[r][1] for r in range(P)}))
    else:
        crank = {r: b["comms"][2][r].index(r) for r in range(P)}
        brank = {r: b["comms"][1][r].index(r) for r in range(P)}
        comms.append(_split(world, {r: crank[r] * zs + az[r] for r in range(P)}, {r: os_[r][1] for r in range(P)}))
        comms.append(_split(world, {r: brank[r] * ys + ay[r] for r in range(P)}, {r: os_[r][2] for r in range(P)}))
    return {"nd": nd, "P": P, "dims": dims, "s": os_, "c": oc, "comms": comms}


def geometry(starts, counts, r2c=False, z_slab=True, y_slab=False, fourier_reshape=False):
    """Everything a plan over these blocks decides.

    Returns dict: dims, grid, reshape, z_slab, y_slab, final_reshape and
    per-layout box lists 'x' (transformed type), 'y', 'z', 'xr' (R2C real X),
    'xb' (user bricks), 'zb' (Fourier-space bricks), each a list over ranks of
    (starts, counts) in the layout's own dim order."""
    br = pencil_init(starts, counts)
    nd, P, dims = br["nd"], br["P"], br["dims"]
    td = list(dims)
    if r2c:
        td[0] = dims[0] // 2 + 1
    reshape = len(br["comms"][0][0]) > 1
    ip = from_bricks(br) if reshape else br
    cm = ip["comms"]
    grid = [len(cm[d][0]) for d in range(nd)]
    zs = ys = False
    if nd == 3:
        if grid[1] == 1 and z_slab:
            zs = True
        elif grid[2] == 1 and y_slab:
            ys = True
    X, Y, Z, XR = [], [], [], []
    for r in range(P):
        xs, xc = list(ip["s"][r]), list(ip["c"][r])
        XR.append((list(xs), list(xc)))
        if r2c:
            xc[0] = td[0]
        X.append((xs, xc))
        if nd == 3:
            y0 = _local(td[1], cm[0], r)
            y1 = _local(td[2], cm[2], r, keep=(xs[2], xc[2]))
            y2 = _local(td[0], cm[1], r)
            Y.append(([y0[0], y1[0], y2[0]], [y0[1], y1[1], y2[1]]))
            z0 = _local(td[2], cm[0], r)
            z1 = _local(td[0], cm[1], r, keep=(y2[0], y2[1]))
            z2 = _local(td[1], cm[2], r)
            Z.append(([z0[0], z1[0], z2[0]], [z0[1], z1[1], z2[1]]))
        else:
            y0 = _local(td[1], cm[0], r)
            y1 = _local(td[0], cm[1], r)
            Y.append(([y0[0], y1[0]], [y0[1], y1[1]]))
    g = {"dims": dims, "tdims": td, "grid": grid, "reshape": reshape, "z_slab": zs, "y_slab": ys,
         "final_reshape": False, "x": X, "y": Y, "z": Z, "xr": XR if r2c else X}
    if not reshape:
        return g
    g["xb"] = [(list(br["s"][r]), list(br["c"][r])) for r in range(P)]
    last = Z if nd == 3 else Y
    local = cm[nd - 1]
    col = {r: local[r].index(r) // len(br["comms"][nd - 1][r]) for r in range(P)}
    key = {r: local[r].index(r) for r in range(P)}
    R3 = _split(local, col, key)
    ZB = []
    for r in range(P):
        slow = sum(last[q][1][nd - 1] for q in R3[r])
        a, n = _local(dims[nd - 1], R3, r)
        st, ct = [a] + [0] * (nd - 1), [n] + [0] * (nd - 1)
        if nd == 3:
            st[1], ct[1] = last[r][0][1], last[r][1][1]
        st[nd - 1] = min(last[q][0][nd - 1] for q in R3[r])
        ct[nd - 1] = slow
        ZB.append((st, ct))
    g["zb"] = ZB
    g["final_reshape"] = len(R3[0]) > 1 and fourier_reshape and not zs
    return g


# ---------------------------------------------------------------------------
# data placement for arbitrary per-rank boxes
# ---------------------------------------------------------------------------

def _axes(nd, aligned):
    if nd == 2:
        return (0, 1) if aligned == 1 else (1, 0)
    return {1: (0, 1, 2), 2: (1, 2, 0), 3: (2, 0, 1)}[aligned]


def pack(g: np.ndarray, boxes, aligned: int) -> np.ndarray:
    """Global array (C order, X fastest) -> packed buffer of all ranks' boxes."""
    nd = g.ndim
    ax = _axes(nd, aligned)
    parts = []
    for st, ct in boxes:
        sl = [slice(None)] * nd
        for d in range(nd):
            sl[nd - 1 - ax[d]] = slice(st[d], st[d] + ct[d])
        blk = g[tuple(sl)]
        # C-order axes of blk are global axes reversed; want pencil dim 0 fastest
        perm = [nd - 1 - ax[d] for d in reversed(range(nd))]
        parts.append(np.ascontiguousarray(blk.transpose(perm)).ravel())
    return np.concatenate(parts) if parts else np.zeros(0, g.dtype)


def unpack(p: np.ndarray, gdims, boxes, aligned: int) -> np.ndarray:
    nd = len(gdims)
    ax = _axes(nd, aligned)
    g = np.zeros(tuple(gdims[::-1]), dtype=p.dtype)
    off = 0
    for st, ct in boxes:
        n = int(np.prod(ct))
        blk = p[off:off + n].reshape([ct[d] for d in reversed(range(nd))])
        off += n
        perm = [nd - 1 - ax[d] for d in reversed(range(nd))]
        inv = np.argsort(perm)
        sl = [slice(None)] * nd
        for d in range(nd):
            sl[nd - 1 - ax[d]] = slice(st[d], st[d] + ct[d])
        g[tuple(sl)] = blk.transpose(inv)
    return g
