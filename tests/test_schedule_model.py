"""CPU model of the index arithmetic of the warp-per-row tile kernels
(dtfft_gb300/csrc/fft_tile.cuh, tile_stages / tile_row_fft): every compiled
(M, E, radices) schedule, run lane by lane in numpy with the kernels' Stockham
indices, exchange swizzle and twiddle exponents, must give the DFT of the row
in natural order (lane t ends with points t + T q).  Also the swizzles the
kernels rely on are permutations of the row, the fused kernel's store warps
write every (row, point) of a tile once to its destination, and the TMA
transpose writes every element of a tile once with its shared-memory reads
inside the tile."""
import numpy as np
import pytest

# (M, E, radices) of the compiled tile kernels (fft_tile_f32.cu / fft_tile_f64.cu)
SCHEDULES = [(256, 8, (8, 8, 4)), (512, 16, (16, 16, 2)), (768, 24, (8, 8, 4, 3)), (1024, 32, (16, 16, 4))]


def xsw(i):
    return i ^ ((i >> 4) & 15)


def osw8(r, i, lgsh):
    return i ^ (((r >> 1) << lgsh) & 15)


def dft(x, s):
    n = len(x)
    k = np.arange(n)
    return np.exp(s * 2j * np.pi * np.outer(k, k) / n) @ x


def model_row(x, E, rads, s):
    M = len(x)
    T = M // E
    tw = np.exp(s * 2j * np.pi * np.arange(M) / M)          # direction table W_M^(s e)
    row = x.astype(complex).copy()
    v = np.array([[row[t + T * q] for q in range(E)] for t in range(T)])
    Ns = 1
    for si, R in enumerate(rads):
        last = si == len(rads) - 1
        B = E // R
        tstep = M // (Ns * R)
        new_row = np.full(M, np.nan, dtype=complex)
        for t in range(T):
            for b in range(B):
                j = t + b * T
                k = (t % Ns) if T % Ns == 0 else (j % Ns)
                w = np.array([v[t][b + r * B] for r in range(R)])
                if Ns > 1:
                    w = w * np.array([tw[(tstep * k * r) % M] for r in range(R)])
                w = dft(w, s)
                if last:
                    for r in range(R):
                        v[t][b + r * B] = w[r]
                else:
                    base = (j - k) * R + k
                    for r in range(R):
                        new_row[xsw(base + r * Ns)] = w[r]
        if not last:
            assert not np.isnan(new_row).any(), "exchange left a slot unwritten"
            v = np.array([[new_row[xsw(t + T * q)] for q in range(E)] for t in range(T)])
        Ns *= R
    out = np.empty(M, dtype=complex)
    for t in range(T):
        for q in range(E):
            out[t + T * q] = v[t][q]
    return out


@pytest.mark.parametrize("M,E,rads", SCHEDULES)
@pytest.mark.parametrize("s", [-1, 1])
def test_tile_schedule_is_the_dft(M, E, rads, s):
    assert int(np.prod(rads)) == M and M == 32 * E
    rng = np.random.default_rng(M)
    x = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    got = model_row(x, E, rads, s)
    ref = np.fft.fft(x) if s < 0 else np.fft.ifft(x) * M
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-12


@pytest.mark.parametrize("M", [256, 512, 768, 1024])
def test_swizzles_are_permutations(M):
    assert sorted(xsw(i) for i in range(M)) == list(range(M))
    for S in (2, 4, 8, 16):                     # complex64 tiles of S rows
        lgNP = (S.bit_length() - 1) - 1
        lgsh = 4 - lgNP
        for r in range(S):
            assert sorted(osw8(r, i, lgsh) for i in range(M)) == list(range(M))


def store_warp_writes(M, S, NSW, nrows, segs):
    """(row, point) pairs each store-warp thread of fft_tile_xpose_kernel
    writes for one complex64 tile (the loop over segments and points of the
    kernel's write-out), with the destination element of each."""
    lgS = S.bit_length() - 1
    lgNP = lgS - 1
    gstep = (32 * NSW) >> lgNP
    out = []
    for st in range(32 * NSW):
        lp = st & ((1 << lgNP) - 1)
        g0 = st >> lgNP
        for (i0, i1, dst_off, di) in segs:
            npts = i1 - i0
            r0 = 2 * lp
            if r0 >= nrows:
                continue
            two = r0 + 1 < nrows
            for ii in range(g0, npts, gstep):
                i = i0 + ii
                d = dst_off + ii * di + r0
                out.append((r0, i, d))
                if two:
                    out.append((r0 + 1, i, d + 1))
    return out


@pytest.mark.parametrize("S", [2, 4, 8, 16])
@pytest.mark.parametrize("NSW", [4, 5, 8])
def test_store_warps_write_every_point_once(S, NSW):
    M = 256
    segs = [(0, 100, 0, 40), (100, 256, 4000, 40)]      # two destination ranks, 40 rows each
    for nrows in sorted({1, max(1, S - 1), S}):
        w = store_warp_writes(M, S, NSW, nrows, segs)
        assert sorted((r, i) for r, i, _ in w) == [(r, i) for r in range(nrows) for i in range(M)]
        for r, i, d in w:
            seg = next(s for s in segs if s[0] <= i < s[1])
            assert d == seg[2] + (i - seg[0]) * seg[3] + r


def tma_tile_writes(ES, ra, rb):
    """(a, b) elements the 256 threads of box_transpose_tma_kernel write for
    one tile with ra x rb valid elements, and the shared-memory byte offsets
    they read (transpose_tma.cu)."""
    IN = 128 // ES
    TA, TB = 4 * IN, 32
    writes, reads = [], []
    for tid in range(256):
        lane, warp = tid & 31, tid >> 5
        b = lane
        if b >= rb:
            continue
        if ES == 4:
            for aq in range(warp, TA // 4, 8):
                a = 4 * aq
                if a >= ra:
                    break
                k, ai = a // IN, a % IN
                chunk = ((ai * ES) >> 4) ^ (b & 7)
                reads.append(k * TB * 128 + b * 128 + chunk * 16)
                for j in range(4):
                    if a + j < ra:
                        writes.append((a + j, b))
        elif ES == 8:
            for ap in range(warp, TA // 2, 8):
                a = 2 * ap
                if a >= ra:
                    break
                k, ai = a // IN, a % IN
                chunk = ((ai * ES) >> 4) ^ (b & 7)
                reads.append(k * TB * 128 + b * 128 + chunk * 16)
                writes.append((a, b))
                if a + 1 < ra:
                    writes.append((a + 1, b))
        else:
            for a in range(warp, TA, 8):
                if a >= ra:
                    break
                k, ai = a // IN, a % IN
                chunk = ai ^ (b & 7)
                reads.append(k * TB * 128 + b * 128 + chunk * 16)
                writes.append((a, b))
    return writes, reads, TA, TB


@pytest.mark.parametrize("ES", [4, 8, 16])
def test_tma_transpose_tile_coverage(ES):
    IN = 128 // ES
    for ra in sorted({1, 3, IN, 4 * IN - 1, 4 * IN}):
        for rb in (1, 7, 31, 32):
            w, r, TA, TB = tma_tile_writes(ES, ra, rb)
            assert sorted(w) == sorted((a, b) for a in range(ra) for b in range(rb))
            assert all(0 <= x and x + 16 <= 4 * TB * 128 for x in r)


def _tma_unswizzle(offset, lb):
    """Byte offset inside a 1024-byte aligned staging buffer that the tensor-map
    swizzle of an lb-byte span reads for logical byte `offset` of the box: the
    16-byte chunk index (bits 4..6 for 128 bytes, 4..5 for 64) is XORed with
    address bits 7..9 (7..8)."""
    if lb == 128:
        return offset ^ (((offset >> 7) & 7) << 4)
    return offset ^ (((offset >> 7) & 3) << 4)


@pytest.mark.parametrize("es,M,rpw", [(8, 256, 2), (8, 512, 2), (16, 256, 2), (16, 512, 2), (8, 768, 1), (8, 1024, 1)])
def test_tensor_store_staging_matches_the_map_swizzle(es, M, rpw):
    """fft_tile_xpose_tma_kernel: compute warp w owns rows rpw*w .. rpw*w + rpw - 1
    of an S-row tile (S = 8 * rpw for complex64, 4 * rpw for complex128) and
    writes point i of them into line i (S * es bytes) at 16-byte chunk
    c ^ (i & 7) (128-byte lines) or c ^ ((i >> 1) & 3) (64-byte lines), where c
    is the chunk that holds the rows in the unswizzled line.  The tensor store
    of a box of lines [i0, i0 + L) with i0 % 8 == 0, read through the line's
    swizzle, must deliver element (u, i) of the destination block from where
    row u's value of point i was written, for every (u, i), each staging byte
    used once."""
    ncw = 8 if es == 8 else 4
    S = ncw * rpw
    lb = S * es
    assert lb in (64, 128)

    def chunk(i, c):
        return (c ^ (i & 7)) << 4 if lb == 128 else (c ^ ((i >> 1) & 3)) << 4

    written = {}
    for w in range(ncw):
        ua = rpw * w
        for i in range(M):
            line = i * lb
            if es == 8 and rpw == 2:
                off = line + chunk(i, w)
                written[off] = (ua, i)
                written[off + 8] = (ua + 1, i)
            elif es == 8:
                written[line + chunk(i, ua >> 1) + 8 * (ua & 1)] = (ua, i)
            else:
                for r in range(rpw):
                    written[line + chunk(i, ua + r)] = (ua + r, i)
    assert len(written) == S * M                         # every (row, point) once
    assert all(0 <= o and o + es <= M * lb for o in written)
    for i0 in sorted({0, 8, 40} | set(range(0, M, 128))):
        L = min(256, M - i0)
        for i in range(i0, i0 + L):
            for u in range(S):
                logical = (i - i0) * lb + u * es          # box element (u, i): u fastest, lb-byte lines
                phys = _tma_unswizzle(i0 * lb + logical, lb)
                assert written[phys] == (u, i)
