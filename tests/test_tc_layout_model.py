"""CPU model of the tensor-core row kernel (dtfft_gb300/csrc/fft_tc.cu,
fft_tc_kernel / TcShape): the two DFT-matrix GEMM stages with the kernel's
operand indices give the DFT of each row, the stage-2 A operand's padded
core-matrix strides place every (row, K) element once inside its buffer, the
32 lanes of a warp write that operand without shared-memory bank conflicts,
the kernel's shared memory and tensor memory admit three or four CTAs per
SM, and the rotated tile loop's mbarrier phases and row-scale slots line up."""
import numpy as np
import pytest

# (R1, R2) of the compiled kernels: m = R1 * R2 (tc_pick)
SHAPES = [(16, 16), (16, 32), (32, 24), (32, 32)]
LBO2 = 144


def sbo2(R1, R2):
    s = (2 * R1 // 8) * LBO2
    if R1 == 16:
        while ((R2 // 8) * s // 4) % 32 != 16:
            s += 16
    return s


def shape(R1, R2):
    S = 128 // R1
    K1 = N1 = 2 * R2
    K2 = N2 = 2 * R1
    G2 = (S * R2 + 127) // 128
    B1, B2 = N1 * K1 * 2, N2 * K2 * 2
    A1 = 128 * K1 * 2
    SB = sbo2(R1, R2)
    A2 = G2 * 16 * SB
    # the stage-1 and stage-2 A operands (hi + lo each) share one region
    a_region = 2 * max(A1, A2)
    off_scale = 2 * (B1 + B2) + a_region
    smem = ((off_scale + 8 * S + 15) & ~15) + 16   # two slots of S row scales
    cols = N1 + G2 * N2
    tmem = next(c for c in (32, 64, 128, 256) if cols <= c)
    return dict(S=S, K1=K1, K2=K2, N1=N1, N2=N2, G2=G2, SB=SB, A1=A1, A2=A2, a_region=a_region,
                smem=smem, tmem=tmem)


def a2_off(r2, k, SB):
    row = r2 & 127
    return (r2 >> 7) * 16 * SB + (row >> 3) * SB + (k >> 3) * LBO2 + (row & 7) * 16 + (k & 7) * 2


@pytest.mark.parametrize("R1,R2", SHAPES)
def test_stage2_operand_layout(R1, R2):
    sh = shape(R1, R2)
    seen = set()
    for r2 in range(sh["G2"] * 128):
        for k in range(0, sh["K2"], 2):
            a = a2_off(r2, k, sh["SB"])
            assert a % 4 == 0 and 0 <= a and a + 4 <= sh["A2"]
            assert a not in seen
            seen.add(a)
    # descriptor fields are 16-byte units; a core matrix (8 rows x 16 bytes) is contiguous
    assert LBO2 % 16 == 0 and sh["SB"] % 16 == 0 and LBO2 >= 128
    assert sh["SB"] >= (sh["K2"] // 8) * LBO2


@pytest.mark.parametrize("R1,R2", SHAPES)
def test_stage2_writes_conflict_free(R1, R2):
    sh = shape(R1, R2)
    for w in range(4):
        for k2 in range(R2):
            banks = {}
            for lane in range(32):
                t = 32 * w + lane
                s1, n1 = t // R1, t % R1
                a = a2_off(s1 * R2 + k2, 2 * n1, sh["SB"]) // 4
                banks.setdefault(a % 32, set()).add(a)
            assert max(len(v) for v in banks.values()) == 1


@pytest.mark.parametrize("R1,R2", SHAPES)
def test_ctas_per_sm(R1, R2):
    """Shared memory (227 KB per CTA budget, 1 KB reserved each) and the SM's
    512 tensor-memory columns admit three CTAs per SM, four at 256 points."""
    sh = shape(R1, R2)
    want = 4 if R1 * R2 == 256 else 3
    assert (227 * 1024) // (sh["smem"] + 1024) >= want
    assert 512 // sh["tmem"] >= want
    assert 2 * sh["A1"] <= sh["a_region"] and 2 * sh["A2"] <= sh["a_region"]


def real_dft(R, sign):
    """Real 2R x 2R form of W_R^(j q): row 2j + a (output re/im), column 2q + b."""
    Bm = np.zeros((2 * R, 2 * R))
    for j in range(R):
        for q in range(R):
            ang = sign * 2 * np.pi * ((j * q) % R) / R
            c, s = np.cos(ang), np.sin(ang)
            Bm[2 * j:2 * j + 2, 2 * q:2 * q + 2] = [[c, -s], [s, c]]
    return Bm


@pytest.mark.parametrize("R1,R2", SHAPES)
@pytest.mark.parametrize("sign", [-1, 1])
def test_two_stage_gemm_matches_dft(R1, R2, sign):
    m = R1 * R2
    sh = shape(R1, R2)
    S = sh["S"]
    rng = np.random.default_rng(m)
    x = rng.standard_normal((S, m)) + 1j * rng.standard_normal((S, m))
    tw = np.exp(sign * 2j * np.pi * np.arange(m) / m)
    # stage 1: A row t = (s1, n1), k = 2 n2 + {re, im}
    A1 = np.zeros((128, 2 * R2))
    for t in range(128):
        s1, n1 = t // R1, t % R1
        v = x[s1, n1 + R1 * np.arange(R2)]
        A1[t, 0::2], A1[t, 1::2] = v.real, v.imag
    D1 = A1 @ real_dft(R2, sign).T          # D[v][n] = sum_k A[v][k] B[n][k]
    # twiddles and stage-2 rows r2 = (s1, k2), k = 2 n1 + {re, im}
    A2 = np.zeros((sh["G2"] * 128, 2 * R1))
    for t in range(128):
        s1, n1 = t // R1, t % R1
        y = D1[t, 0::2] + 1j * D1[t, 1::2]
        z = y * tw[(n1 * np.arange(R2)) % m]
        r2 = s1 * R2 + np.arange(R2)
        A2[r2, 2 * n1], A2[r2, 2 * n1 + 1] = z.real, z.imag
    D2 = A2 @ real_dft(R1, sign).T
    out = np.zeros((S, m), dtype=complex)
    for r2 in range(S * R2):
        s, k2 = r2 // R2, r2 % R2
        out[s, np.arange(R1) * R2 + k2] = D2[r2, 0::2] + 1j * D2[r2, 1::2]
    ref = np.fft.fft(x, axis=1) if sign < 0 else np.fft.ifft(x, axis=1) * m
    assert np.abs(out - ref).max() <= 1e-9 * np.abs(ref).max()


def _rotated_schedule(cta, grid, ntiles):
    """Event list of one CTA of the tensor-core kernel's rotated tile loop:
    ("commit", group, tile), ("wait", parity), ("scale_w", slot, tile),
    ("scale_r", slot, tile)."""
    ev = []
    phase = 0

    def stage1(tl, b):
        ev.append(("scale_w", b, tl))
        ev.append(("commit", "mma1", tl))

    if cta < ntiles:
        stage1(cta, 0)
    buf = 0
    tile = cta
    while tile < ntiles:
        ev.append(("wait", phase, "mma1", tile))
        phase ^= 1
        ev.append(("commit", "mma2", tile))
        ev.append(("wait", phase, "mma2", tile))
        phase ^= 1
        if tile + grid < ntiles:
            stage1(tile + grid, buf ^ 1)
        ev.append(("scale_r", buf, tile))
        tile += grid
        buf ^= 1
    return ev


@pytest.mark.parametrize("grid,ntiles", [(1, 1), (1, 5), (3, 3), (3, 10), (4, 17), (456, 1365)])
def test_rotated_loop_bookkeeping(grid, ntiles):
    """The rotated loop keeps one MMA group in flight at a time, so one
    mbarrier with alternating parity serves both stages: every wait is for
    the group committed just before it, with the parity of that completion;
    a tile's results are scaled by the slot its own stage 1 wrote, and no slot
    is rewritten before it is read; nothing is in flight at a normal exit."""
    for cta in range(min(grid, ntiles)):
        ev = _rotated_schedule(cta, grid, ntiles)
        outstanding = None
        completions = 0
        slots = {}
        for e in ev:
            if e[0] == "commit":
                assert outstanding is None, "two MMA groups in flight"
                outstanding = (e[1], e[2])
            elif e[0] == "wait":
                assert outstanding == (e[2], e[3])
                assert e[1] == completions % 2          # parity of this completion
                completions += 1
                outstanding = None
            elif e[0] == "scale_w":
                assert slots.get(e[1]) is None, "slot rewritten before it was read"
                slots[e[1]] = e[2]
            elif e[0] == "scale_r":
                assert slots.get(e[1]) == e[2]
                slots[e[1]] = None
        assert outstanding is None
        tiles = list(range(cta, ntiles, grid))
        assert [e[2] for e in ev if e[0] == "scale_r"] == tiles
