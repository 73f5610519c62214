"""CPU check of the packed linear DP schedule (csrc/linear4.cu): four DP rows
per lane in two registers of two 16-bit halves.

A numpy emulation of one warp, step by step, with the kernel's exact
arithmetic: 32-bit packed registers, per-half wrapping add-min
(__viaddmin_u16x2), full 32-bit adds (with carries between the halves) for
the insert candidates, byte permutes for the cost operands, the queue and
boundary-slab timing, per-block column windows, the forced out-of-band
cells and the clamp of the first strips.  Layout:
  * lane k owns rows 128t + 4k + m (m = 0..3) of strip t; row m runs
    lam[m] = (0, 1, 3, 4) steps behind row 0, lane k runs 7k steps behind
    lane 0, so row 4k+m is at band index i at step tW + 7k + lam[m] + i
    (lane k-1's row 3 reaches lane k's row 0 two steps after it is computed:
    the shuffle that carries it runs a step ahead, off the critical path);
  * X = {row 0, row 2}, Y = {row 1, row 3} (low half, high half);
  * W = max(roundup32(wd + 4), 288): at least 4 out-of-band steps between
    strips, so that every strip-dependent input of a lane (column window,
    cost profile, delete costs) switches at one step, d = 0.
The emulated costs and the alignments walked back from the emulated moves
must equal the oracle's cost_2 and align_2 (no GPU needed).
"""
import numpy as np
import pytest

from oracle import oracle as O
from poyd_gb300 import synth

M16 = 0xFFFF
INF16 = 0xC000
INF2 = 0xC000C000
LAM = (0, 1, 3, 4)
LANE_LAG = 7  # lane k-1's row 3 feeds lane k's row 0 two steps later
R3_LAG = LANE_LAG * 31 + 4  # lane 31's row 3 relative to lane 0's row 0
MIN_PERIOD = 288  # lane 31's row-3 values flushed two blocks before lane 0 reads them


def band(a, b, m):
    la, lb = len(a), len(b)
    swap = la < lb
    s1, s2 = (b, a) if swap else (a, b)
    l1, l2 = len(s1), len(s2)
    dw = O.deltaw(a, b, m)
    dif = l1 - l2
    width, height = min(50 + dw, l2), min(dif + 50 + dw, l1)
    full = delta = 0
    if np.float32(1.5) * np.float32(l2) <= np.float32(l1):
        full = 1
    elif 2 * height < l1:
        delta = 1
    elif 8 >= l1 - height:
        full = 1
    dlo, dhi = (-(l1 - 1), l2 - 1) if full else (delta - height, width - 1)
    return swap, np.asarray(s1, np.int64), np.asarray(s2, np.int64), dlo, dhi - dlo + 1


def add_min16(a, b, c):
    """__viaddmin_u16x2: per half min((a + b) mod 2^16, c)."""
    lo = np.minimum((a + b) & M16, c & M16)
    hi = np.minimum(((a >> 16) + (b >> 16)) & M16, (c >> 16) & M16)
    return (hi << 16) | lo


def lop_inf(a, mask):
    """LOP3 (a & ~mask) | (INF2 & mask): halves selected by `mask` (0xFFFF
    per half) become exactly INF16."""
    return (a & ~mask & 0xFFFFFFFF) | (INF2 & mask)


def eligible(L1, L2, maxc, sc):
    """The 16-bit lanes hold every in-band value (with 260 rows of slack for
    the rows past the matrix) below INF16."""
    return sc * maxc * (max(L1, L2) + 260) + 6 < INF16


# Row thresholds of the first-strips mask: row m of a lane is out of the
# matrix (j < 0) or not started while its step offset d (from the lane's
# strip start) is below a threshold.  Variant by the lane's row-0 offset
# off0 = -dlo - (first row of the lane): off0 <= 0, 1, 2 use thresholds on
# d itself; off0 >= 3 on e = d - off0.
TRI_TH = {0: (0, 1, 3, 4), 1: (1, 1, 3, 4), 2: (2, 2, 3, 4), 3: (0, 0, 1, 1)}
# Right-edge forced cells: row m at band index wd, e = lam[m] steps after
# the lane's edge anchor (next strip start - (W - wd)).
EDGE_AT = LAM


def masks_from(th, e):
    """(X mask, Y mask): X = rows 0, 2; Y = rows 1, 3."""
    mk = [np.where(e < th[mm], M16, 0) for mm in range(4)]
    return mk[0] | (mk[2] << 16), mk[1] | (mk[3] << 16)


def emulate4(a, b, m, choice=True, kinds=None, trace=None):
    cost = O.cm_tables(m)["cost"].reshape(32, 32).astype(np.int64)
    gap = 16
    swap, s1, s2, dlo, wd = band(a, b, m)
    L1, L2 = len(s1), len(s2)
    swaped = not swap
    sc = 4 if choice else 1
    maxc = int(cost[1:32, 1:32].max())
    assert eligible(L1, L2, maxc, sc)
    T = (L1 + 127) // 128
    W = max((wd + 4 + 31) // 32 * 32, MIN_PERIOD)
    Gg = W - wd
    nblk = ((T - 1) * W + R3_LAG + wd + 31) // 32
    rank_i = (1 if swaped else 2) if choice else 0
    rank_d = (3 - rank_i) if choice else 0
    bias = sc * int(cost[s1[0], s2[0]])
    k = np.arange(32, dtype=np.int64)
    tri_last = max(0, (-dlo - 1) // 128)  # strips with rows left of column 0 (and strip 0)

    def row_char(t, mm):
        r = 128 * t + 4 * k + mm
        ok = (t >= 0) & (t < T) & (r < L1)
        return np.where(ok, s1[np.clip(r, 0, L1 - 1)], gap)

    cache = {}

    def strip_consts(t):
        """Per lane: row characters, packed delete costs (X, Y) and the cost
        profile prof[c] (four bytes: rows 0..3 against column char c)."""
        if t not in cache:
            ach = [row_char(t, mm) for mm in range(4)]
            cd = [sc * cost[x, gap] + rank_d for x in ach]
            prof = np.zeros((32, 32), np.int64)
            for mm in range(4):
                prof |= (sc * cost[ach[mm][None, :], np.arange(32)[:, None]]) << (8 * mm)
            cache[t] = (ach, cd[0] | (cd[2] << 16), cd[1] | (cd[3] << 16), prof)
        return cache[t]

    gtab = sc * cost[gap, :] + rank_i

    def lookups(t, G):
        """Window word (column char, insert cost) and profile word of lane
        k's row 0 column at step G in strip t."""
        j = 128 * t + dlo + (G - t * W) - (LANE_LAG - 4) * k
        c = np.where((j >= 0) & (j < L2), s2[np.clip(j, 0, L2 - 1)], gap)
        return gtab[c], strip_consts(t)[3][c, k]

    def block_kind(G0):
        t = G0 // W
        o = G0 - t * W
        for tt in (t, t + 1):  # the period of the block and the next one
            if 0 <= tt <= tri_last:
                end = tt * W + max(-dlo - 128 * tt + (LANE_LAG - 4) * 31 + 1, R3_LAG)
                if G0 <= end and G0 + 31 >= tt * W:
                    return "slow"
        if o + 31 >= W - Gg or o <= R3_LAG:
            return "mixed"
        return "plain"

    # boundary slab: the row above strip t (values in the high half)
    bnd = np.full(wd, INF16 << 16, np.int64)
    bnd[-dlo] = 0

    def qload(blk):
        G = 32 * blk + k
        t = G // W
        x = G - t * W + 1
        x = np.where(x == W, 0, x)
        return np.where(x < wd, bnd[np.minimum(x, wd - 1)], INF16 << 16)

    X = np.full(32, INF2, np.int64)
    Y = X.copy()
    Yp = X.copy()  # Y two steps back: lane k-1's row 3 for lane k's row 0
    DXp = X.copy()
    DXp[0] = (INF16 << 16) | (bnd[0] >> 16)
    g_prev = np.full(32, 0, np.int64)
    pr_prev = np.zeros(32, np.int64)
    q = qload(0)
    dm = np.zeros((nblk, 32, 8), np.int64)
    result = None
    rf = L1 - 1
    tf, kf, mf = rf // 128, (rf % 128) // 4, rf % 4
    Gf = tf * W + LANE_LAG * kf + LAM[mf] + (L2 - 1 - rf - dlo)
    for blk in range(nblk):
        G0 = 32 * blk
        qn = qload(blk + 1)
        kind = block_kind(G0)
        if Gf // 32 == blk:
            kind = "slow"
        if kinds is not None:
            kinds[kind] = kinds.get(kind, 0) + 1
        for v in range(32):
            G = G0 + v
            recv = np.roll(Yp, 1)
            up = recv.copy()
            up[0] = q[0]
            q = np.roll(q, -1)
            t_l = (G - LANE_LAG * k) // W  # the strip each lane's lookups use
            g = np.zeros(32, np.int64)
            pr = np.zeros(32, np.int64)
            cdX = np.zeros(32, np.int64)
            cdY = np.zeros(32, np.int64)
            for t in np.unique(t_l):
                sel = t_l == t
                gg, pp = lookups(t, G)
                _, cx, cy, _ = strip_consts(t)
                g[sel], pr[sel], cdX[sel], cdY[sel] = gg[sel], pp[sel], cx[sel], cy[sel]
            if kind == "plain":
                assert (t_l == t_l[0]).all()
            DX = ((Y & M16) << 16) | (up >> 16)
            caX = (pr & 0xFF) | (((pr_prev >> 16) & 0xFF) << 16)
            caY = ((pr >> 8) & 0xFF) | (((pr_prev >> 24) & 0xFF) << 16)
            ci = g | (g_prev << 16)
            # right edge: row m at index wd of the strip before each switch
            e = (G - LANE_LAG * k + Gg) % W
            t_old = (G - LANE_LAG * k + Gg) // W - 1
            ex, ey = masks_from((1, 2, 4, 5), np.where(t_old >= 0, e, 99))
            ex0, ey0 = masks_from((0, 1, 3, 4), np.where(t_old >= 0, e, 99))
            fx, fy = ex & ~ex0, ey & ~ey0   # exactly e == lam[m]
            # first strips: rows left of column 0 or not yet started, relative
            # to the block's strip t0 (lanes still in strip t0 - 1 of a later
            # period are not masked: their cells left of column 0 stay >= INF)
            t0 = G0 // W
            d = G - LANE_LAG * k - t0 * W
            off0 = -dlo - 128 * t0 - 4 * k
            var = np.clip(off0, 0, 3)
            tx = np.zeros(32, np.int64)
            ty = np.zeros(32, np.int64)
            if t0 <= tri_last:
                gate = (t0 == 0) | (t_l == t0)
                for vv in range(4):
                    sel = (var == vv) & gate
                    ee = d - off0 if vv == 3 else d
                    mx, my = masks_from(TRI_TH[vv], ee)
                    tx[sel], ty[sel] = mx[sel], my[sel]
            if kind == "plain":
                assert not (fx | fy | tx | ty).any()
            if kind != "slow":
                assert not (tx | ty).any()
            # align and insert terms first (they need no value of this step);
            # the insert add is one 32-bit add of both halves
            tX = add_min16(DXp, caX, (X + ci) & 0xFFFFFFFF)
            tY = add_min16(X, caY, (Y + ci) & 0xFFFFFFFF)
            Xn = add_min16(DX, cdX, tX)
            if choice:
                rX = Xn & 0x00030003
                wx = 4 * (v // 16) + (v // 8) % 2
                dm[blk, :, wx] = (dm[blk, :, wx] * 4 + rX) & 0xFFFFFFFF
                Xn = Xn & 0xFFFCFFFC
            Xn = lop_inf(Xn, fx | tx)
            Yn = add_min16(Xn, cdY, tY)
            if choice:
                rY = Yn & 0x00030003
                wy = 4 * (v // 16) + 2 + (v // 8) % 2
                dm[blk, :, wy] = (dm[blk, :, wy] * 4 + rY) & 0xFFFFFFFF
                Yn = Yn & 0xFFFCFFFC
            Yn = lop_inf(Yn, fy | ty)
            if G == Gf:
                reg = Xn if mf in (0, 2) else Yn
                result = int((reg[kf] >> (16 if mf >= 2 else 0)) & M16)
            if trace is not None:  # cell values by (row, band index), for debugging
                for mm in range(4):
                    reg = Xn if mm in (0, 2) else Yn
                    val = (reg >> (16 if mm >= 2 else 0)) & M16
                    tt = (G - LANE_LAG * k - LAM[mm]) // W
                    ii = G - LANE_LAG * k - LAM[mm] - tt * W
                    rr = 128 * tt + 4 * k + mm
                    for kk in range(32):
                        if 0 <= rr[kk] < L1 and ii[kk] < wd:
                            trace[(int(rr[kk]), int(ii[kk]))] = int(val[kk])
            q[31] = Yn[31]
            Yp = Y
            DXp, X, Y, g_prev, pr_prev = DX, Xn, Yn, g, pr
        for L in range(32):  # lane 31's row-3 values of this block: the next boundary row
            p = G0 + L - R3_LAG
            t31 = p // W
            x = p - t31 * W
            if p >= 0 and x < wd:
                bnd[x] = q[L]
        q = qn
    cost_v = (result - bias) // sc
    if not choice:
        return cost_v, None
    r, j, ra, rb = L1 - 1, L2 - 1, [], []
    while r > 0 or (r == 0 and j >= 0):
        t, kk, mm = r // 128, (r % 128) // 4, r % 4
        G = t * W + LANE_LAG * kk + LAM[mm] + (j - r) - dlo
        vv = G % 32
        wrd = int(dm[G // 32, kk, 4 * (vv // 16) + 2 * (mm & 1) + (vv // 8) % 2])
        code = (wrd >> (2 * (7 - vv % 8) + 16 * (mm >> 1))) & 3
        mv = 0 if code == 0 else (1 if (code == 1) == swaped else 2)
        cr = s1[r] if mv != 1 else gap
        cc = s2[j] if mv != 2 else gap
        r -= mv != 1
        j -= mv != 2
        ca, cb = (cc, cr) if swap else (cr, cc)
        ra.append(ca)
        rb.append(cb)
    return cost_v, (np.array(ra[::-1], np.uint8), np.array(rb[::-1], np.uint8))


def _cases():
    rng = np.random.default_rng(11)
    g = synth.with_gap
    out = []
    for n1, n2 in [(0, 0), (0, 5), (1, 1), (2, 7), (130, 128), (127, 129), (200, 301),
                   (500, 10), (250, 251), (300, 140), (700, 690), (90, 400)]:
        out.append((g(synth.random_dna(rng, n1, 0.1)), g(synth.random_dna(rng, n2, 0.1))))
    A, B = synth.pair_batch(5, 3, lmin=600, lmax=1300)
    out += list(zip(A, B))
    # gap-bearing sequences (wide deltaw: the full-rows band case) and a
    # full plane by the length ratio
    a = g(synth.random_dna(rng, 900, 0.05))
    b = synth.mutate(rng, a[1:].copy(), 0.15, 0.02)
    sel = rng.random(len(b)) < 0.5
    b[sel] = 16 | b[sel]
    out.append((a, g(b)))
    a = g(synth.random_dna(rng, 1400, 0.05))
    out.append((a, g(synth.mutate(rng, a[1:850].copy(), 0.2, 0.03))))
    return out


@pytest.mark.parametrize("model", [(1, 2), (3, 1)])
def test_packed_schedule_matches_oracle(model):
    m = O.cm_dna(model[0], model[1], -1)
    for a, b in _cases():
        c_ref, ra, rb = O.align_2(a, b, m)
        c_choice, (ea, eb) = emulate4(a, b, m, choice=True)
        # costs-only mode (values x1, no moves) on the shorter pairs
        c_cost = emulate4(a, b, m, choice=False)[0] if len(a) + len(b) < 1000 else c_ref
        assert c_choice == c_ref == c_cost == O.cost_2(a, b, m), (len(a), len(b))
        assert np.array_equal(ea, ra) and np.array_equal(eb, rb), (len(a), len(b))
