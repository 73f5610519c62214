"""CPU check of the linear DP's continuous-strip schedule (csrc/linear.cu).

A numpy emulation of one warp -- 32 lanes x 2 rows, one step at a time --
with the kernel's timing: lane k works on strip t during steps
[tW + 3k, tW + 3k + W), W = max(roundup32(wd + 2), 160); the value of the
row above arrives from lane k-1 (lane 0: from the boundary queue, refilled
one 32-step block ahead and flushed by lane 31 after each block); column
characters are read per lane (the per-warp windows); out-of-band cells are
masked; values carry x4 and the move rank in kDpChoice.  The emulated costs
and the alignments walked back from the emulated 2-bit moves must equal the
oracle's cost_2 and align_2 (no GPU needed).
"""
import numpy as np
import pytest

from oracle import oracle as O
from poyd_gb300 import synth


def _band(a, b, m):
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


def emulate(a, b, m, choice=True):
    cost = O.cm_tables(m)["cost"].reshape(32, 32).astype(np.int64)
    gap = 16
    swap, s1, s2, dlo, wd = _band(a, b, m)
    L1, L2 = len(s1), len(s2)
    swaped = not swap
    T = (L1 + 63) // 64
    W = max((wd + 2 + 31) // 32 * 32, 160)
    nblk = ((T - 1) * W + 94 + wd + 31) // 32
    sc, INF = (4, 3 << 25) if choice else (1, 1 << 25)
    rank_i = (1 if swaped else 2) if choice else 0
    rank_d = (3 - rank_i) if choice else 0
    bias = sc * cost[s1[0], s2[0]]
    bnd = np.full(max(wd, 1), INF, np.int64)
    bnd[-dlo] = 0
    k = np.arange(32)
    HA = np.full(32, INF, np.int64)
    HB, diag, Pk = HA.copy(), HA.copy(), HA.copy()

    def qload(blk):
        G = 32 * blk + k
        t = G // W
        x = G - t * W + 1
        x = np.where(x == W, 0, x)
        return np.where(x < wd, bnd[np.minimum(x, wd - 1)], INF)

    q = qload(0)
    diag[0] = bnd[0]
    dm = np.zeros((nblk, 32, 4), np.uint64)
    result = None
    for blk in range(nblk):
        G0 = 32 * blk
        qn = qload(blk + 1)
        for u in range(32):
            G = G0 + u
            up = np.empty(32, np.int64)
            up[1:] = Pk[:-1]
            up[0] = q[0]
            q = np.roll(q, -1)
            pA = G - 3 * k
            s = np.floor_divide(pA, W)
            iA = pA - s * W
            rA = 64 * s + 2 * k
            rB = rA + 1
            jc = rA + dlo + iA
            c = np.where((jc >= 0) & (jc < L2), s2[np.clip(jc, 0, L2 - 1)], 0)
            inside = (s >= 0) & (s < T)
            offA, offB = np.maximum(0, -dlo - rA), np.maximum(0, -dlo - rB)
            vA = inside & (rA < L1) & (iA >= offA) & (iA < wd)
            vB = inside & (rB < L1) & (iA - 1 >= offB) & (iA - 1 < wd)
            aA = np.where(inside & (rA < L1), s1[np.clip(rA, 0, L1 - 1)], 0)
            aB = np.where(inside & (rB < L1), s1[np.clip(rB, 0, L1 - 1)], 0)
            g = sc * cost[gap, c] + rank_i
            raw = np.minimum(np.minimum(diag + sc * cost[aA, c], HA + g),
                             up + sc * cost[aA, gap] + rank_d)
            ha = np.where(vA, raw & ~3 if choice else raw, INF)
            raw2 = np.minimum(np.minimum(HA + sc * cost[aB, c], HB + g),
                              ha + sc * cost[aB, gap] + rank_d)
            hb = np.where(vB, raw2 & ~3 if choice else raw2, INF)
            if choice:
                e = 1 if u >= 16 else 0
                dm[blk, :, e] = (dm[blk, :, e] * 4 + (raw & 3).astype(np.uint64)) & 0xffffffff
                dm[blk, :, 2 + e] = (dm[blk, :, 2 + e] * 4 + (raw2 & 3).astype(np.uint64)) & 0xffffffff
            fa = vA & (rA == L1 - 1) & (iA == L2 - L1 - dlo)
            fb = vB & (rB == L1 - 1) & (iA - 1 == L2 - L1 - dlo)
            if fa.any():
                result = int(ha[fa][0])
            if fb.any():
                result = int(hb[fb][0])
            Pk = hb
            q[31] = hb[31]
            diag, HA, HB = up, ha, hb
        for L in range(32):  # lane 31's second-row values become the boundary row
            pa = G0 + L - 93
            s31 = pa // W
            x = pa - s31 * W - 1
            if s31 >= 0 and 0 <= x < wd:
                bnd[x] = q[L]
        q = qn
    cost_v = (result - bias) // sc
    if not choice:
        return cost_v, None
    r, j, ra, rb = L1 - 1, L2 - 1, [], []
    while r > 0 or (r == 0 and j >= 0):
        kk, h, t = (r % 64) // 2, r & 1, r // 64
        G = t * W + 3 * kk + (j - r) - dlo + h
        w = int(dm[G // 32, kk, 2 * h + (1 if G % 32 >= 16 else 0)])
        code = (w >> (2 * (15 - G % 16))) & 3
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
    for n1, n2 in [(0, 0), (0, 5), (1, 1), (2, 7), (130, 128), (63, 65), (200, 301),
                   (500, 10), (250, 251), (300, 140)]:
        out.append((g(synth.random_dna(rng, n1, 0.1)), g(synth.random_dna(rng, n2, 0.1))))
    return out


@pytest.mark.parametrize("model", [(1, 2), (3, 1)])
def test_continuous_schedule_matches_oracle(model):
    m = O.cm_dna(model[0], model[1], -1)
    for a, b in _cases():
        c_ref, ra, rb = O.align_2(a, b, m)
        c_choice, (ea, eb) = emulate(a, b, m, choice=True)
        c_cost, _ = emulate(a, b, m, choice=False)
        assert c_choice == c_ref == c_cost == O.cost_2(a, b, m), (len(a), len(b))
        assert np.array_equal(ea, ra) and np.array_equal(eb, rb), (len(a), len(b))
