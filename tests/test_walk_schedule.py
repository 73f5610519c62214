"""The warp-parallel traceback of the packed DP kernel (tb_pair4_solo in
csrc/linear4.cu: lanes read a diagonal run of moves, a ballot finds its
end, each lane writes its own column) against the serial walk it replaces
(tb_pair4: backtrack_2d, algn.c:3551-3666, with ancestor_2's median,
algn.c:4126-4147), emulated on the CPU over random move grids, both
argument orders and both tie priorities, with output slots large enough
and too small (the walk must then fail the same way)."""
import numpy as np
import pytest

GAP = 16


def serial(code, s1, s2, med, swaped, swap, cap):
    l1, l2 = code.shape
    r, j, n = l1 - 1, l2 - 1, 0
    oa, ob, ow, om = [bytearray(cap) for _ in range(4)]
    nm = 0
    bad = False
    while r > 0 or (r == 0 and j >= 0):
        if j < 0 or n + 2 >= cap:
            bad = True; break
        c = code[r, j]
        move = 0 if c == 0 else (1 if (c == 1) == swaped else 2)
        dr, dj = move != 1, move != 2
        cr = s1[r] if dr else GAP
        cc = s2[j] if dj else GAP
        r -= dr; j -= dj
        ca, cb = (cc, cr) if swap else (cr, cc)
        md = med[ca][cb]
        oa[cap - 1 - n] = ca; ob[cap - 1 - n] = cb; ow[cap - 1 - n] = md
        if md != GAP:
            om[cap - 1 - nm] = md; nm += 1
        n += 1
    if not bad:
        om[cap - 1 - nm] = GAP
    return bad, n, nm + 1, bytes(oa), bytes(ob), bytes(ow), bytes(om)


def parallel(code, s1, s2, med, swaped, swap, cap):
    l1, l2 = code.shape
    r, j, n, nm = l1 - 1, l2 - 1, 0, 0
    oa, ob, ow, om = [bytearray(cap) for _ in range(4)]
    bad = False
    while r > 0 or (r == 0 and j >= 0):
        if j < 0 or n + 2 >= cap:
            bad = True; break
        codes = []
        for lane in range(32):
            ri, ji = r - lane, j - lane
            codes.append(int(code[ri, ji]) if (ri >= 0 and ji >= 0 and n + lane + 2 < cap) else 4)
        stop = [c != 0 for c in codes]
        f = stop.index(True) if any(stop) else 32
        cf = codes[f & 31]
        step_f = f < 32 and cf != 4
        move_f = (1 if (cf == 1) == swaped else 2) if step_f else 0
        keeps = []
        mds = []
        for lane in range(32):
            writes = lane < f or (lane == f and step_f)
            md = GAP
            if writes:
                dr = lane < f or move_f != 1
                dj = lane < f or move_f != 2
                ri, ji = r - lane, j - lane
                cr = s1[ri] if dr else GAP
                cc = s2[ji] if dj else GAP
                ca, cb = (cc, cr) if swap else (cr, cc)
                md = med[ca][cb]
                pos = cap - 1 - (n + lane)
                oa[pos] = ca; ob[pos] = cb; ow[pos] = md
            keeps.append(writes and md != GAP); mds.append(md)
        rank = 0
        for lane in range(32):
            if keeps[lane]:
                om[cap - 1 - (nm + rank)] = mds[lane]; rank += 1
        n += f + (1 if step_f else 0)
        nm += rank
        r -= f + (1 if (step_f and move_f != 1) else 0)
        j -= f + (1 if (step_f and move_f != 2) else 0)
    if not bad:
        om[cap - 1 - nm] = GAP
    return bad, n, nm + 1, bytes(oa), bytes(ob), bytes(ow), bytes(om)


@pytest.mark.parametrize("seed", [1, 2])
def test_parallel_walk_equals_serial_walk(seed):
    rng = np.random.default_rng(seed)
    for t in range(1500):
        l1, l2 = rng.integers(1, 90, size=2)
        p = rng.choice([0.0, 0.05, 0.3, 0.8])
        code = np.where(rng.random((l1, l2)) < p, rng.integers(1, 4, size=(l1, l2)), 0)
        s1 = rng.integers(1, 32, size=l1); s2 = rng.integers(1, 32, size=l2)
        s1[0] = s2[0] = GAP
        med = rng.integers(1, 33, size=(33, 33)); med[med == 32] = GAP
        swaped, swap = bool(rng.integers(2)), bool(rng.integers(2))
        cap = int(rng.choice([l1 + l2 + 2, max(3, (l1 + l2) // 2)]))
        a = serial(code, s1, s2, med, swaped, swap, cap)
        b = parallel(code, s1, s2, med, swaped, swap, cap)
        assert a == b, (t, l1, l2, p, a[:3], b[:3])
