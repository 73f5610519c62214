"""Node readjustment of the Iterative cost modes, batched on the GPU.

``DOS.readjust`` (seqCS.ml:680-722) re-estimates one node's DO sequence
from its three neighbours: with ``ThreeD`` through
``Sequence.Align.readjust_3d`` (the three-sequence kernel, ``three.py``),
with ``ApproxD`` through ``Sequence.readjust`` (sequence.ml:1166-1195),
built from pairwise alignments, ``median_2`` and ``Align.closest``; nodes
with empty neighbours take the rules of seqCS.ml:699-719.  Every stage of
every node of a batch is one batched call of the library."""
from __future__ import annotations

import numpy as np

from . import align, three
from .align import CostMatrix, PairBatch

GAP = 16


def _empty(s) -> bool:
    return bool(np.all(np.asarray(s) == GAP))


def select_one(s: np.ndarray, cm: CostMatrix) -> np.ndarray:
    """``Sequence.select_one`` (sequence.ml:1143-1156): every element
    becomes its lowest state (combination alphabets)."""
    s = np.asarray(s, np.uint8)
    if np.any(s == 0):
        raise ValueError("select_one: an element with no states")
    return (s & ((-s.astype(np.int16)) & 0xFF).astype(np.uint8)).astype(np.uint8)


def algn_medians(pairs, cm: CostMatrix):
    """The ``algn`` of Sequence.readjust / DOS.readjust before select_one,
    for a list of (s1, s2): (costs, medians).  Linear: align_2, then
    ``median_2`` (algn_CAML_median_2_no_gaps) of the aligned pair; affine:
    align_affine_3's median."""
    if not pairs:
        return [], []
    res = align.align_2(PairBatch.from_host([p[0] for p in pairs], [p[1] for p in pairs]),
                        cm).to_host()
    costs = [r["cost"] for r in res]
    if cm.affine:
        return costs, [r["median"] for r in res]
    return costs, align.columns("median_2_no_gaps", [r["a"] for r in res],
                                [r["b"] for r in res], cm)


def closest_many(pairs, cm: CostMatrix):
    """``Align.closest s1 s2`` (sequence.ml:967-1033) for (s1, s2) pairs:
    s2's single sequence against s1."""
    if not pairs:
        return []
    b = PairBatch.from_host([p[0] for p in pairs], [p[1] for p in pairs])
    return [r["median"] for r in align.closest(b, cm, dos_empty=False).to_host()]


def seq_readjust(triples, cm: CostMatrix):
    """``Sequence.readjust a b m cm parent`` (ApproxD) for (a, b, parent)
    triples: (costs, sequences).  Three batched stages: the pairwise
    medians ab, bc, ac; each aligned with the third sequence; the cheapest
    centre's median made closest to the third."""
    n = len(triples)
    if n == 0:
        return [], []
    st1 = []
    for a, b, c in triples:
        st1 += [(a, b), (b, c), (a, c)]
    c1, m1 = algn_medians(st1, cm)
    st2 = []
    for i, (a, b, c) in enumerate(triples):
        ab, bc, ac = m1[3 * i], m1[3 * i + 1], m1[3 * i + 2]
        st2 += [(ab, c), (bc, a), (ac, b)]
    c2, _ = algn_medians(st2, cm)
    pick, costs = [], []
    for i, (a, b, c) in enumerate(triples):
        ab, bc, ac = m1[3 * i], m1[3 * i + 1], m1[3 * i + 2]
        cabc = c2[3 * i] + c1[3 * i]
        cbca = c2[3 * i + 1] + c1[3 * i + 1]
        cacb = c2[3 * i + 2] + c1[3 * i + 2]
        if cabc <= cbca:
            choice = (cabc, (c, ab)) if cabc <= cacb else (cacb, (b, ac))
        elif cbca < cacb:
            choice = (cbca, (a, bc))
        else:
            choice = (cacb, (b, ac))
        costs.append(choice[0])
        pick.append(choice[1])
    return costs, closest_many(pick, cm)


def dos_readjust(items, cm: CostMatrix, mode: str = "three"):
    """Batched ``DOS.readjust`` for items (ch1, ch2, parent, mine) of uint8
    sequences with their leading gap; mode "three" (Iterative ThreeD) or
    "approx" (ApproxD).  Returns (changed, new sequence, cost) per item;
    changed is ``0 <> compare res mine`` (seqCS.ml:721)."""
    if mode not in ("three", "approx"):
        raise ValueError("mode is 'three' or 'approx'")
    out = [None] * len(items)
    full, one = [], []
    for i, (c1, c2, p, mine) in enumerate(items):
        e1, e2, ep = _empty(c1), _empty(c2), _empty(p)
        if not (e1 or e2 or ep):
            full.append(i)
        elif e1 and (e2 or ep):
            out[i] = (np.asarray(c1, np.uint8).copy(), 0)
        elif e2 and ep:
            out[i] = (np.asarray(c2, np.uint8).copy(), 0)
        else:
            one.append((i, (c1, c2) if ep else (c1, p) if e2 else (c2, p)))
    if full:
        if mode == "three":
            r = three.readjust_3d(three.TripleBatch.from_host(
                [(items[i][0], items[i][1], items[i][3], items[i][2]) for i in full]), cm).to_host()
            for i, x in zip(full, r):
                out[i] = (x["median"], x["cost"])
        else:
            cs, ss = seq_readjust([(items[i][0], items[i][1], items[i][2]) for i in full], cm)
            for i, c, s in zip(full, cs, ss):
                out[i] = (s, c)
    if one:
        cs, ms = algn_medians([pr for _, pr in one], cm)
        for (i, _), c, med in zip(one, cs, ms):
            out[i] = (select_one(med, cm), c)
    res = []
    for (c1, c2, p, mine), (s, c) in zip(items, out):
        mine = np.asarray(mine, np.uint8)
        res.append((not (len(s) == len(mine) and np.array_equal(s, mine)), s, int(c)))
    return res
