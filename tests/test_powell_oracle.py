"""The oracle's three-sequence alignment (or_powell_3d: Powell's cost model,
ukkCommon.c:206-391, by dynamic programming) against the reference's own
powell_3D_align (ukkCommon.c:111-143, ukk.checkp.c): the committed golden
costs and alignments (tests/golden/make_powell_golden.py), and the compiled
reference itself where it is built; plus the 3-D median table
(cost_matrix.ml:803-851) and readjust_3d's early returns
(sequence.ml:1117-1140) on hand-worked cases."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from poyd_gb300 import synth

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "powell_golden.npz")
PARAMS = [(1, 0, 2), (1, 2, 1), (2, 3, 1)]


def unpack(data, lens):
    offs = np.concatenate([[0], np.cumsum(lens)])
    return [data[offs[i]:offs[i + 1]] for i in range(len(lens))]


def golden():
    g = np.load(GOLDEN)
    T = list(zip(*(unpack(g[k + "_data"], g[k + "_len"]) for k in "abc")))
    return g, T


def collapse(s):
    """The character powell_3D_align aligns for each element past the
    leading gap (copySequence, ukkCommon.c:84-105)."""
    out = []
    for x in s[1:]:
        for b in (1, 2, 4, 8):
            if x & b:
                out.append(b)
                break
    return np.array(out, np.uint8)


def check_rows(t, rows):
    """The rows are an alignment of the three collapsed inputs with the
    leading gap column first."""
    n = len(rows[0])
    assert all(len(r) == n for r in rows)
    assert all(r[0] == 16 for r in rows)
    for s, r in zip(t, rows):
        assert np.array_equal(r[1:][r[1:] != 16], collapse(s))
    assert not np.any((rows[0][1:] == 16) & (rows[1][1:] == 16) & (rows[2][1:] == 16))


# the CPU suite restates the triples of up to 400k cells (44 of 79); the
# GPU tests compare every golden triple
CPU_CELLS = 400_000


@pytest.mark.parametrize("p", PARAMS)
def test_oracle_cost_equals_reference_golden(p):
    g, T = golden()
    key = "%d_%d_%d" % p
    want = g["cost_" + key]
    rows = [unpack(g["al%s_%s_data" % (q, key)], g["al%s_%s_len" % (q, key)]) for q in "abc"]
    same = 0
    for i, t in enumerate(T):
        if len(t[0]) * len(t[1]) * len(t[2]) > CPU_CELLS:
            continue
        c, ra, rb, rc = O.powell_3d(*t, *p)
        assert c == want[i], (i, [len(x) for x in t], c, want[i])
        check_rows(t, (ra, rb, rc))
        # the reference's own rows cost what it returned, under the model
        ref_rows = (rows[0][i], rows[1][i], rows[2][i])
        check_rows(t, ref_rows)
        assert O.powell_alignment_cost(*ref_rows, *p) == want[i]
        assert O.powell_alignment_cost(ra, rb, rc, *p) == c
        same += all(np.array_equal(x, y) for x, y in zip((ra, rb, rc), ref_rows))
    assert same > 0


def test_oracle_cost_equals_compiled_reference():
    if O.ref() is None:
        pytest.skip("compiled reference not built here")
    T = synth.triple_batch(11, 40, lmin=0, lmax=24, sub=(0.1, 0.5), indel=(0.02, 0.2), ambig=0.1)
    for i, t in enumerate(T):
        p = PARAMS[i % 3]
        assert O.powell_3d(*t, *p)[0] == O.powell_3d(*t, *p, reference=True)[0]


def test_cost_is_symmetric_in_the_three_sequences():
    for t in synth.triple_batch(3, 8, lmin=5, lmax=40):
        c = {O.powell_3d(*(t[k] for k in perm), 1, 2, 1)[0]
             for perm in [(0, 1, 2), (1, 0, 2), (2, 1, 0), (1, 2, 0)]}
        assert len(c) == 1


def test_median3_table_hand_cases():
    m = O.cm_dna(1, 2, -1)  # sub 1, indel 2, metric
    tab = O.median3_table(m)
    A, C, G, T, GAP = 1, 2, 4, 8, 16

    def med(i, j, k):
        return int(tab[(i << 10) | (j << 5) | k])

    assert med(A, A, C) == A
    assert med(C, G, G) == G
    assert med(A, C, G) == A            # three-way tie: the lowest bit
    assert med(T, G, C) == C
    assert med(A, GAP, GAP) == GAP      # 2 for the gap against 4 for A
    assert med(A, C, GAP) == A          # gap: 2+2+0 = 4 > A: 0+1+2 = 3
    assert med(GAP, GAP, GAP) == GAP
    assert med(A | C, C, G) == C        # C costs 0+0+1 against A's 0+1+1


def test_readjust_3d_early_returns():
    m = O.cm_dna(1, 2, -1)
    a = np.array([16, 1, 2, 4], np.uint8)
    b = np.array([16, 1, 4], np.uint8)
    p = np.array([16, 2, 4, 8, 8], np.uint8)
    e = np.array([16], np.uint8)
    # equal lengths keep m
    cur = np.array([16, 8, 8, 8], np.uint8)
    c, r, ch = O.readjust_3d(a, a, cur, np.array([16, 1, 1, 1], np.uint8), m)
    assert (c, list(r), ch) == (0, list(cur), False)
    # an empty child gives the other one
    c, r, ch = O.readjust_3d(e, b, cur, p, m)
    assert (c, list(r), ch) == (0, list(b), True)
    c, r, ch = O.readjust_3d(a, e, a, p, m)
    assert (c, list(r), ch) == (0, list(a), False)
    # both children empty and the parent empty: the parent
    c, r, ch = O.readjust_3d(e, e, cur, e, m)
    assert (c, list(r), ch) == (0, [16], True)
    # otherwise the median of the three-way alignment
    c, r, ch = O.readjust_3d(a, b, cur, p, m)
    assert c == O.powell_3d(a, b, p, 1, 0, 2)[0]
    assert r[0] == 16 and ch


def test_readjust_3d_fails_like_the_reference_on_gap_elements():
    m = O.cm_dna(1, 2, -1)
    bad = np.array([16, 1, 16, 2], np.uint8)
    with pytest.raises(ValueError):
        O.readjust_3d(bad, np.array([16, 1], np.uint8), np.array([16], np.uint8),
                      np.array([16, 4, 4], np.uint8), m)
