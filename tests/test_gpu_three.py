"""The CUDA three-sequence alignment (csrc/three.cu) against the reference's
golden powell_3D_align costs (tests/golden/powell_golden.npz) and against the
oracle (or_powell_3d, or_readjust_3d) bit for bit: cost, the three aligned
rows, the median of align_3_powell_inter (sequence.ml:1089-1115) and
readjust_3d's early returns and changed flags (sequence.ml:1117-1140)."""
import os

import numpy as np
import pytest
import torch

from oracle import oracle as O
from poyd_gb300 import align, native, synth, three

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "powell_golden.npz")
PARAMS = [(1, 0, 2), (1, 2, 1), (2, 3, 1)]


def unpack(data, lens):
    offs = np.concatenate([[0], np.cumsum(lens)])
    return [data[offs[i]:offs[i + 1]] for i in range(len(lens))]


@pytest.mark.parametrize("p", PARAMS)
def test_golden_costs_and_oracle_rows(p):
    g = np.load(GOLDEN)
    T = list(zip(*(unpack(g[k + "_data"], g[k + "_len"]) for k in "abc")))
    key = "%d_%d_%d" % p
    res = three.align_3_powell(three.TripleBatch.from_host(T), *p).to_host()
    want = g["cost_" + key]
    assert [r["cost"] for r in res] == want.tolist()
    for i, t in enumerate(T):
        if len(t[0]) * len(t[1]) * len(t[2]) > 1_000_000:
            assert O.powell_alignment_cost(res[i]["a"], res[i]["b"], res[i]["c"], *p) == want[i]
            continue
        c, ra, rb, rc = O.powell_3d(*t, *p)
        assert c == res[i]["cost"]
        for x, y in zip((ra, rb, rc), (res[i]["a"], res[i]["b"], res[i]["c"])):
            assert np.array_equal(x, y), i


def test_median_and_readjust_match_oracle():
    rng = np.random.default_rng(9)
    items = []
    T = synth.triple_batch(21, 40, lmin=0, lmax=70)
    for i, (s1, s2, p) in enumerate(T):
        cur = synth.with_gap(synth.random_dna(rng, int(rng.integers(0, 60))))
        items.append((s1, s2, cur, p))
    e = np.array([16], np.uint8)
    a, b, p = T[0]
    items += [
        (a, a.copy(), a.copy(), a.copy()),               # equal lengths keep m
        (e, b, a, p), (a, e, a, p), (e, e, a, e),        # empty children / parent
        (e, e, a, p),                                    # both children empty: align
        (a, b, e, p), (a, b, p.copy(), p),
    ]
    for sub, indel, go in [(1, 2, -1), (1, 1, 2), (2, 1, 3)]:
        cm = align.CostMatrix.dna(sub, indel, None if go < 0 else go)
        m = O.cm_dna(sub, indel, go)
        tab = O.median3_table(m)
        assert np.array_equal(three.median3_table(cm), tab)
        res = three.readjust_3d(three.TripleBatch.from_host(items), cm).to_host()
        for i, it in enumerate(items):
            c, med, ch = O.readjust_3d(*it, m, tab)
            assert (res[i]["cost"], res[i]["changed"]) == (c, ch), (i, sub, indel, go)
            assert np.array_equal(res[i]["median"], med), (i, sub, indel, go)


def test_single_call_matches_oracle():
    for t in synth.triple_batch(5, 6, lmin=1, lmax=50):
        ra, rb, rc, c = three.powell_3D_align(*t, 1, 2, 1)
        c2, *rows = O.powell_3d(*t, 1, 2, 1)
        assert c == c2
        for x, y in zip((ra, rb, rc), rows):
            assert np.array_equal(x, y)


def test_element_without_base_fails_loudly():
    bad = (np.array([16, 1, 16, 2], np.uint8), np.array([16, 1], np.uint8),
           np.array([16, 4, 4], np.uint8))
    good = synth.triple_batch(1, 1, lmin=3, lmax=5)[0]
    with pytest.raises(native.PoydError) as ei:
        r = three.align_3_powell(three.TripleBatch.from_host([good, bad]), 1, 0, 2)
    assert ei.value.code == -1


def test_long_triples_properties():
    # 300-400 bp: the oracle is too slow at this size; the rows must be an
    # alignment of the inputs whose model cost is the returned optimum, the
    # optimum must not depend on the order of the three sequences, and a
    # triple of one sequence three times costs nothing.
    T = synth.triple_batch(31, 6, lmin=300, lmax=400)
    res = three.align_3_powell(three.TripleBatch.from_host(T), 1, 2, 1).to_host()
    rot = three.align_3_powell(three.TripleBatch.from_host([(t[2], t[0], t[1]) for t in T]),
                               1, 2, 1).to_host()
    for t, r, q in zip(T, res, rot):
        assert r["cost"] == q["cost"]
        assert O.powell_alignment_cost(r["a"], r["b"], r["c"], 1, 2, 1) == r["cost"]
        for s, row in zip(t, (r["a"], r["b"], r["c"])):
            col = row[1:][row[1:] != 16]
            assert len(col) == len(s) - 1
    same = three.align_3_powell(three.TripleBatch.from_host([(T[0][0],) * 3]), 1, 2, 1).to_host()
    assert same[0]["cost"] == 0


def test_packed_and_32_bit_kernels_agree(monkeypatch):
    # the 16-bit kernel (default) and the 32-bit one give the same rows
    T = synth.triple_batch(12, 24, lmin=0, lmax=90)
    b = three.TripleBatch.from_host(T)
    packed = three.align_3_powell(b, 1, 2, 1).to_host()
    monkeypatch.setenv("POYD_P3_PACKED", "0")
    wide = three.align_3_powell(b, 1, 2, 1).to_host()
    for x, y in zip(packed, wide):
        assert x["cost"] == y["cost"]
        for k in "abc":
            assert np.array_equal(x[k], y[k])


def test_optimum_above_the_16_bit_range_is_redone_in_32_bits():
    # mm = ge = 100: the optima exceed 3,072, the 16-bit kernel's range
    T = synth.triple_batch(8, 5, lmin=30, lmax=40, sub=(0.3, 0.5), indel=(0.05, 0.1))
    T.append(synth.triple_batch(9, 1, lmin=3, lmax=5)[0])
    res = three.align_3_powell(three.TripleBatch.from_host(T), 100, 0, 100).to_host()
    assert max(r["cost"] for r in res) > 3072
    for t, r in zip(T, res):
        c, *rows = O.powell_3d(*t, 100, 0, 100)
        assert c == r["cost"]
        for x, k in zip(rows, "abc"):
            assert np.array_equal(x, r[k])


def test_workspace_release_then_reuse():
    T = synth.triple_batch(14, 4, lmin=10, lmax=40)
    b = three.TripleBatch.from_host(T)
    first = three.align_3_powell(b, 1, 2, 1).to_host()
    native.check(native.lib().poyd_workspace_release())
    again = three.align_3_powell(b, 1, 2, 1).to_host()
    assert [r["cost"] for r in first] == [r["cost"] for r in again]
    assert all(np.array_equal(x["a"], y["a"]) for x, y in zip(first, again))


def test_cluster_and_single_block_kernels_agree(monkeypatch):
    # a small batch runs a thread-block cluster per triple; the one-block
    # kernel (large batches) must give the same rows
    for go in (0, 2):
        T = synth.triple_batch(13 + go, 6, lmin=60, lmax=140)
        b = three.TripleBatch.from_host(T)
        monkeypatch.delenv("POYD_P3_CLUSTER", raising=False)
        cl = three.align_3_powell(b, 1, go, 1).to_host()
        monkeypatch.setenv("POYD_P3_CLUSTER", "0")
        one = three.align_3_powell(b, 1, go, 1).to_host()
        for t, x, y in zip(T, cl, one):
            assert x["cost"] == y["cost"]
            for k in "abc":
                assert np.array_equal(x[k], y[k])
        c, *rows = O.powell_3d(*T[0], 1, go, 1)
        assert c == cl[0]["cost"] and all(np.array_equal(r, cl[0][k]) for r, k in zip(rows, "abc"))
