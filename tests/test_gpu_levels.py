"""The level engine (poyd_median_levels): a whole downpass in one call gives
the oracle's medians, costs and Fitch / Sankoff rows at every node, the
same as one call per level, and survives a pool too small for its bound
(POYD_ESPACE, compaction, second call)."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from poyd_gb300 import align, learned, search, simulate
from tests.oracle_backend import OracleBackend

pytestmark = pytest.mark.gpu


def _levels(t):
    mc = t.min_codes()
    out = []
    for level in t.levels():
        lv = np.array(level, np.int64)
        a, b = search._by_code(t.kids[lv, 0], t.kids[lv, 1], mc)
        out.append((a, b, lv))
    return out


def _same_nodes(g, o, nodes):
    for v in nodes:
        assert np.array_equal(g.node_seq(v), o.node_seq(v)), v
        if g.nf:
            assert np.array_equal(g.node_fitch(v), o.node_fitch(v)), v
        if g.ns:
            s = g.node_sank(v).astype(np.int64)
            s[s >= (1 << 30)] = O.SANK_INF
            assert np.array_equal(s, np.asarray(o.node_sank(v), np.int64)), v


@pytest.mark.parametrize("seed", [5, 23])
def test_one_call_downpass_matches_oracle_and_per_level_calls(seed):
    data = simulate.simulate(seed, 40, 300, n_fitch=50, n_sank=8)
    t = learned.random_tree(data.n_taxa, seed + 1)
    lv = _levels(t)
    g1 = search.GpuBackend(data, align.CostMatrix.default())
    r1 = g1.median_levels(lv)
    g2 = search.GpuBackend(data, align.CostMatrix.default())
    r2 = [g2.medians(a, b, out) for a, b, out in lv]
    o = OracleBackend(data, O.cm_dna(1, 2, -1))
    r3 = o.median_levels(lv)
    for x, y, z in zip(r1, r2, r3):
        for k in range(2):
            assert np.array_equal(x[k], y[k]) and np.array_equal(x[k], np.asarray(z[k], np.int64))
    internal = [v for v in t.nodes() if v >= t.n]
    _same_nodes(g1, o, internal)
    _same_nodes(g2, o, internal)


def test_pool_too_small_compacts_and_retries():
    data = simulate.simulate(8, 30, 400, n_fitch=20, n_sank=4)
    t = learned.random_tree(data.n_taxa, 9)
    g = search.GpuBackend(data, align.CostMatrix.default())
    # shrink the pool to the leaves' bytes plus a little: the first call
    # must be refused and then succeed after compaction
    live = int(g.len.sum())
    g._compact()
    g.pool = g.pool[:live + 4096].clone()
    assert g.top == live
    lv = _levels(t)
    res = g.median_levels(lv)
    assert g.pool.numel() > live + 4096
    o = OracleBackend(data, O.cm_dna(1, 2, -1))
    for x, z in zip(res, o.median_levels(lv)):
        assert np.array_equal(x[0], np.asarray(z[0], np.int64))
    _same_nodes(g, o, [v for v in t.nodes() if v >= t.n])
    torch.cuda.synchronize()
