"""The Iterative modes' tree adjustment (search.adjust_tree,
allDirChar.ml:488-668) on the CPU oracle backend: the level-batched
schedule gives exactly the one-vertex-at-a-time results, the accepted cost
never exceeds the diagnosis's, and the traversal visits every interior
vertex with its three neighbours."""
import numpy as np
import pytest

from oracle import oracle as O
from poyd_gb300 import learned, search, simulate
from tests.oracle_backend import OracleBackend


def test_order_and_levels_cover_the_tree():
    t = learned.random_tree(9, 3)
    adj = search.unrooted_adjacency(t)
    order, nbrs = search.adjust_order(t, adj)
    assert sorted(order) == sorted(v for v in adj if v >= t.n)
    for v in order:
        assert sorted(nbrs[v]) == sorted(adj[v])
    pos = {v: i for i, v in enumerate(order)}
    lv = search.adjust_levels(order, adj)
    where = {v: i for i, g in enumerate(lv) for v in g}
    for v in order:
        for u in adj[v]:
            if u in pos and pos[u] < pos[v]:
                assert where[u] < where[v]


@pytest.mark.parametrize("mode", ["three", "approx"])
def test_batched_schedule_equals_sequential(mode):
    data = simulate.simulate(5, 9, 40, 0, 0, sub_per_branch=0.15, indel_rate=0.03)
    t = learned.random_tree(data.n_taxa, 11)
    res = []
    for batched in (True, False):
        be = OracleBackend(data, O.cm_dna(1, 2, -1))
        res.append(search.adjust_tree(t, be, mode, batched=batched))
    a, b = res
    assert (a.cost, a.initial_cost, a.passes, a.changes) == (b.cost, b.initial_cost, b.passes, b.changes)
    assert a.cost <= a.initial_cost
    assert a.calls <= b.calls
    for v in a.seqs:
        assert np.array_equal(a.seqs[v], b.seqs[v])
