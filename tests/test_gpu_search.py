"""Config 0 parity: a Wagner build plus one SPR pass on 20 taxa x ~300 bp
(seeded Yule tree, JC 0.05/site/branch, indels 0.01/site) with Fitch and
Sankoff characters, driven once through the CUDA kernels and once through
the CPU oracle: identical trees, tree costs and every per-node median."""
import numpy as np
import pytest

from oracle import oracle as O
from poyd_gb300 import align, search, simulate
from tests.oracle_backend import OracleBackend

pytestmark = pytest.mark.gpu


def _compare_nodes(t, g, o):
    for v in t.nodes():
        assert np.array_equal(g.node_seq(v), o.node_seq(v)), v
        if g.nf:
            assert np.array_equal(g.node_fitch(v), o.node_fitch(v)), v
        if g.ns:
            assert np.array_equal(g.node_sank(v), o.node_sank(v)), v


@pytest.mark.parametrize("seed,n_fitch,n_sank", [(7, 0, 0), (8, 60, 12)])
def test_wagner_and_spr_match_oracle(seed, n_fitch, n_sank):
    data = simulate.simulate(seed, 20, 300, n_fitch, n_sank)
    g = search.GpuBackend(data, align.CostMatrix.default())
    o = OracleBackend(data, O.cm_dna(1, 2, -1))
    tg, dg = search.wagner(data.n_taxa, g)
    to, do = search.wagner(data.n_taxa, o)
    assert tg.newick() == to.newick()
    assert dg.total == do.total and dg.do_cost == do.do_cost
    _compare_nodes(tg, g, o)
    sg = search.spr_pass(tg, g, max_moves=6)
    so = search.spr_pass(to, o, max_moves=6)
    assert tg.newick() == to.newick()
    assert (sg.cost_before, sg.cost_after, sg.moves_accepted) == \
        (so.cost_before, so.cost_after, so.moves_accepted)
    assert sg.cost_after <= sg.cost_before
    _compare_nodes(tg, g, o)
