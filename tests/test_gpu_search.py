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


@pytest.mark.parametrize("seed,n_fitch,n_sank,sub,indel,go", [(11, 0, 0, 1, 2, -1),
                                                              (12, 40, 8, 1, 2, -1),
                                                              (13, 0, 0, 1, 1, -1),
                                                              (14, 0, 0, 2, 1, 1)])
def test_root_costs_match_oracle(seed, n_fitch, n_sank, sub, indel, go):
    """All-rootings diagnosis (every directed subtree median, then every
    edge's root median) through the CUDA kernels equals the oracle's, for
    linear matrices and an affine one (gap opening 1)."""
    data = simulate.simulate(seed, 24, 400, n_fitch, n_sank)
    g = search.GpuBackend(data, align.CostMatrix.dna(sub, indel, go if go >= 0 else None))
    o = OracleBackend(data, O.cm_dna(sub, indel, go))
    t, diag = search.wagner(data.n_taxa, o)
    rg = search.root_costs(t, g)
    ro = search.root_costs(t, o)
    assert np.array_equal(rg.edges, ro.edges)
    assert np.array_equal(rg.costs, ro.costs)
    assert rg.best() == ro.best() and rg.best()[0] <= diag.total


@pytest.mark.parametrize("sub,indel,go", [(1, 2, -1), (2, 1, 1), (3, 1, 5)])
def test_final_cost_matches_oracle(sub, indel, go):
    """Best rooting, single-state assignment and the edge-distance sum
    through the CUDA kernels equal the oracle's, with two DO character
    sets sharing one root."""
    sets = [simulate.simulate(s, 20, 300) for s in (21, 22)]
    cm = align.CostMatrix.dna(sub, indel, go if go >= 0 else None)
    om = O.cm_dna(sub, indel, go)
    t, _ = search.wagner(sets[0].n_taxa, OracleBackend(sets[0], om))
    fg = search.final_cost(t, [search.GpuBackend(d, cm) for d in sets])
    fo = search.final_cost(t, [OracleBackend(d, om) for d in sets])
    assert (fg.cost, fg.root_edge, fg.root_cost) == (fo.cost, fo.root_edge, fo.root_cost)


@pytest.mark.parametrize("seed,n_fitch,n_sank", [(31, 0, 0), (32, 40, 6)])
def test_tbr_pass_matches_oracle(seed, n_fitch, n_sank):
    """A TBR pass (every clade re-rooting scored in one batch, exact
    evaluation of the best moves) through the CUDA kernels and through the
    oracle: identical candidates, scores, trees, costs and node medians."""
    data = simulate.simulate(seed, 18, 250, n_fitch, n_sank)
    g = search.GpuBackend(data, align.CostMatrix.default())
    o = OracleBackend(data, O.cm_dna(1, 2, -1))
    tg, dg = search.wagner(data.n_taxa, g)
    to, do = search.wagner(data.n_taxa, o)
    assert tg.newick() == to.newick()
    cg = search.tbr_candidates(tg, g)
    co = search.tbr_candidates(to, o)
    for x, y in zip(cg, co):
        assert np.array_equal(np.asarray(x), np.asarray(y))
    sg = search.tbr_pass(tg, g, max_moves=6, diag=dg)
    so = search.tbr_pass(to, o, max_moves=6, diag=do)
    assert tg.newick() == to.newick()
    assert (sg.cost_before, sg.cost_after, sg.moves_accepted) == \
        (so.cost_before, so.cost_after, so.moves_accepted)
    assert sg.cost_after <= sg.cost_before
    _compare_nodes(tg, g, o)


def test_search_with_an_empty_leaf_matches_oracle():
    """An all-gap leaf sequence (an empty '#' fragment): the DOS.median and
    join-cost empty rules through the CUDA kernels equal the oracle's."""
    data = simulate.simulate(41, 16, 200, 20, 3)
    data.seqs[5] = np.array([16], np.uint8)
    g = search.GpuBackend(data, align.CostMatrix.default())
    o = OracleBackend(data, O.cm_dna(1, 2, -1))
    tg, dg = search.wagner(data.n_taxa, g)
    to, do = search.wagner(data.n_taxa, o)
    assert tg.newick() == to.newick() and dg.total == do.total
    sg = search.spr_pass(tg, g, max_moves=6, diag=dg)
    so = search.spr_pass(to, o, max_moves=6, diag=do)
    assert tg.newick() == to.newick() and sg.cost_after == so.cost_after
    _compare_nodes(tg, g, o)
    assert search.final_cost(tg, g).cost == search.final_cost(to, o).cost
