"""The Iterative modes' tree adjustment (search.adjust_tree over batched
DOS.readjust on the GPU) against the same driver over the CPU oracle:
identical accepted costs, passes, changes and adjusted sequences."""
import numpy as np
import pytest

from oracle import oracle as O
from poyd_gb300 import align, learned, search, simulate
from tests.oracle_backend import OracleBackend

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", ["three", "approx"])
@pytest.mark.parametrize("model", [(1, 2, -1), (1, 2, 3)])
def test_adjust_tree_matches_oracle(mode, model):
    sub, indel, go = model
    for seed in (5, 7):
        data = simulate.simulate(seed, 14, 80, 0, 0, sub_per_branch=0.15, indel_rate=0.03)
        t = learned.random_tree(data.n_taxa, 11 + seed)
        g = search.GpuBackend(data, align.CostMatrix.dna(sub, indel, None if go < 0 else go))
        o = OracleBackend(data, O.cm_dna(sub, indel, go))
        rg = search.adjust_tree(t, g, mode)
        ro = search.adjust_tree(t, o, mode)
        assert (rg.cost, rg.initial_cost, rg.passes, rg.changes) == \
            (ro.cost, ro.initial_cost, ro.passes, ro.changes), (seed, mode, model)
        assert rg.cost <= rg.initial_cost
        for v in ro.seqs:
            assert np.array_equal(rg.seqs[v], ro.seqs[v]), (seed, v)
