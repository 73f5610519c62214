"""The CUDA linear path reproduces the golden vectors made by the
reference's own compiled algn.c (tests/golden/make_golden.py)."""
import numpy as np
import pytest

from poyd_gb300 import align
from tests import golden_io as G

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("model", G.LINEAR)
def test_linear_golden_vectors(model):
    g = G.load()
    tag = "lin_%d_%d" % model
    cm = align.CostMatrix.dna(*model)
    batch = align.PairBatch.from_host(g["A"], g["B"])
    cost, _ = align.cost_2(batch, cm)
    assert np.array_equal(cost.cpu().numpy(), g[tag + "_cost"])
    cost_dos, _ = align.cost_2(batch, cm, deltaw="dos")
    assert np.array_equal(cost_dos.cpu().numpy(), g[tag + "_cost_dos"])
    res = align.align_2(batch, cm).to_host()
    al_a, al_b = G.seqs(g, tag + "_al_a"), G.seqs(g, tag + "_al_b")
    anc, mwg = G.seqs(g, tag + "_anc"), G.seqs(g, tag + "_mwg")
    for i, r in enumerate(res):
        assert r["cost"] == g[tag + "_cost"][i]
        assert np.array_equal(r["a"], al_a[i]) and np.array_equal(r["b"], al_b[i]), i
        assert np.array_equal(r["median"], anc[i]) and np.array_equal(r["median_wg"], mwg[i]), i
