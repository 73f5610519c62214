"""The oracle restatement reproduces the golden vectors the reference's own
compiled C kernels produced (tests/golden/make_golden.py)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import golden_io as G


@pytest.fixture(scope="module")
def golden():
    return G.load()


@pytest.mark.parametrize("model", G.LINEAR)
def test_linear_golden(golden, model):
    m = O.cm_dna(model[0], model[1], -1)
    tag = "lin_%d_%d" % model
    al_a, al_b = G.seqs(golden, tag + "_al_a"), G.seqs(golden, tag + "_al_b")
    anc, mwg = G.seqs(golden, tag + "_anc"), G.seqs(golden, tag + "_mwg")
    for i, (a, b) in enumerate(zip(golden["A"], golden["B"])):
        assert O.cost_2(a, b, m) == golden[tag + "_cost"][i]
        assert O.cost_2(a, b, m, max(abs(len(a) - len(b)), 8)) == golden[tag + "_cost_dos"][i]
        c, ra, rb = O.align_2(a, b, m)
        assert c == golden[tag + "_cost"][i]
        assert np.array_equal(ra, al_a[i]) and np.array_equal(rb, al_b[i]), i
        assert np.array_equal(O.ancestor_2(ra, rb, m), anc[i]), i
        assert np.array_equal(O.median_2_with_gaps(ra, rb, m), mwg[i]), i


@pytest.mark.parametrize("model", G.AFFINE)
def test_affine_golden(golden, model):
    m = O.cm_dna(*model)
    tag = "aff_%d_%d_%d" % model
    med, mwg = G.seqs(golden, tag + "_median"), G.seqs(golden, tag + "_mwg")
    ri, rj = G.seqs(golden, tag + "_resi"), G.seqs(golden, tag + "_resj")
    for i, (a, b) in enumerate(zip(golden["A"], golden["B"])):
        assert O.cost_affine_3(a, b, m) == golden[tag + "_cost"][i], i
        c, m1, w1, i1, j1 = O.align_affine_3(a, b, m)
        assert c == golden[tag + "_cost_bt"][i], i
        assert np.array_equal(m1, med[i]) and np.array_equal(w1, mwg[i]), i
        assert np.array_equal(i1, ri[i]) and np.array_equal(j1, rj[i]), i


def test_fitch_golden(golden):
    nodes = golden["fitch_nodes"]
    c, med = O.nonadd_median(nodes[0], nodes[1])
    assert c == golden["fitch_cost01"][0]
    assert np.array_equal(med, golden["fitch_median01"])
    for i in range(6):
        for j in range(6):
            assert O.nonadd_distance(nodes[i], nodes[j]) == golden["fitch_dist"][i, j]
    F = O.nonadd_median_3(nodes[2], nodes[3], nodes[4], nodes[5])
    assert np.array_equal(F, golden["fitch_median3"])


def test_default_matrix_tables():
    """Cost_matrix.Two_D.default: sub 1 / indel 2 over A,C,G,T,gap."""
    t = O.cm_tables(O.cm_dna(1, 2, -1))
    cost = t["cost"].reshape(32, 32)
    assert cost[1, 2] == 1 and cost[1, 16] == 2 and cost[16, 16] == 0
    assert cost[3, 1] == 0            # {A,C} vs A share A
    assert cost[3, 12] == 1           # {A,C} vs {G,T}: one substitution
    assert t["median"].reshape(32, 32)[1, 2] == 3
    assert t["tail"][1] == 2 and t["prepend"][4] == 2
