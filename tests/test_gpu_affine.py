"""Parity of the CUDA affine-gap path (cost_affine_3 / align_affine_3) with
the oracle and the reference's golden vectors (bit-exact)."""
import numpy as np
import pytest

from oracle import oracle as O
from poyd_gb300 import align, synth
from tests import golden_io as G

pytestmark = pytest.mark.gpu

MODELS = [(1, 2, 3), (2, 1, 1), (3, 1, 5), (1, 1, 0)]


def _pairs(seed, n, lmax):
    A, B = synth.pair_batch(seed, n, lmin=1, lmax=lmax)
    rng = np.random.default_rng(seed)
    g = synth.with_gap
    for n1, n2 in [(0, 0), (0, 9), (4, 0), (1, 1), (45, 200), (200, 45), (41, 40), (39, 41),
                   (80, 81), (300, 120), (120, 300), (64, 1)]:
        A.append(g(synth.random_dna(rng, n1, 0.1)))
        B.append(g(synth.random_dna(rng, n2, 0.1)))
    a = synth.random_dna(rng, 260)
    b = a.copy()
    b[::5] = 16
    b[30:90] = 16
    A.append(g(a))
    B.append(g(b))
    # indel runs wider than the 40-column band edge
    a = synth.random_dna(rng, 400)
    b = np.concatenate([a[:100], a[170:]])
    A.append(g(a))
    B.append(g(b))
    return A, B


@pytest.mark.parametrize("model", MODELS)
def test_affine_cost_matches_oracle(model):
    A, B = _pairs(31 + model[2], 50, 900)
    cm = align.CostMatrix.dna(*model)
    om = O.cm_dna(*model)
    cost, cells = align.cost_2(align.PairBatch.from_host(A, B), cm, band_cells=True)
    cost = cost.cpu().numpy()
    cells = cells.cpu().numpy()
    for i, (a, b) in enumerate(zip(A, B)):
        assert cost[i] == O.cost_affine_3(a, b, om), (model, i, len(a), len(b))
        assert cells[i] == O.band_cells_affine(len(a), len(b))


@pytest.mark.parametrize("model", MODELS)
def test_affine_align_matches_oracle(model):
    A, B = _pairs(77 + model[0], 40, 800)
    cm = align.CostMatrix.dna(*model)
    om = O.cm_dna(*model)
    res = align.align_2(align.PairBatch.from_host(A, B), cm).to_host()
    for i, (a, b) in enumerate(zip(A, B)):
        c, med, mwg, ri, rj = O.align_affine_3(a, b, om)
        r = res[i]
        assert r["cost"] == c, (model, i, len(a), len(b))
        assert np.array_equal(r["a"], ri) and np.array_equal(r["b"], rj), (model, i)
        assert np.array_equal(r["median"], med) and np.array_equal(r["median_wg"], mwg), (model, i)


@pytest.mark.parametrize("model", G.AFFINE)
def test_affine_golden_vectors(model):
    g = G.load()
    tag = "aff_%d_%d_%d" % model
    cm = align.CostMatrix.dna(*model)
    batch = align.PairBatch.from_host(g["A"], g["B"])
    cost, _ = align.cost_2(batch, cm)
    assert np.array_equal(cost.cpu().numpy(), g[tag + "_cost"])
    res = align.align_2(batch, cm).to_host()
    med, ri = G.seqs(g, tag + "_median"), G.seqs(g, tag + "_resi")
    for i, r in enumerate(res):
        assert r["cost"] == g[tag + "_cost_bt"][i]
        assert np.array_equal(r["median"], med[i]) and np.array_equal(r["a"], ri[i])
