"""The packed linear DP (csrc/linear4.cu: four rows per lane in 16-bit
halves) against the 32-bit kernel (csrc/linear.cu, forced with
POYD_PACKED=0) and the oracle, on the same batches: costs (cost_2 under the
three deltaw policies) and every output of align_2, bit-exact."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from poyd_gb300 import align, synth
from tests.regimes import config1_pairs

pytestmark = pytest.mark.gpu


def _batch(seed, n, lmax):
    A, B = synth.pair_batch(seed, n, lmin=1, lmax=lmax)
    rng = np.random.default_rng(seed)
    g = synth.with_gap
    for n1, n2 in [(0, 0), (0, 9), (4, 0), (1, 1), (127, 129), (128, 128), (130, 2),
                   (600, 40), (40, 600), (255, 256), (900, 880)]:
        A.append(g(synth.random_dna(rng, n1, 0.1)))
        B.append(g(synth.random_dna(rng, n2, 0.1)))
    return A, B


def _both(monkeypatch, fn):
    monkeypatch.setenv("POYD_PACKED", "0")
    ref = fn()
    monkeypatch.setenv("POYD_PACKED", "1")
    got = fn()
    monkeypatch.delenv("POYD_PACKED")
    return ref, got


@pytest.mark.parametrize("model", [(1, 2), (1, 1), (3, 1), (2, 3)])
def test_packed_align_matches_32bit_and_oracle(model, monkeypatch):
    A, B = _batch(40 + model[0] * 3 + model[1], 120, 2500)
    cm = align.CostMatrix.dna(*model)
    om = O.cm_dna(model[0], model[1], -1)
    batch = align.PairBatch.from_host(A, B)
    ref, got = _both(monkeypatch, lambda: align.align_2(batch, cm).to_host())
    for i, (a, b) in enumerate(zip(A, B)):
        c, ra, rb = O.align_2(a, b, om)
        r = got[i]
        assert r["cost"] == c, (model, i, len(a), len(b))
        assert np.array_equal(r["a"], ra) and np.array_equal(r["b"], rb), (model, i)
        assert np.array_equal(r["median"], O.ancestor_2(ra, rb, om)), (model, i)
        assert np.array_equal(r["median_wg"], O.median_2_with_gaps(ra, rb, om)), (model, i)
        for k in ("cost", "a", "b", "median", "median_wg"):
            assert np.array_equal(ref[i][k], got[i][k]), (model, i, k)


@pytest.mark.parametrize("deltaw", [None, "dos", "explicit"])
def test_packed_cost_matches_32bit(deltaw, monkeypatch):
    A, B = _batch(77, 200, 3000)
    cm = align.CostMatrix.dna(1, 2)
    batch = align.PairBatch.from_host(A, B)
    dw = deltaw
    if deltaw == "explicit":
        dw = torch.from_numpy(np.random.default_rng(3).integers(0, 400, len(A)).astype(np.int32)).cuda()
    ref, got = _both(monkeypatch, lambda: align.cost_2(batch, cm, deltaw=dw)[0].cpu().numpy())
    assert np.array_equal(ref, got)
    om = O.cm_dna(1, 2, -1)
    for i in range(0, len(A), 7):
        if deltaw is None:
            assert got[i] == O.cost_2(A[i], B[i], om), i


def test_packed_config1_regime(monkeypatch):
    """The benchmark's regime (1,500-5,000 bp, every band case): both kernels
    give the same outputs."""
    A, B = config1_pairs(4242, 48)
    cm = align.CostMatrix.default()
    batch = align.PairBatch.from_host(A, B)
    ref, got = _both(monkeypatch, lambda: align.align_2(batch, cm).to_host())
    for i in range(len(A)):
        for k in ("cost", "a", "b", "median", "median_wg"):
            assert np.array_equal(ref[i][k], got[i][k]), (i, k)
