"""Parity of the batched Sequence.Align.closest (DOS.to_single) with the
oracle, bit-exact, for linear and affine matrices."""
import numpy as np
import pytest

from oracle import oracle as O
from poyd_gb300 import align, synth

pytestmark = pytest.mark.gpu

MODELS = [(1, 2, -1), (1, 1, -1), (2, 1, 1), (3, 1, 5)]


def _pairs(seed):
    rng = np.random.default_rng(seed)
    g = synth.with_gap
    P, M = [], []
    for t in range(300):
        n1 = int(rng.integers(0, 400))
        p = synth.random_dna(rng, n1, 0.1)
        m = synth.mutate(rng, p, 0.15, 0.04)
        if t % 5 == 0:
            m = m.copy()
            m[rng.random(len(m)) < 0.2] = synth.AMBIG[0]
        P.append(g(p))
        M.append(g(m))
    # identical sequences, empty parent, empty node, both empty
    s = g(synth.random_dna(rng, 90, 0.2))
    P += [s, g(np.zeros(0, np.uint8)), g(synth.random_dna(rng, 30)), g(np.zeros(0, np.uint8))]
    M += [s.copy(), g(synth.random_dna(rng, 50, 0.3)), g(np.zeros(0, np.uint8)),
          g(np.zeros(0, np.uint8))]
    # gap-and-base codes (17..31) on one side
    a = synth.random_dna(rng, 200, 0.05)
    b = a.copy()
    b[rng.random(len(b)) < 0.3] = 31
    P.append(g(a))
    M.append(g(b))
    P.append(g(b))
    M.append(g(a))
    return P, M


@pytest.mark.parametrize("model", MODELS)
def test_closest_matches_oracle(model):
    sub, indel, go = model
    P, M = _pairs(sub * 10 + indel)
    cm = align.CostMatrix.dna(sub, indel, go if go >= 0 else None)
    om = O.cm_dna(sub, indel, go)
    res = align.closest(align.PairBatch.from_host(P, M), cm, dos_empty=True).to_host()
    for i, (p, m) in enumerate(zip(P, M)):
        want = O.closest(p, m, om, dos_empty=True)
        assert np.array_equal(res[i]["median"], want), i


def test_closest_without_dos_rule():
    """Without DOS.to_single's rule an all-gap parent is aligned as is."""
    cm = align.CostMatrix.default()
    om = O.cm_dna(1, 2, -1)
    rng = np.random.default_rng(5)
    P = [synth.with_gap(np.zeros(0, np.uint8))] * 3
    M = [synth.with_gap(synth.random_dna(rng, n, 0.3)) for n in (1, 17, 60)]
    res = align.closest(align.PairBatch.from_host(P, M), cm, dos_empty=False).to_host()
    for i in range(3):
        assert np.array_equal(res[i]["median"], O.closest(P[i], M[i], om, dos_empty=False))
