"""Batched DOS.readjust of the Iterative modes (poyd_gb300/iterative.py:
ThreeD through the three-sequence kernel, ApproxD through batched pairwise
alignments, median_2 and Align.closest) against the oracle's composition
(oracle.dos_readjust, seqCS.ml:680-722 over sequence.ml:1117-1195), result
for result: the new sequence, its cost and the changed flag, including
nodes with empty neighbours."""
import numpy as np
import pytest

from oracle import oracle as O
from poyd_gb300 import align, iterative, synth

pytestmark = pytest.mark.gpu


def items():
    rng = np.random.default_rng(4)
    out = []
    for a, b, p in synth.triple_batch(41, 24, lmin=0, lmax=80, ambig=0.05):
        mine = a.copy() if rng.random() < 0.5 else synth.with_gap(synth.random_dna(rng, 30))
        out.append((a, b, p, mine))
    e = np.array([16], np.uint8)
    a, b, p, mine = out[1]
    out += [(e, b, p, mine), (a, e, p, mine), (a, b, e, mine), (e, e, p, mine),
            (e, b, e, mine), (a, e, e, mine), (e, e, e, mine), (a, b, p, b.copy())]
    return out


@pytest.mark.parametrize("mode", ["three", "approx"])
@pytest.mark.parametrize("model", [(1, 2, -1), (1, 1, -1), (1, 2, 3)])
def test_dos_readjust_matches_oracle(mode, model):
    sub, indel, go = model
    cm = align.CostMatrix.dna(sub, indel, None if go < 0 else go)
    m = O.cm_dna(sub, indel, go)
    it = items()
    got = iterative.dos_readjust(it, cm, mode)
    for k, x in enumerate(it):
        ch, res, cost = O.dos_readjust(mode, x[0], x[1], x[2], x[3], m)
        assert got[k][0] == ch and got[k][2] == cost, (k, mode, model, got[k][2], cost)
        assert np.array_equal(got[k][1], res), (k, mode, model)
