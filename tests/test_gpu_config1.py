"""The batched CUDA path at the benchmark's lengths (1,500-5,000 bp), compared
in full with the oracle: 64 pairs of the benchmark's generator plus pairs in
every band case of algn_fill_plane_2 (the same pairs the oracle is pinned on
against the compiled reference), for four linear and three affine models.
Bit-exact: every cost, aligned sequence and median."""
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from oracle import oracle as O
from poyd_gb300 import align
from tests.regimes import band_case, config1_pairs

pytestmark = pytest.mark.gpu

MODELS = [(1, 2, -1), (1, 1, -1), (3, 1, -1), (2, 3, -1), (1, 2, 3), (2, 1, 1), (3, 1, 5)]


def _oracle_all(A, B, om):
    # ctypes drops the GIL: the oracle runs on host threads, no fork
    with ThreadPoolExecutor(8) as ex:
        return list(ex.map(lambda ab: O.dos_median(ab[0], ab[1], om), zip(A, B)))


@pytest.mark.parametrize("model", MODELS)
def test_config1_lengths_match_oracle(model):
    A, B = config1_pairs(900 + sum(model), 64)
    assert len(A) == 72
    cm = align.CostMatrix.dna(model[0], model[1], None if model[2] < 0 else model[2])
    om = O.cm_dna(*model)
    if model[2] < 0:
        cases = {band_case(max(len(a), len(b)), min(len(a), len(b)), O.deltaw(a, b, om))
                 for a, b in zip(A, B)}
        assert cases == {"full", "narrow", "rows"}
    batch = align.PairBatch.from_host(A, B)
    res = align.align_2(batch, cm).to_host()
    cost, _ = align.cost_2(batch, cm)
    cost = cost.cpu().numpy()
    want = _oracle_all(A, B, om)
    for i, (c, med, ra, rb, wg) in enumerate(want):
        r = res[i]
        assert r["cost"] == c, (model, i, len(A[i]), len(B[i]))
        assert np.array_equal(r["a"], ra) and np.array_equal(r["b"], rb), (model, i)
        assert np.array_equal(r["median"], med), (model, i)
        assert np.array_equal(r["median_wg"], wg), (model, i)
        if model[2] < 0:
            assert cost[i] == c, (model, i)
        else:
            assert cost[i] == O.cost_affine_3(A[i], B[i], om), (model, i)
