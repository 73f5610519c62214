"""Column operations on aligned pairs (median_2_with_gaps, median_2_no_gaps,
ancestor_2, worst_2, verify_2) through the CUDA kernels against the
oracle, batched and single-pair, bit-exact."""
import numpy as np
import pytest

from oracle import oracle as O
from poyd_gb300 import align, synth

pytestmark = pytest.mark.gpu

MODELS = [(1, 2, -1), (1, 1, -1), (2, 1, 1), (3, 1, 5)]
ORACLE = {"median_2_with_gaps": O.median_2_with_gaps, "median_2_no_gaps": O.median_2,
          "ancestor_2": O.ancestor_2, "worst_2": O.worst_2, "verify_2": O.verify_2}


def _aligned(model, seed=11, n=80):
    """Aligned pairs from the oracle's own alignments, plus edge cases."""
    sub, indel, go = model
    om = O.cm_dna(sub, indel, go)
    rng = np.random.default_rng(seed)
    A, B = [], []
    for t in range(n):
        a = synth.with_gap(synth.random_dna(rng, int(rng.integers(0, 300)), 0.1))
        b = synth.with_gap(synth.mutate(rng, a[1:], 0.2, 0.05))
        if t % 9 == 0:
            b = b.copy()
            b[rng.random(len(b)) < 0.2] = 17 + int(rng.integers(0, 15))  # gap-and-base codes
            b[0] = 16
        if go >= 0:
            _, _, _, ra, rb = O.align_affine_3(a, b, om)
        else:
            _, ra, rb = O.align_2(a, b, om)
        A.append(ra)
        B.append(rb)
    # a lone leading-gap column, gap runs on both sides, gap-and-base columns
    A += [np.array([16], np.uint8), np.array([16, 1, 16, 16, 4, 16], np.uint8),
          np.array([16, 17, 18, 1, 16], np.uint8)]
    B += [np.array([16], np.uint8), np.array([16, 16, 2, 8, 16, 16], np.uint8),
          np.array([16, 16, 24, 20, 2], np.uint8)]
    return A, B, om


@pytest.mark.parametrize("model", MODELS)
@pytest.mark.parametrize("op", sorted(ORACLE))
def test_columns_match_oracle(model, op):
    A, B, om = _aligned(model)
    cm = align.CostMatrix.dna(model[0], model[1], model[2] if model[2] >= 0 else None)
    got = align.columns(op, A, B, cm)
    for i, (a, b) in enumerate(zip(A, B)):
        want = ORACLE[op](a, b, om)
        if isinstance(want, np.ndarray):
            assert np.array_equal(got[i], want), (op, i)
        else:
            assert got[i] == want, (op, i)
    for i in (0, len(A) - 2, len(A) - 1):
        single = align.column_pair(op, A[i], B[i], cm)
        want = ORACLE[op](A[i], B[i], om)
        assert np.array_equal(np.asarray(single), np.asarray(want)), (op, i)
