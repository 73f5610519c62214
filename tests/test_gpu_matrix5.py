"""A user-supplied 5x5 transformation matrix that breaks the triangle
inequality (Cost_matrix.Two_D.of_list, cost_matrix.ml:520-538 takes the
bitwise fill for it) through the CUDA linear and affine paths and the
column kernels, against the oracle, bit-exact."""
import numpy as np
import pytest

from oracle import oracle as O
from poyd_gb300 import align, synth

pytestmark = pytest.mark.gpu

# A, C, G, T, gap: A-C costs more than A-G + G-C
NONMETRIC = np.array([[0, 7, 2, 3, 4],
                      [7, 0, 2, 5, 4],
                      [2, 2, 0, 1, 3],
                      [3, 5, 1, 0, 4],
                      [4, 4, 3, 4, 0]], np.int32)


def _oracle_cm(gap_open):
    m = O.OrCM()
    O.lib().or_cm_of_matrix5(O.C.byref(m), NONMETRIC.ctypes.data_as(O.i32p), gap_open)
    assert not m.is_metric
    return m


def _pairs(seed):
    A, B = synth.pair_batch(seed, 40, lmin=1, lmax=700)
    rng = np.random.default_rng(seed)
    for n1, n2 in [(0, 0), (0, 7), (6, 0), (1, 1), (64, 63), (200, 90)]:
        A.append(synth.with_gap(synth.random_dna(rng, n1, 0.1)))
        B.append(synth.with_gap(synth.random_dna(rng, n2, 0.1)))
    return A, B


@pytest.mark.parametrize("gap_open", [None, 2])
def test_nonmetric_matrix_matches_oracle(gap_open):
    cm = align.CostMatrix.of_matrix5(NONMETRIC, gap_open)
    om = _oracle_cm(-1 if gap_open is None else gap_open)
    assert np.array_equal(cm.tables()["cost"], np.ctypeslib.as_array(om.cost))
    A, B = _pairs(41 if gap_open is None else 42)
    res = align.align_2(align.PairBatch.from_host(A, B), cm).to_host()
    RA, RB = [], []
    for i, (a, b) in enumerate(zip(A, B)):
        if gap_open is None:
            c, ra, rb = O.align_2(a, b, om)
            assert np.array_equal(res[i]["median"], O.ancestor_2(ra, rb, om)), i
        else:
            c, med, _, ra, rb = O.align_affine_3(a, b, om)
            assert np.array_equal(res[i]["median"], med), i
        assert res[i]["cost"] == c, (i, len(a), len(b))
        assert np.array_equal(res[i]["a"], ra) and np.array_equal(res[i]["b"], rb), i
        RA.append(ra)
        RB.append(rb)
    for op, fn in (("median_2_with_gaps", O.median_2_with_gaps), ("worst_2", O.worst_2),
                   ("verify_2", O.verify_2)):
        got = align.columns(op, RA, RB, cm)
        for i, (ra, rb) in enumerate(zip(RA, RB)):
            assert np.array_equal(np.asarray(got[i]), np.asarray(fn(ra, rb, om))), (op, i)
