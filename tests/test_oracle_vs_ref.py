"""The oracle restatement against the reference's own C kernels compiled from
source (oracle/build_ref.sh) on seeded random inputs.  Skipped where the
reference sources are absent (the compiled reference does not travel)."""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import oracle as O
from poyd_gb300 import synth

REF_SRC = os.environ.get("POYD_REFERENCE_SRC", "/root/reference/src")
pytestmark = pytest.mark.skipif(not os.path.exists(os.path.join(REF_SRC, "algn.c")),
                                reason="reference sources not present")


@pytest.fixture(scope="module")
def R():
    O.build_ref(REF_SRC)
    r = O.ref()
    assert r is not None
    return r


def P(a):
    return a.ctypes.data_as(O.u8p)


def _pairs(seed, n, lmax):
    rng = np.random.default_rng(seed)
    A, B = [], []
    for t in range(n):
        n1 = int(rng.integers(0, lmax))
        n2 = int(rng.integers(0, lmax)) if t % 3 == 0 else max(0, n1 + int(rng.integers(-80, 80)))
        a = synth.with_gap(synth.random_dna(rng, n1, 0.05))
        b = synth.with_gap(synth.mutate(rng, synth.random_dna(rng, n2, 0.05), 0.2, 0.03))
        if t % 7 == 0:
            b[rng.random(len(b)) < 0.1] = 16
        A.append(a)
        B.append(b)
    return A, B


@pytest.mark.parametrize("model", [(1, 2), (1, 1), (3, 1), (2, 3)])
def test_linear_vs_reference(R, model):
    m = O.cm_dna(model[0], model[1], -1)
    rc = R.ref_cm_new(C.byref(m))
    A, B = _pairs(model[0] * 10 + model[1], 80, 1500)
    for a, b in zip(A, B):
        dw = O.deltaw(a, b, m)
        cap = len(a) + len(b) + 2
        o1, o2 = np.zeros(cap, np.uint8), np.zeros(cap, np.uint8)
        n = C.c_int()
        c_ref = R.ref_align_2(P(a), len(a), P(b), len(b), rc, dw, P(o1), P(o2), C.byref(n))
        c, ra, rb = O.align_2(a, b, m)
        assert c == c_ref
        assert np.array_equal(ra, o1[:n.value]) and np.array_equal(rb, o2[:n.value])
        t = np.zeros(len(ra) + 2, np.uint8)
        k = R.ref_ancestor_2(P(ra), P(rb), len(ra), rc, P(t))
        assert np.array_equal(O.ancestor_2(ra, rb, m), t[:k])
        assert R.ref_worst_2(P(ra), P(rb), len(ra), rc) == O.worst_2(ra, rb, m)
    R.ref_cm_free(rc)


@pytest.mark.parametrize("model", [(1, 2, 3), (2, 1, 1), (3, 1, 5)])
def test_affine_vs_reference(R, model):
    m = O.cm_dna(*model)
    rc = R.ref_cm_new(C.byref(m))
    A, B = _pairs(sum(model), 50, 1200)
    for a, b in zip(A, B):
        assert O.cost_affine_3(a, b, m) == R.ref_cost_affine_3(P(a), len(a), P(b), len(b), rc)
        cap = len(a) + len(b) + 3
        bufs = [np.zeros(cap, np.uint8) for _ in range(4)]
        lm, lw, lr = C.c_int(), C.c_int(), C.c_int()
        c_ref = R.ref_align_affine_3(P(a), len(a), P(b), len(b), rc, P(bufs[0]), C.byref(lm),
                                     P(bufs[1]), C.byref(lw), P(bufs[2]), P(bufs[3]),
                                     C.byref(lr))
        c, med, mwg, ri, rj = O.align_affine_3(a, b, m)
        assert c == c_ref
        assert np.array_equal(med, bufs[0][:lm.value]) and np.array_equal(mwg, bufs[1][:lw.value])
        assert np.array_equal(ri, bufs[2][:lr.value]) and np.array_equal(rj, bufs[3][:lr.value])
    R.ref_cm_free(rc)


def test_fitch_vs_reference(R):
    rng = np.random.default_rng(11)
    for _ in range(20):
        n = int(rng.integers(1, 4000))
        a = rng.integers(1, 256, n).astype(np.uint8)
        b = rng.integers(1, 256, n).astype(np.uint8)
        r1 = np.zeros(n, np.uint8)
        c1 = R.ref_nonadd8_median(P(a), P(b), n, P(r1))
        c2, r2 = O.nonadd_median(a, b)
        assert c1 == c2 and np.array_equal(r1, r2)
        assert R.ref_nonadd8_distance(P(a), P(b), n) == O.nonadd_distance(a, b)
