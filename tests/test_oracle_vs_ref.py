"""The oracle restatement against the reference's own C kernels compiled from
source (oracle/build_ref.sh) on seeded random inputs.  Skipped where the
reference sources are absent (the compiled reference does not travel)."""
import ctypes as C
import os
import platform

import numpy as np
import pytest

from oracle import oracle as O
from poyd_gb300 import synth
from tests.regimes import band_case, config1_pairs

@pytest.fixture(scope="module")
def R():
    if O.build_ref() is None:
        pytest.skip("reference sources not present")
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


@pytest.mark.parametrize("model", [(1, 2), (1, 1), (3, 1), (2, 3)])
def test_linear_vs_reference_config1_lengths(R, model):
    """align_2 + ancestor_2 + median_2_with_gaps at 1,500-5,000 bp, every
    band case of algn_fill_plane_2 included."""
    m = O.cm_dna(model[0], model[1], -1)
    rc = R.ref_cm_new(C.byref(m))
    A, B = config1_pairs(400 + model[0] * 10 + model[1], 40)
    cases = set()
    for a, b in zip(A, B):
        dw = O.deltaw(a, b, m)
        cases.add(band_case(max(len(a), len(b)), min(len(a), len(b)), dw))
        cap = len(a) + len(b) + 2
        o1, o2 = np.zeros(cap, np.uint8), np.zeros(cap, np.uint8)
        n = C.c_int()
        c_ref = R.ref_align_2(P(a), len(a), P(b), len(b), rc, dw, P(o1), P(o2), C.byref(n))
        c, ra, rb = O.align_2(a, b, m)
        assert c == c_ref, (model, len(a), len(b))
        assert np.array_equal(ra, o1[:n.value]) and np.array_equal(rb, o2[:n.value])
        t = np.zeros(len(ra) + 2, np.uint8)
        k = R.ref_ancestor_2(P(ra), P(rb), len(ra), rc, P(t))
        assert np.array_equal(O.ancestor_2(ra, rb, m), t[:k])
        w = np.zeros(len(ra) + 2, np.uint8)
        k = R.ref_median_2_with_gaps(P(ra), P(rb), len(ra), rc, P(w))
        assert np.array_equal(O.median_2_with_gaps(ra, rb, m), w[:k])
    R.ref_cm_free(rc)
    assert cases == {"full", "narrow", "rows"}


@pytest.mark.parametrize("model", [(1, 2, 3), (2, 1, 1), (3, 1, 5)])
def test_affine_vs_reference_config1_lengths(R, model):
    """cost_affine_3 and align_affine_3 at 1,500-5,000 bp."""
    m = O.cm_dna(*model)
    rc = R.ref_cm_new(C.byref(m))
    A, B = config1_pairs(500 + sum(model), 40)
    for a, b in zip(A, B):
        assert O.cost_affine_3(a, b, m) == R.ref_cost_affine_3(P(a), len(a), P(b), len(b), rc)
        cap = len(a) + len(b) + 3
        bufs = [np.zeros(cap, np.uint8) for _ in range(4)]
        lm, lw, lr = C.c_int(), C.c_int(), C.c_int()
        c_ref = R.ref_align_affine_3(P(a), len(a), P(b), len(b), rc, P(bufs[0]), C.byref(lm),
                                     P(bufs[1]), C.byref(lw), P(bufs[2]), P(bufs[3]),
                                     C.byref(lr))
        c, med, mwg, ri, rj = O.align_affine_3(a, b, m)
        assert c == c_ref, (model, len(a), len(b))
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


# A 5x5 input (A, C, G, T, gap) that breaks the triangle inequality
# (A-C costs more than A-G + G-C), so the tables take the bitwise fill
# (cost_matrix.ml:520-538) rather than the metric one.
NONMETRIC = np.array([[0, 7, 2, 3, 4],
                      [7, 0, 2, 5, 4],
                      [2, 2, 0, 1, 3],
                      [3, 5, 1, 0, 4],
                      [4, 4, 3, 4, 0]], np.int32)


def _cm(model):
    if model == "nonmetric":
        m = O.OrCM()
        O.lib().or_cm_of_matrix5(C.byref(m), NONMETRIC.ctypes.data_as(O.i32p), -1)
        assert not m.is_metric
        return m
    return O.cm_dna(*model)


def _aligned(m, seed, n, lmax):
    A, B = _pairs(seed, n, lmax)
    out = []
    for a, b in zip(A, B):
        if m.cost_model == 1:
            _, _, _, ra, rb = O.align_affine_3(a, b, m)
        else:
            _, ra, rb = O.align_2(a, b, m)
        out.append((ra, rb))
    # gap-and-base codes on both sides of a column, and a lone gap column
    out.append((np.array([16, 17, 18, 1, 16, 31], np.uint8),
                np.array([16, 16, 24, 20, 2, 15], np.uint8)))
    out.append((np.array([16], np.uint8), np.array([16], np.uint8)))
    return out


@pytest.mark.parametrize("model", [(1, 2, -1), (3, 1, -1), "nonmetric", (1, 2, 3), (2, 1, 1)])
def test_column_ops_vs_reference(R, model):
    """median_2_with_gaps, median_2_no_gaps, ancestor_2, worst_2 and
    verify_2 (algn.c) on aligned pairs, the oracle against the reference."""
    m = _cm(model)
    rc = R.ref_cm_new(C.byref(m))
    for ra, rb in _aligned(m, 31, 40, 900):
        n = len(ra)
        for name, want in (("ref_median_2_with_gaps", O.median_2_with_gaps(ra, rb, m)),
                           ("ref_median_2_no_gaps", O.median_2(ra, rb, m)),
                           ("ref_ancestor_2", O.ancestor_2(ra, rb, m))):
            t = np.zeros(n + 2, np.uint8)
            k = getattr(R, name)(P(ra), P(rb), n, rc, P(t))
            assert np.array_equal(want, t[:k]), name
        assert R.ref_worst_2(P(ra), P(rb), n, rc) == O.worst_2(ra, rb, m)
        assert R.ref_verify_2(P(ra), P(rb), n, rc) == O.verify_2(ra, rb, m)
    R.ref_cm_free(rc)


def test_nonmetric_align_vs_reference(R):
    m = _cm("nonmetric")
    rc = R.ref_cm_new(C.byref(m))
    for a, b in zip(*_pairs(77, 40, 1000)):
        dw = O.deltaw(a, b, m)
        cap = len(a) + len(b) + 2
        o1, o2 = np.zeros(cap, np.uint8), np.zeros(cap, np.uint8)
        n = C.c_int()
        c_ref = R.ref_align_2(P(a), len(a), P(b), len(b), rc, dw, P(o1), P(o2), C.byref(n))
        c, ra, rb = O.align_2(a, b, m)
        assert c == c_ref
        assert np.array_equal(ra, o1[:n.value]) and np.array_equal(rb, o2[:n.value])
    R.ref_cm_free(rc)


@pytest.mark.parametrize("dw", [0, 1, 5, 40, 400])
def test_explicit_band_vs_reference(R, dw):
    """simple_2 with a caller-chosen band width (the ?deltaw argument of
    Sequence.Align.cost_2): the cost depends on the band, and both agree."""
    m = O.cm_dna(1, 2, -1)
    rc = R.ref_cm_new(C.byref(m))
    for a, b in zip(*_pairs(dw + 3, 30, 700)):
        s1, s2 = (a, b) if len(a) >= len(b) else (b, a)
        assert O.simple_2(s1, s2, m, dw) == R.ref_simple_2(P(s1), len(s1), P(s2), len(s2), rc, dw)
    R.ref_cm_free(rc)


def test_fitch_median_3_vs_reference(R):
    rng = np.random.default_rng(12)
    for _ in range(20):
        n = int(rng.integers(1, 3000))
        A, N, D1, D2 = (rng.integers(1, 256, n).astype(np.uint8) for _ in range(4))
        f = np.zeros(n, np.uint8)
        R.ref_nonadd8_median_3(P(A), P(N), P(D1), P(D2), n, P(f))
        assert np.array_equal(O.nonadd_median_3(A, N, D1, D2), f)


@pytest.mark.skipif(platform.machine() != "x86_64",
                    reason="the asm/C switch of algn.c exists on x86-64 only")
def test_reference_c_cell_path_vs_oracle(R):
    """algn.c has an inline-asm cell path (x86-64 with MMX) and a plain-C
    one (algn.c:375-453, the one an arm64 build compiles).  The C path,
    built with POYD_REF_C_PATH=1, agrees with the oracle as the asm path
    does."""
    assert O.build_ref(env=dict(os.environ, POYD_REF_C_PATH="1")) is not None
    Rc = C.CDLL(os.path.join(os.path.dirname(O.REF_PATH), "libporef_cpath.so"))
    Rc.ref_cm_new.argtypes = [C.POINTER(O.OrCM)]
    Rc.ref_cm_new.restype = C.c_void_p
    Rc.ref_cm_free.argtypes = [C.c_void_p]
    Rc.ref_align_2.argtypes = [O.u8p, C.c_int, O.u8p, C.c_int, C.c_void_p, C.c_int, O.u8p,
                               O.u8p, C.POINTER(C.c_int)]
    for model in [(1, 2), (3, 1)]:
        m = O.cm_dna(model[0], model[1], -1)
        rc = Rc.ref_cm_new(C.byref(m))
        for a, b in zip(*_pairs(90 + model[0], 30, 1200)):
            cap = len(a) + len(b) + 2
            o1, o2 = np.zeros(cap, np.uint8), np.zeros(cap, np.uint8)
            n = C.c_int()
            c_ref = Rc.ref_align_2(P(a), len(a), P(b), len(b), rc, O.deltaw(a, b, m), P(o1), P(o2),
                                   C.byref(n))
            c, ra, rb = O.align_2(a, b, m)
            assert c == c_ref
            assert np.array_equal(ra, o1[:n.value]) and np.array_equal(rb, o2[:n.value])
        Rc.ref_cm_free(rc)


def _sparse_sets(rng, n, width):
    """n non-empty state sets of 1-3 states out of `width`, so that about
    half of the pairs do not intersect."""
    out = np.zeros(n, np.uint64)
    for _ in range(3):
        bit = rng.integers(0, width, n).astype(np.uint64)
        keep = rng.random(n) < 0.6
        out |= np.where(keep, np.uint64(1) << bit, np.uint64(0))
    out[out == 0] = np.uint64(1) << rng.integers(0, width, int((out == 0).sum())).astype(np.uint64)
    return out.astype({8: np.uint8, 16: np.uint16, 32: np.uint32}[width])


@pytest.mark.parametrize("width", [16, 32])
def test_wide_fitch_vs_reference(R, width):
    """NonaddCS16 / NonaddCS32 (nonaddCSc.c at CHARSIZE 16 / 32): median,
    distance and median_3 of the oracle against the reference."""
    rng = np.random.default_rng(width)
    med = getattr(R, "ref_nonadd%d_median" % width)
    dist = getattr(R, "ref_nonadd%d_distance" % width)
    med3 = getattr(R, "ref_nonadd%d_median_3" % width)
    for n in (1, 7, 8, 9, 31, 200, 1999):
        a, b, c, d = (_sparse_sets(rng, n, width) for _ in range(4))
        r = np.zeros_like(a)
        c_ref = med(a.ctypes.data, b.ctypes.data, n, r.ctypes.data)
        c_or, r_or = O.nonadd_median_w(a, b, width)
        assert c_ref == c_or and np.array_equal(r, r_or), n
        assert dist(a.ctypes.data, b.ctypes.data, n) == O.nonadd_distance_w(a, b, width)
        f = np.zeros_like(a)
        med3(a.ctypes.data, b.ctypes.data, c.ctypes.data, d.ctypes.data, n, f.ctypes.data)
        assert np.array_equal(f, O.nonadd_median_3_w(a, b, c, d, width)), n


def test_fitch_dist_2_vs_reference(R):
    """char_nonadd8_CAML_dist_2 (nonaddCSc.c:1349-1376)."""
    rng = np.random.default_rng(13)
    for n in (1, 15, 16, 17, 500, 3001):
        a, b, c = (_sparse_sets(rng, n, 8) for _ in range(3))
        assert R.ref_nonadd8_dist_2(P(a), P(b), P(c), n) == O.nonadd_dist_2(a, b, c)
