"""The single-pair drop-ins keep the OCaml externals' protocol:
algn_CAML_simple_2 leaves the direction matrix in a Matrix.m stand-in and
algn_CAML_backtrack_2d reads it with either tie priority (swaped)."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from poyd_gb300 import align, native, synth

pytestmark = pytest.mark.gpu


def P(a):
    return C.c_void_p(a.ctypes.data)


def test_simple_2_then_backtrack_both_priorities():
    L = native.lib()
    L.poyd_matrix_create.restype = C.c_void_p
    L.poyd_matrix_free.argtypes = [C.c_void_p]
    mat = L.poyd_matrix_create()
    cm = align.CostMatrix.default()
    om = O.cm_dna(1, 2, -1)
    rng = np.random.default_rng(12)
    try:
        for t in range(12):
            n1 = int(rng.integers(1, 700))
            n2 = max(0, n1 - int(rng.integers(0, 80)))
            s1 = synth.with_gap(synth.random_dna(rng, n1, 0.05))
            s2 = synth.with_gap(synth.mutate(rng, synth.random_dna(rng, n2, 0.05), 0.2, 0.03))
            if len(s2) > len(s1):
                s1, s2 = s2, s1
            dw = int(rng.integers(0, 100))
            cost = C.c_int32()
            assert L.poyd_algn_simple_2(P(s1), len(s1), P(s2), len(s2), cm.ref, C.c_void_p(mat),
                                        dw, C.byref(cost)) == 0, L.poyd_last_error()
            c_ref, dm = O.simple_2(s1, s2, om, dw, want_dm=True)
            assert cost.value == c_ref
            for swaped in (1, 0):
                cap = len(s1) + len(s2)
                r1 = np.zeros(cap, np.uint8)
                r2 = np.zeros(cap, np.uint8)
                n = C.c_int32()
                assert L.poyd_algn_backtrack_2d(P(s1), len(s1), P(s2), len(s2), P(r1), P(r2), cap,
                                                C.byref(n), C.c_void_p(mat), cm.ref, swaped) == 0
                o1 = np.zeros(cap + 1, np.uint8)
                o2 = np.zeros(cap + 1, np.uint8)
                k = O.lib().or_backtrack_2d(s1.ctypes.data_as(O.u8p), len(s1),
                                            s2.ctypes.data_as(O.u8p), len(s2),
                                            dm.ctypes.data_as(C.POINTER(C.c_uint16)),
                                            C.byref(om), swaped, o1.ctypes.data_as(O.u8p),
                                            o2.ctypes.data_as(O.u8p))
                assert n.value == k
                assert np.array_equal(r1[cap - k:], o1[:k]) and np.array_equal(r2[cap - k:], o2[:k])
                # algn_CAML_align_2d: the two calls in one
                q1 = np.zeros(cap, np.uint8)
                q2 = np.zeros(cap, np.uint8)
                m, c2 = C.c_int32(), C.c_int32()
                assert L.poyd_algn_align_2d(P(s1), len(s1), P(s2), len(s2), cm.ref,
                                            C.c_void_p(mat), P(q1), P(q2), cap, C.byref(m), dw,
                                            swaped, C.byref(c2)) == 0, L.poyd_last_error()
                assert c2.value == c_ref and m.value == k
                assert np.array_equal(q1, r1) and np.array_equal(q2, r2)
    finally:
        L.poyd_matrix_free(C.c_void_p(mat))


def test_affine_single_pair():
    L = native.lib()
    cm = align.CostMatrix.dna(1, 2, 3)
    om = O.cm_dna(1, 2, 3)
    rng = np.random.default_rng(4)
    for t in range(6):
        a = synth.with_gap(synth.random_dna(rng, int(rng.integers(1, 500)), 0.05))
        b = synth.with_gap(synth.mutate(rng, a[1:], 0.2, 0.04))
        cost = C.c_int32()
        assert L.poyd_algn_cost_affine_3(P(a), len(a), P(b), len(b), cm.ref, C.byref(cost)) == 0
        assert cost.value == O.cost_affine_3(a, b, om)
        cap = len(a) + len(b) + 2
        bufs = [np.zeros(cap, np.uint8) for _ in range(4)]
        lens = (C.c_int32 * 3)()
        assert L.poyd_algn_align_affine_3(P(a), len(a), P(b), len(b), cm.ref, *[P(x) for x in bufs],
                                          cap, lens, C.byref(cost)) == 0
        c, med, mwg, ri, rj = O.align_affine_3(a, b, om)
        assert cost.value == c
        assert np.array_equal(bufs[0][cap - lens[0]:], ri) and np.array_equal(bufs[1][cap - lens[0]:], rj)
        assert np.array_equal(bufs[2][cap - lens[1]:], med)
        assert np.array_equal(bufs[3][cap - lens[2]:], mwg)
