"""The C-ABI library: builds, loads, exports every entry point the public
header declares, and its cost-matrix constructors match the oracle's
restatement of cost_matrix.ml.  No GPU needed."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from oracle import oracle as O
from poyd_gb300 import build, native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "poyd_gb300.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(poyd_[A-Za-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return native.lib()


def test_library_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


@pytest.mark.parametrize("model", [(1, 2, -1), (1, 1, -1), (3, 1, -1), (2, 1, 1), (3, 1, 5),
                                   (1, 2, 3), (1, 1, 0)])
def test_cost_matrix_matches_oracle(lib, model):
    m = native.PoydCM()
    assert lib.poyd_cm_dna(C.byref(m), *model) == 0
    o = O.cm_dna(*model)
    for f in ("cost", "worst", "prepend", "tail", "median"):
        assert np.array_equal(np.ctypeslib.as_array(getattr(m, f)),
                              np.ctypeslib.as_array(getattr(o, f))), f
    assert (m.cost_model, m.gap_open, m.is_metric) == (o.cost_model, o.gap_open, o.is_metric)


def test_cost_matrix_arbitrary_5x5(lib):
    rng = np.random.default_rng(3)
    for t in range(20):
        mat = rng.integers(0, 6, size=(5, 5)).astype(np.int32)
        if t % 2 == 0:
            mat = np.minimum(mat, mat.T)
            np.fill_diagonal(mat, 0)
        m = native.PoydCM()
        assert lib.poyd_cm_of_matrix5(C.byref(m), mat.ctypes.data, -1) == 0
        o = native.PoydCM()
        O.lib().or_cm_of_matrix5(C.cast(C.byref(o), C.POINTER(O.OrCM)),
                                 mat.ctypes.data_as(O.i32p), -1)
        for f in ("cost", "worst", "median"):
            assert np.array_equal(np.ctypeslib.as_array(getattr(m, f)),
                                  np.ctypeslib.as_array(getattr(o, f))), (t, f)


def test_errors_are_reported_without_a_gpu(lib):
    m = native.PoydCM()
    lib.poyd_cm_dna(C.byref(m), 1, 2, -1)
    m.lcm = 4  # not the DNA combinations alphabet
    rc = lib.poyd_cost_2_batch(C.byref(m), 1, None, None, None, None, None, 0, None, None,
                               None, None)
    assert rc == -5
    assert b"alphabet" in lib.poyd_last_error()


def _dna(lib, gap_open=-1):
    m = native.PoydCM()
    assert lib.poyd_cm_dna(C.byref(m), 1, 2, gap_open) == 0
    return m


def test_argument_checks_without_a_gpu(lib):
    """Checks that return before any CUDA call, with the reference's
    failure cases (failwith in the OCaml stubs) as negative codes."""
    L = C.CDLL(native.LIB_PATH)   # own handle: argtypes set here stay local
    vp, i32 = C.c_void_p, C.c_int32
    cmp = C.POINTER(native.PoydCM)
    L.poyd_algn_simple_2.argtypes = [vp, i32, vp, i32, cmp, vp, i32, vp]
    L.poyd_algn_cost_affine_3.argtypes = [vp, i32, vp, i32, cmp, vp]
    L.poyd_last_error.restype = C.c_char_p
    lin, aff = _dna(lib), _dna(lib, 3)
    s = np.array([16, 1, 2, 4], np.uint8)
    p = s.ctypes.data
    cost = C.c_int32()
    L.poyd_matrix_create.restype = vp
    L.poyd_matrix_free.argtypes = [vp]
    mat = L.poyd_matrix_create()  # host allocation only
    EINVAL, ERANGE, EUNSUP = -1, -3, -5
    # simple_2 wants len(s1) >= len(s2) >= 1, the linear model and a matrix
    assert L.poyd_algn_simple_2(p, 2, p, 3, C.byref(lin), mat, 0, C.byref(cost)) == EINVAL
    assert L.poyd_algn_simple_2(p, 3, p, 0, C.byref(lin), mat, 0, C.byref(cost)) == EINVAL
    assert L.poyd_algn_simple_2(p, 4, p, 4, C.byref(aff), mat, 0, C.byref(cost)) == EINVAL
    assert L.poyd_algn_simple_2(p, 4, p, 4, C.byref(lin), None, 0, C.byref(cost)) == EINVAL
    assert b"null argument" in L.poyd_last_error()
    # the affine entry points want an affine matrix
    assert L.poyd_algn_cost_affine_3(p, 4, p, 4, C.byref(lin), C.byref(cost)) == EINVAL
    assert b"affine" in L.poyd_last_error()
    # matrices the GPU path does not implement, or costs out of range
    bad = _dna(lib)
    bad.tail[1] += 1
    assert L.poyd_algn_cost_affine_3(p, 4, p, 4, C.byref(bad), C.byref(cost)) == EUNSUP
    bad = _dna(lib)
    bad.cost[(1 << 5) | 2] = -1
    assert L.poyd_algn_simple_2(p, 4, p, 4, C.byref(bad), mat, 0, C.byref(cost)) == ERANGE
    bad = _dna(lib)
    bad.cost[(1 << 5) | 2] = 1 << 16
    assert L.poyd_algn_simple_2(p, 4, p, 4, C.byref(bad), mat, 0, C.byref(cost)) == ERANGE
    L.poyd_matrix_free(mat)
    bad = _dna(lib, 3)
    bad.gap_open = 1 << 16
    assert L.poyd_algn_cost_affine_3(p, 4, p, 4, C.byref(bad), C.byref(cost)) == ERANGE
    # host-buffer batch: a null matrix, a negative count or a null buffer
    assert lib.poyd_align_2_host(None, 1, p, None, None, None, None, None, None, 0, None, None,
                                 0) == EINVAL
    assert lib.poyd_align_2_host(C.byref(lin), -1, p, None, None, None, None, None, None, 0,
                                 None, None, 0) == EINVAL
    assert lib.poyd_align_2_host(C.byref(lin), 1, None, None, None, None, None, None, None, 0,
                                 None, None, 0) == EINVAL
    assert lib.poyd_align_2_host(C.byref(lin), 0, None, None, None, None, None, None, None, 0,
                                 None, None, 0) == 0   # an empty batch is a no-op
    # wide Fitch rows: 9 characters of 2 (4) bytes need 32 (48) byte rows
    buf = np.zeros(64, np.uint8)
    b16 = buf.ctypes.data + (-buf.ctypes.data) % 16   # 16-byte aligned inside buf
    assert lib.poyd_nonadd16_distance_batch(C.c_void_p(b16), C.c_int64(16), 9, 1, None, None,
                                            None, None) == EINVAL
    assert lib.poyd_nonadd32_median_batch(C.c_void_p(b16), C.c_int64(32), 9, 1, None, None,
                                          None, None, None) == EINVAL
    assert lib.poyd_nonadd16_median_3_batch(C.c_void_p(b16 + 8), C.c_int64(32), 9, 1, None,
                                            None, None, None, None, None) == EINVAL
    assert lib.poyd_nonadd32_distance_batch(C.c_void_p(b16), C.c_int64(48), 9, 0, None, None,
                                            None, None) == 0   # nothing to do
    # null index arrays or a null distance output with pairs to do
    idx = np.zeros(1, np.int32)
    ip = C.c_void_p(idx.ctypes.data)
    dist = np.zeros(1, np.int64)
    dp = C.c_void_p(dist.ctypes.data)
    v, i64 = C.c_void_p(b16), C.c_int64(16)
    for W in (8, 16, 32):
        dist_f = getattr(lib, "poyd_nonadd%d_distance_batch" % W)
        med_f = getattr(lib, "poyd_nonadd%d_median_batch" % W)
        med3_f = getattr(lib, "poyd_nonadd%d_median_3_batch" % W)
        ln = 16 // (W // 8)
        assert dist_f(v, i64, ln, 1, None, ip, dp, None) == EINVAL
        assert dist_f(v, i64, ln, 1, ip, None, dp, None) == EINVAL
        assert dist_f(v, i64, ln, 1, ip, ip, None, None) == EINVAL
        assert b"null argument" in lib.poyd_last_error()
        assert med_f(v, i64, ln, 1, ip, None, v, None, None) == EINVAL
        assert med3_f(v, i64, ln, 1, ip, ip, None, ip, v, None) == EINVAL
        assert med3_f(v, i64, ln, 1, ip, ip, ip, None, v, None) == EINVAL
    # single-pair column operations: null outputs
    assert lib.poyd_algn_median_2_with_gaps(p, p, 4, C.byref(lin), None, None) == EINVAL
    assert lib.poyd_algn_worst_2(p, p, 4, C.byref(lin), None) == EINVAL


def test_header_matches_exported_list():
    """The header's declarations and the loader's list of entry points
    (native.EXPORTED) are the same set, and every typed signature the
    loader sets up names one of them."""
    assert declared_symbols() == sorted(native.EXPORTED)
    assert {n for n, _, _ in native.SIGNATURES} <= set(native.EXPORTED)


def test_median_levels_argument_checks_without_a_gpu(lib):
    """poyd_median_levels refuses bad level lists, and a pool too small for
    its bound with POYD_ESPACE and the bound, all before any CUDA call."""
    L = C.CDLL(native.LIB_PATH)
    L.poyd_last_error.restype = C.c_char_p
    L.poyd_median_levels.argtypes = [C.POINTER(native.PoydCM), C.POINTER(native.PoydNodeStore),
                                     C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p,
                                     C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.c_void_p,
                                     C.c_void_p]
    cm = _dna(lib)
    store = native.PoydNodeStore(pool=64, pool_size=1 << 20)  # never dereferenced here
    off = np.zeros(8, np.int64)
    ln = np.array([100, 120, 90, 0, 0, 0, 0, 0], np.int32)

    def call(start, a, b, out, size=1 << 20, top=0):
        store.pool_size = size
        st, aa, bb, oo = (np.asarray(x, np.int32) for x in (start, a, b, out))
        t, need = C.c_int64(top), C.c_int64(-1)
        rc = L.poyd_median_levels(C.byref(cm), C.byref(store), 8, off.ctypes.data, ln.ctypes.data,
                                  len(st) - 1, st.ctypes.data, aa.ctypes.data, bb.ctypes.data,
                                  oo.ctypes.data, C.byref(t), C.byref(need), None, None)
        return rc, need.value, L.poyd_last_error()

    EINVAL, ESPACE = -1, -6
    assert call([0, 1], [0], [9], [4])[0] == EINVAL            # id out of range
    assert call([0, 2], [0, 1], [1, 2], [4, 4])[0] == EINVAL   # node 4 written twice
    assert call([0, 2], [0, 4], [1, 2], [4, 5])[0] == EINVAL   # output read in its own level
    assert b"same level" in call([0, 2], [0, 4], [1, 2], [4, 5])[2]
    assert call([0, 1], [0], [3], [4])[0] == EINVAL            # input without a sequence
    assert call([1, 1], [0], [1], [4])[0] == EINVAL            # level_start[0] != 0
    # two levels: 4 = m(0, 1), 5 = m(4, 2); bound slots 4*cap(100,120) and
    # 4*cap(220, 90), each level rounded to 128 bytes, plus 128
    slot = lambda x, y: 4 * ((x + y + 2 + 3) // 4 * 4)
    bound = sum((slot(*p) + 127) // 128 * 128 for p in [(100, 120), (220, 90)]) + 128
    rc, need, msg = call([0, 1, 2], [0, 4], [1, 2], [4, 5], size=1000)
    assert rc == ESPACE and need == bound and b"pool too small" in msg
    assert np.array_equal(ln, [100, 120, 90, 0, 0, 0, 0, 0])   # nothing changed
    assert call([0, 0], [], [], [])[0] == 0                     # no pairs: a no-op


def test_autotune_table_without_a_gpu(lib):
    """The autotuner's kept variants: set, read back, cleared; bad values
    and arguments refused (host tables only)."""
    L = native.lib()
    assert L.poyd_autotune_clear() == 0
    p, b, s = C.c_int32(), C.c_int32(), C.c_int32()
    assert L.poyd_autotune_get(0, 1, 16, 7, C.byref(p), C.byref(b), C.byref(s)) == 0
    assert L.poyd_autotune_set(0, 1, 16, 7, 0, 2, -1) == 0
    assert L.poyd_autotune_get(0, 1, 16, 7, C.byref(p), C.byref(b), C.byref(s)) == 1
    assert (p.value, b.value, s.value) == (0, 2, -1)
    assert L.poyd_autotune_get(0, 0, 16, 7, C.byref(p), C.byref(b), C.byref(s)) == 0  # cost mode
    assert L.poyd_autotune_set(0, 1, 16, 7, 2, 1, 0) == -1     # packed is -1, 0 or 1
    assert L.poyd_autotune_set(0, 1, 16, 7, 1, -1, 0) == -1    # blocks per SM >= 0
    assert L.poyd_autotune_get(0, 1, 16, 7, None, C.byref(b), C.byref(s)) == -1
    assert L.poyd_autotune_clear() == 0
    assert L.poyd_autotune_get(0, 1, 16, 7, C.byref(p), C.byref(b), C.byref(s)) == 0
    # an affine matrix or an empty batch is refused before any CUDA call
    res = native.PoydTuneResult()
    aff = _dna(lib, 3)
    assert L.poyd_autotune_batch(C.byref(aff), 1, 4, None, None, None, None, None, 0, None,
                                 None, None, None, 0, 1, C.byref(res), None) == -5
    lin = _dna(lib)
    assert L.poyd_autotune_batch(C.byref(lin), 1, 0, None, None, None, None, None, 0, None,
                                 None, None, None, 0, 1, C.byref(res), None) == -1


@pytest.mark.parametrize("model", [(1, 2, -1), (1, 1, -1), (2, 1, 3)])
def test_median3_table_matches_oracle(lib, model):
    """poyd_cm_median3 (host code: Three_D.of_two_dim_comb) equals the
    oracle's table for metric DNA matrices."""
    sub, indel, go = model
    cm = native.PoydCM()
    native.check(lib.poyd_cm_dna(C.byref(cm), sub, indel, go))
    tab = np.zeros(32768, np.uint8)
    native.check(lib.poyd_cm_median3(C.byref(cm), tab.ctypes.data))
    assert np.array_equal(tab, O.median3_table(O.cm_dna(sub, indel, go)))


def test_three_sequence_argument_checks_without_a_gpu(lib):
    """The three-sequence entry points refuse bad arguments before any CUDA
    call: a negative count, Powell's parameter rule (ukkCommon.c:130), null
    arrays, a null cost matrix."""
    L = C.CDLL(native.LIB_PATH)
    L.poyd_last_error.restype = C.c_char_p
    vp = C.c_void_p
    L.poyd_powell_3d_batch.argtypes = [C.c_int32] + [vp] * 7 + [C.c_int32] * 3 + [vp] * 5 + [vp]
    L.poyd_readjust_3d_batch.argtypes = [vp, C.c_int32] + [vp] * 15
    d = np.zeros(64, np.uint8)
    p = d.ctypes.data
    assert L.poyd_powell_3d_batch(-1, p, p, p, p, p, p, p, 1, 0, 2, None, p, p, p, p, None) == -1
    assert L.poyd_powell_3d_batch(0, p, p, p, p, p, p, p, 1, 0, 2, None, p, p, p, p, None) == 0
    assert L.poyd_powell_3d_batch(1, p, p, p, p, p, p, p, 0, 0, 2, None, p, p, p, p, None) == -1
    assert b"mm > 0" in L.poyd_last_error()
    assert L.poyd_powell_3d_batch(1, p, p, p, p, p, None, p, 1, 0, 2, None, p, p, p, p, None) == -1
    assert L.poyd_readjust_3d_batch(None, 1, *([p] * 14), None) == -1
    cm = native.PoydCM()
    native.check(lib.poyd_cm_of_matrix5(C.byref(cm), (C.c_int32 * 25)(*([1] * 25)), -1))
    cm.combinations = 0
    assert L.poyd_readjust_3d_batch(C.byref(cm), 1, *([p] * 14), None) == -5


def test_median3_table_non_metric_matches_oracle(lib):
    """poyd_cm_median3 over arbitrary 5x5 matrices (the non-metric ones
    take the gap into a median only where two of the three states hold
    it) equals the oracle's Three_D.of_two_dim_comb."""
    rng = np.random.default_rng(8)
    for t in range(8):
        mat = rng.integers(0, 6, size=(5, 5)).astype(np.int32)
        if t % 2 == 0:
            mat = np.minimum(mat, mat.T)
            np.fill_diagonal(mat, 0)
        m = native.PoydCM()
        assert lib.poyd_cm_of_matrix5(C.byref(m), mat.ctypes.data, -1) == 0
        o = O.OrCM()
        O.lib().or_cm_of_matrix5(C.byref(o), mat.ctypes.data_as(O.i32p), -1)
        assert m.is_metric == o.is_metric
        tab = np.zeros(32768, np.uint8)
        native.check(lib.poyd_cm_median3(C.byref(m), tab.ctypes.data))
        assert np.array_equal(tab, O.median3_table(o)), t
