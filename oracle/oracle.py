"""ctypes bindings for the CPU oracle (TEST INFRASTRUCTURE ONLY).

Two libraries live here:

* ``_build/liboracle.so`` -- the plain-C restatement of the reference's
  scoring path (``poy_oracle.c``), built by ``build_oracle.sh``;
* ``_ref/libporef.so`` -- the reference's own ``algn.c``, ``ukkCommon.c`` /
  ``ukk.checkp.c`` and ``nonaddCSc.c`` compiled from source by
  ``build_ref.sh`` where the sources are available.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU arms use this
module, and only to check or time against the CUDA path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libporef.so")

u8p = C.POINTER(C.c_uint8)
i32p = C.POINTER(C.c_int32)
i64p = C.POINTER(C.c_int64)


class OrCM(C.Structure):
    """Mirror of ``or_cm`` (poy_oracle.h)."""

    _fields_ = [
        ("lcm", C.c_int32), ("gap", C.c_int32), ("a_sz", C.c_int32),
        ("combinations", C.c_int32), ("cost_model", C.c_int32),
        ("gap_open", C.c_int32), ("is_metric", C.c_int32),
        ("all_elements", C.c_int32),
        ("cost", C.c_int32 * 1024), ("worst", C.c_int32 * 1024),
        ("prepend", C.c_int32 * 32), ("tail", C.c_int32 * 32),
        ("median", C.c_uint8 * 1024),
    ]


class OrResultSet(C.Structure):
    """Mirror of ``or_result_set`` (poy_oracle.h): host copies of a batched
    align_2 result (costs, slot bytes, slot offsets, lengths)."""

    _fields_ = [("cost", C.c_void_p), ("out", C.c_void_p), ("off", C.c_void_p),
                ("len", C.c_void_p)]


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB_PATH):
        subprocess.check_call(["sh", os.path.join(HERE, "build_oracle.sh")],
                              stdout=subprocess.DEVNULL)
    return LIB_PATH


def build_ref(src_dir: str | None = None, env: dict | None = None) -> str | None:
    """Compile the reference C kernels when their sources are present
    (build_ref.sh finds them: `src_dir`, else POYD_REFERENCE_SRC, else the
    recipe's default location).  Returns the library path, or None where
    the sources are absent."""
    cmd = ["sh", os.path.join(HERE, "build_ref.sh")] + ([src_dir] if src_dir else [])
    r = subprocess.run(cmd, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, text=True,
                       env=env)
    if r.returncode == 2:  # the recipe's "sources not found"
        return None
    if r.returncode:
        raise RuntimeError("build_ref.sh failed: " + r.stderr[-2000:])
    return REF_PATH


_lib = None
_ref = None


def _ptr(a, t=u8p):
    return a.ctypes.data_as(t)


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.or_cm_dna.argtypes = [C.POINTER(OrCM), C.c_int, C.c_int, C.c_int]
        L.or_cm_of_matrix5.argtypes = [C.POINTER(OrCM), i32p, C.c_int]
        L.or_cost2_deltaw.argtypes = [u8p, C.c_int, u8p, C.c_int, C.c_int, C.c_int, C.c_int]
        L.or_simple_2.argtypes = [u8p, C.c_int, u8p, C.c_int, C.POINTER(OrCM), C.c_int,
                                  C.POINTER(C.c_uint16)]
        L.or_band_cells_linear.argtypes = [C.c_int, C.c_int, C.c_int]
        L.or_band_cells_linear.restype = C.c_int64
        L.or_band_cells_affine.argtypes = [C.c_int, C.c_int]
        L.or_band_cells_affine.restype = C.c_int64
        L.or_align_2.argtypes = [u8p, C.c_int, u8p, C.c_int, C.POINTER(OrCM), u8p, u8p,
                                 C.POINTER(C.c_int)]
        L.or_cost_2.argtypes = [u8p, C.c_int, u8p, C.c_int, C.POINTER(OrCM), C.c_int, C.c_int]
        for n in ("or_median_2_with_gaps", "or_median_2_no_gaps", "or_ancestor_2"):
            getattr(L, n).argtypes = [u8p, u8p, C.c_int, C.POINTER(OrCM), u8p]
        for n in ("or_worst_2", "or_verify_2"):
            getattr(L, n).argtypes = [u8p, u8p, C.c_int, C.POINTER(OrCM)]
        L.or_cost_affine_3.argtypes = [u8p, C.c_int, u8p, C.c_int, C.POINTER(OrCM)]
        L.or_align_affine_3.argtypes = [u8p, C.c_int, u8p, C.c_int, C.POINTER(OrCM), u8p,
                                        C.POINTER(C.c_int), u8p, C.POINTER(C.c_int), u8p, u8p,
                                        C.POINTER(C.c_int)]
        L.or_dos_median.argtypes = [u8p, C.c_int, u8p, C.c_int, C.POINTER(OrCM), u8p,
                                    C.POINTER(C.c_int), u8p, u8p, u8p, C.POINTER(C.c_int)]
        L.or_closest.argtypes = [u8p, C.c_int, u8p, C.c_int, C.POINTER(OrCM), C.c_int, u8p]
        L.or_dos_median_many.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_int, C.POINTER(OrCM),
                                         C.c_void_p]
        L.or_dos_median_many.restype = C.c_int64
        L.or_dos_median_check_many.argtypes = [C.c_void_p] * 6 + [C.c_int, C.POINTER(OrCM),
                                                                  C.c_void_p, C.c_int,
                                                                  C.c_void_p, C.c_void_p]
        L.or_dos_median_check_many.restype = C.c_int64
        L.or_candidate_scores.argtypes = [C.c_void_p] * 4 + [C.c_int, C.c_void_p, C.c_int, C.c_int,
                                                             C.c_void_p, C.c_void_p, C.c_void_p,
                                                             C.c_int, C.POINTER(OrCM), C.c_void_p]
        L.or_nonadd_median.argtypes = [u8p, u8p, C.c_int, u8p]
        L.or_nonadd_median.restype = C.c_int64
        L.or_nonadd_distance.argtypes = [u8p, u8p, C.c_int]
        L.or_nonadd_distance.restype = C.c_int64
        L.or_nonadd_median_3.argtypes = [u8p, u8p, u8p, u8p, C.c_int, u8p]
        L.or_nonadd_dist_2.argtypes = [u8p, u8p, u8p, C.c_int]
        L.or_nonadd_dist_2.restype = C.c_int64
        for w in (16, 32):
            getattr(L, "or_nonadd%d_median" % w).argtypes = [C.c_void_p] * 2 + [C.c_int, C.c_void_p]
            getattr(L, "or_nonadd%d_median" % w).restype = C.c_int64
            getattr(L, "or_nonadd%d_distance" % w).argtypes = [C.c_void_p] * 2 + [C.c_int]
            getattr(L, "or_nonadd%d_distance" % w).restype = C.c_int64
            getattr(L, "or_nonadd%d_median_3" % w).argtypes = [C.c_void_p] * 4 + [C.c_int, C.c_void_p]
        L.or_sank_elt_median.argtypes = [C.c_int, i64p, i64p, i64p, i64p, i64p, i64p]
        L.or_sank_elt_distance.argtypes = [C.c_int, i64p, i64p, i64p]
        L.or_sank_elt_median_3.argtypes = [C.c_int, i64p, i64p, i64p, C.c_uint32, i64p, i64p,
                                           i64p, i64p, C.POINTER(C.c_uint32)]
        L.or_sank_elt_distance.restype = C.c_double
        L.or_powell_3d.argtypes = [u8p, C.c_int, u8p, C.c_int, u8p, C.c_int, C.c_int, C.c_int,
                                   C.c_int, u8p, u8p, u8p, C.POINTER(C.c_int)]
        L.or_powell_alignment_cost.argtypes = [u8p, u8p, u8p, C.c_int, C.c_int, C.c_int, C.c_int]
        L.or_median3_table.argtypes = [C.POINTER(OrCM), u8p]
        L.or_readjust_3d.argtypes = [u8p, C.c_int, u8p, C.c_int, u8p, C.c_int, u8p, C.c_int,
                                     C.POINTER(OrCM), u8p, u8p, C.POINTER(C.c_int),
                                     C.POINTER(C.c_int)]
        _lib = L
    return _lib


def ref():
    """The compiled reference, or None when it is not built here."""
    global _ref
    if _ref is None and os.path.exists(REF_PATH):
        R = C.CDLL(REF_PATH)
        R.ref_cm_new.argtypes = [C.POINTER(OrCM)]
        R.ref_cm_new.restype = C.c_void_p
        R.ref_cm_free.argtypes = [C.c_void_p]
        R.ref_simple_2.argtypes = [u8p, C.c_int, u8p, C.c_int, C.c_void_p, C.c_int]
        R.ref_align_2.argtypes = [u8p, C.c_int, u8p, C.c_int, C.c_void_p, C.c_int, u8p, u8p,
                                  C.POINTER(C.c_int)]
        R.ref_cost_affine_3.argtypes = [u8p, C.c_int, u8p, C.c_int, C.c_void_p]
        R.ref_align_affine_3.argtypes = [u8p, C.c_int, u8p, C.c_int, C.c_void_p, u8p,
                                         C.POINTER(C.c_int), u8p, C.POINTER(C.c_int), u8p, u8p,
                                         C.POINTER(C.c_int)]
        for n in ("ref_ancestor_2", "ref_median_2_with_gaps", "ref_median_2_no_gaps"):
            getattr(R, n).argtypes = [u8p, u8p, C.c_int, C.c_void_p, u8p]
        for n in ("ref_worst_2", "ref_verify_2"):
            getattr(R, n).argtypes = [u8p, u8p, C.c_int, C.c_void_p]
        R.ref_nonadd8_median.argtypes = [u8p, u8p, C.c_int, u8p]
        R.ref_nonadd8_median.restype = C.c_long
        R.ref_nonadd8_distance.argtypes = [u8p, u8p, C.c_int]
        R.ref_nonadd8_distance.restype = C.c_long
        R.ref_nonadd8_median_3.argtypes = [u8p, u8p, u8p, u8p, C.c_int, u8p]
        R.ref_nonadd8_dist_2.argtypes = [u8p, u8p, u8p, C.c_int]
        R.ref_nonadd8_dist_2.restype = C.c_long
        for w in (16, 32):
            getattr(R, "ref_nonadd%d_median" % w).argtypes = [C.c_void_p] * 2 + [C.c_int, C.c_void_p]
            getattr(R, "ref_nonadd%d_median" % w).restype = C.c_long
            getattr(R, "ref_nonadd%d_distance" % w).argtypes = [C.c_void_p] * 2 + [C.c_int]
            getattr(R, "ref_nonadd%d_distance" % w).restype = C.c_long
            getattr(R, "ref_nonadd%d_median_3" % w).argtypes = [C.c_void_p] * 4 + [C.c_int, C.c_void_p]
        R.ref_powell_3d.argtypes = [u8p, C.c_int, u8p, C.c_int, u8p, C.c_int, C.c_int, C.c_int,
                                    C.c_int, u8p, u8p, u8p, C.POINTER(C.c_int)]
        _ref = R
    return _ref


# --------------------------------------------------------------------------
# Pythonic wrappers over the restatement
# --------------------------------------------------------------------------

def cm_dna(sub: int = 1, indel: int = 2, gap_open: int = -1) -> OrCM:
    m = OrCM()
    lib().or_cm_dna(C.byref(m), sub, indel, gap_open)
    return m


def cm_tables(m: OrCM) -> dict:
    return {
        "cost": np.ctypeslib.as_array(m.cost).copy(),
        "worst": np.ctypeslib.as_array(m.worst).copy(),
        "prepend": np.ctypeslib.as_array(m.prepend).copy(),
        "tail": np.ctypeslib.as_array(m.tail).copy(),
        "median": np.ctypeslib.as_array(m.median).copy(),
        "cost_model": m.cost_model, "gap_open": m.gap_open, "gap": m.gap,
    }


def _u8(x):
    return np.ascontiguousarray(x, dtype=np.uint8)


def deltaw(a, b, m: OrCM, explicit: int | None = None) -> int:
    a, b = _u8(a), _u8(b)
    if len(a) >= len(b):
        s1, s2 = a, b
    else:
        s1, s2 = b, a
    return lib().or_cost2_deltaw(_ptr(s1), len(s1), _ptr(s2), len(s2), m.gap,
                                 0 if explicit is None else 1, explicit or 0)


def cost_2(a, b, m: OrCM, explicit_deltaw: int | None = None) -> int:
    a, b = _u8(a), _u8(b)
    return lib().or_cost_2(_ptr(a), len(a), _ptr(b), len(b), C.byref(m),
                           0 if explicit_deltaw is None else 1, explicit_deltaw or 0)


def simple_2(s1, s2, m: OrCM, dw: int, want_dm: bool = False):
    s1, s2 = _u8(s1), _u8(s2)
    dm = np.zeros(len(s1) * len(s2), dtype=np.uint16) if want_dm else None
    c = lib().or_simple_2(_ptr(s1), len(s1), _ptr(s2), len(s2), C.byref(m), dw,
                          dm.ctypes.data_as(C.POINTER(C.c_uint16)) if want_dm else None)
    return (c, dm) if want_dm else c


def band_cells_linear(l1: int, l2: int, dw: int) -> int:
    return lib().or_band_cells_linear(max(l1, l2), min(l1, l2), dw)


def band_cells_affine(l1: int, l2: int) -> int:
    return lib().or_band_cells_affine(l1, l2)


def align_2(a, b, m: OrCM):
    a, b = _u8(a), _u8(b)
    ra = np.zeros(len(a) + len(b) + 2, np.uint8)
    rb = np.zeros_like(ra)
    n = C.c_int()
    c = lib().or_align_2(_ptr(a), len(a), _ptr(b), len(b), C.byref(m), _ptr(ra), _ptr(rb),
                         C.byref(n))
    return c, ra[:n.value].copy(), rb[:n.value].copy()


def _pair_fn(name, a, b, m, extra=1):
    a, b = _u8(a), _u8(b)
    out = np.zeros(len(a) + extra + 1, np.uint8)
    n = getattr(lib(), name)(_ptr(a), _ptr(b), len(a), C.byref(m), _ptr(out))
    return out[:n].copy()


def median_2_with_gaps(a, b, m):
    return _pair_fn("or_median_2_with_gaps", a, b, m)


def median_2(a, b, m):
    return _pair_fn("or_median_2_no_gaps", a, b, m)


def ancestor_2(a, b, m):
    return _pair_fn("or_ancestor_2", a, b, m)


def worst_2(a, b, m):
    a, b = _u8(a), _u8(b)
    return lib().or_worst_2(_ptr(a), _ptr(b), len(a), C.byref(m))


def verify_2(a, b, m):
    a, b = _u8(a), _u8(b)
    return lib().or_verify_2(_ptr(a), _ptr(b), len(a), C.byref(m))


def cost_affine_3(a, b, m):
    a, b = _u8(a), _u8(b)
    return lib().or_cost_affine_3(_ptr(a), len(a), _ptr(b), len(b), C.byref(m))


def align_affine_3(a, b, m):
    a, b = _u8(a), _u8(b)
    cap = len(a) + len(b) + 2
    med, mwg, ri, rj = (np.zeros(cap + 1, np.uint8) for _ in range(4))
    lm, lw, lr = C.c_int(), C.c_int(), C.c_int()
    c = lib().or_align_affine_3(_ptr(a), len(a), _ptr(b), len(b), C.byref(m), _ptr(med),
                                C.byref(lm), _ptr(mwg), C.byref(lw), _ptr(ri), _ptr(rj),
                                C.byref(lr))
    return (c, med[:lm.value].copy(), mwg[:lw.value].copy(), ri[:lr.value].copy(),
            rj[:lr.value].copy())


def dos_median(a, b, m):
    """DOS.median: (cost, median, aligned a, aligned b, median with gaps)."""
    a, b = _u8(a), _u8(b)
    cap = len(a) + len(b) + 2
    sm, ra, rb, wg = (np.zeros(cap + 1, np.uint8) for _ in range(4))
    lm, la = C.c_int(), C.c_int()
    c = lib().or_dos_median(_ptr(a), len(a), _ptr(b), len(b), C.byref(m), _ptr(sm),
                            C.byref(lm), _ptr(ra), _ptr(rb), _ptr(wg), C.byref(la))
    return (c, sm[:lm.value].copy(), ra[:la.value].copy(), rb[:la.value].copy(),
            wg[:la.value].copy())


def closest(parent, mine, m, dos_empty: bool = True):
    """DOS.to_single (dos_empty) / Sequence.Align.closest: the single
    sequence of `mine` given its parent's single sequence."""
    p, s = _u8(parent), _u8(mine)
    out = np.zeros(len(p) + len(s) + 2, np.uint8)
    n = lib().or_closest(_ptr(p), len(p), _ptr(s), len(s), C.byref(m), int(dos_empty), _ptr(out))
    if n < 0:
        raise ValueError("closest: a column of `mine` has no states")
    return out[:n].copy()


def powell_3d(a, b, c, mm, go, ge, reference=False):
    """powell_3D_align (ukkCommon.c:111-143) on three sequences with their
    leading gap: (cost, aligned a, aligned b, aligned c).  reference=True
    runs the compiled reference instead of the restatement."""
    a, b, c = _u8(a), _u8(b), _u8(c)
    cap = len(a) + len(b) + len(c)
    oa, ob, oc = (np.zeros(cap, np.uint8) for _ in range(3))
    n = C.c_int()
    f = ref().ref_powell_3d if reference else lib().or_powell_3d
    cost = f(_ptr(a), len(a), _ptr(b), len(b), _ptr(c), len(c), mm, go, ge, _ptr(oa), _ptr(ob),
             _ptr(oc), C.byref(n))
    if cost < 0:
        raise ValueError("powell_3d: an element holds none of A, C, G, T")
    k = n.value
    return cost, oa[:k].copy(), ob[:k].copy(), oc[:k].copy()


def powell_alignment_cost(a, b, c, mm, go, ge):
    """The least alignmentCost (ukkCommon.c:345-391) of aligned rows."""
    a, b, c = _u8(a), _u8(b), _u8(c)
    return lib().or_powell_alignment_cost(_ptr(a), _ptr(b), _ptr(c), len(a), mm, go, ge)


def median3_table(m):
    """Cost_matrix.Three_D.of_two_dim_comb medians, indexed (i<<10)|(j<<5)|k."""
    t = np.zeros(32768, np.uint8)
    lib().or_median3_table(C.byref(m), _ptr(t))
    return t


def readjust_3d(s1, s2, cur, p, m, tab3=None):
    """Sequence.Align.readjust_3d s1 s2 cur cm cm3 p: (cost, new median,
    changed)."""
    s1, s2, cur, p = _u8(s1), _u8(s2), _u8(cur), _u8(p)
    if tab3 is None:
        tab3 = median3_table(m)
    res = np.zeros(len(s1) + len(s2) + len(p) + len(cur) + 1, np.uint8)
    lr, ch = C.c_int(), C.c_int()
    cost = lib().or_readjust_3d(_ptr(s1), len(s1), _ptr(s2), len(s2), _ptr(cur), len(cur),
                                _ptr(p), len(p), C.byref(m), _ptr(tab3), _ptr(res), C.byref(lr),
                                C.byref(ch))
    if cost < 0:
        raise ValueError("readjust_3d: an element holds none of A, C, G, T")
    return cost, res[:lr.value].copy(), bool(ch.value)


def select_one(s, m):
    """Sequence.select_one (sequence.ml:1143-1156): every element becomes its
    lowest state (combination alphabets; list_of_bits, cost_matrix.ml:206-217,
    sorted ascending)."""
    s = _u8(s)
    if not m.combinations:
        return s.copy()
    if np.any(s == 0):
        raise ValueError("select_one: an element with no states")
    return (s & ((-s.astype(np.int16)) & 0xFF).astype(np.uint8)).astype(np.uint8)


def algn_median(s1, s2, m):
    """The `algn` of Sequence.readjust / DOS.readjust (sequence.ml:1168-1178,
    seqCS.ml:684-698) before select_one: (cost, median); linear: align_2 then
    median_2 (algn_CAML_median_2_no_gaps); affine: align_affine_3's median."""
    if m.cost_model == 1:
        c, med, _mwg, _ri, _rj = align_affine_3(s1, s2, m)
        return c, med
    c, ra, rb = align_2(s1, s2, m)
    return c, median_2(ra, rb, m)


def seq_readjust(a, b, parent, m):
    """Sequence.readjust a b m cm parent, ApproxD mode (sequence.ml:1166-1195):
    the three pairwise medians, each aligned with the third sequence; the
    cheapest centre's median made closest to the third (Align.closest,
    sequence.ml:967-1033).  Returns (cost, sequence)."""
    c = parent
    cab, ab = algn_median(a, b, m)
    cbc, bc = algn_median(b, c, m)
    cac, ac = algn_median(a, c, m)
    cabc = algn_median(ab, c, m)[0] + cab
    cbca = algn_median(bc, a, m)[0] + cbc
    cacb = algn_median(ac, b, m)[0] + cac
    if cabc <= cbca:
        if cabc <= cacb:
            return cabc, closest(c, ab, m, dos_empty=False)
        return cacb, closest(b, ac, m, dos_empty=False)
    if cbca < cacb:
        return cbca, closest(a, bc, m, dos_empty=False)
    return cacb, closest(b, ac, m, dos_empty=False)


def dos_readjust(mode, ch1, ch2, parent, mine, m, tab3=None):
    """DOS.readjust (seqCS.ml:680-722) of one DO character: mode "three"
    (Iterative ThreeD: Sequence.Align.readjust_3d) or "approx" (ApproxD:
    Sequence.readjust), with the rules for empty neighbours.  Returns
    (changed, new sequence, cost); changed is `0 <> compare res mine`."""
    ch1, ch2, parent, mine = _u8(ch1), _u8(ch2), _u8(parent), _u8(mine)
    gap = m.gap
    e1, e2, ep = (bool(np.all(x == gap)) for x in (ch1, ch2, parent))
    if not (e1 or e2 or ep):
        if mode == "three":
            cost, res, _ = readjust_3d(ch1, ch2, mine, parent, m, tab3)
        else:
            cost, res = seq_readjust(ch1, ch2, parent, m)
    elif e1 and e2:
        cost, res = 0, ch1.copy()
    elif e1 and ep:
        cost, res = 0, ch1.copy()
    elif e2 and ep:
        cost, res = 0, ch2.copy()
    else:
        x, y = (ch1, ch2) if ep else (ch1, parent) if e2 else (ch2, parent)
        cost, med = algn_median(x, y, m)
        res = select_one(med, m)
    changed = not (len(res) == len(mine) and np.array_equal(res, mine))
    return changed, res, int(cost)


def nonadd_median(a, b):
    a, b = _u8(a), _u8(b)
    r = np.zeros(len(a), np.uint8)
    c = lib().or_nonadd_median(_ptr(a), _ptr(b), len(a), _ptr(r))
    return c, r


def nonadd_distance(a, b):
    a, b = _u8(a), _u8(b)
    return lib().or_nonadd_distance(_ptr(a), _ptr(b), len(a))


def nonadd_dist_2(a, b, c) -> int:
    """char_nonadd_CAML_dist_2: characters where a meets neither b nor c."""
    a, b, c = _u8(a), _u8(b), _u8(c)
    return int(lib().or_nonadd_dist_2(_ptr(a), _ptr(b), _ptr(c), len(a)))


def nonadd_median_3(A, N, D1, D2):
    A, N, D1, D2 = (_u8(x) for x in (A, N, D1, D2))
    F = np.zeros(len(A), np.uint8)
    lib().or_nonadd_median_3(_ptr(A), _ptr(N), _ptr(D1), _ptr(D2), len(A), _ptr(F))
    return F


SANK_INF = ((1 << 62) - 1) // 4


_WIDE = {8: np.uint8, 16: np.uint16, 32: np.uint32}


def _wide(x, width):
    return np.ascontiguousarray(x, dtype=_WIDE[width])


def nonadd_median_w(a, b, width: int):
    """Fitch median of width-bit state sets (NonaddCS8/16/32): (added
    cost, median)."""
    if width == 8:
        return nonadd_median(a, b)
    a, b = _wide(a, width), _wide(b, width)
    res = np.zeros_like(a)
    c = getattr(lib(), "or_nonadd%d_median" % width)(a.ctypes.data, b.ctypes.data, len(a),
                                                     res.ctypes.data)
    return int(c), res


def nonadd_distance_w(a, b, width: int) -> int:
    if width == 8:
        return nonadd_distance(a, b)
    a, b = _wide(a, width), _wide(b, width)
    return int(getattr(lib(), "or_nonadd%d_distance" % width)(a.ctypes.data, b.ctypes.data, len(a)))


def nonadd_median_3_w(A, N, D1, D2, width: int):
    if width == 8:
        return nonadd_median_3(A, N, D1, D2)
    A, N, D1, D2 = (_wide(x, width) for x in (A, N, D1, D2))
    F = np.zeros_like(A)
    getattr(lib(), "or_nonadd%d_median_3" % width)(A.ctypes.data, N.ctypes.data, D1.ctypes.data,
                                                   D2.ctypes.data, len(A), F.ctypes.data)
    return F


def sank_elt_median(tcm, a_s, b_s):
    tcm = np.ascontiguousarray(tcm, np.int64)
    a_s = np.ascontiguousarray(a_s, np.int64)
    b_s = np.ascontiguousarray(b_s, np.int64)
    k = len(a_s)
    c, e, beta = (np.zeros(k, np.int64) for _ in range(3))
    lib().or_sank_elt_median(k, _ptr(tcm, i64p), _ptr(a_s, i64p), _ptr(b_s, i64p),
                             _ptr(c, i64p), _ptr(e, i64p), _ptr(beta, i64p))
    return c, e, beta


def sank_elt_median_3(tcm, a_s, a_e, a_best, n_s, l_s, r_s):
    """elt_median_3: (final e, best-state bits) of a node from its
    ancestor's final (a_e, a_best bits; 0 = the cheapest states of a_s), its
    preliminary s and its children's preliminary s."""
    tcm = np.ascontiguousarray(tcm, np.int64)
    a_s, a_e, n_s, l_s, r_s = (np.ascontiguousarray(x, np.int64) for x in (a_s, a_e, n_s, l_s, r_s))
    k = len(n_s)
    e = np.zeros(k, np.int64)
    best = C.c_uint32()
    lib().or_sank_elt_median_3(k, _ptr(tcm, i64p), _ptr(a_s, i64p), _ptr(a_e, i64p),
                               int(a_best), _ptr(n_s, i64p), _ptr(l_s, i64p), _ptr(r_s, i64p),
                               _ptr(e, i64p), C.byref(best))
    return e, int(best.value)


def sank_elt_distance(tcm, a_s, b_s):
    tcm = np.ascontiguousarray(tcm, np.int64)
    a_s = np.ascontiguousarray(a_s, np.int64)
    b_s = np.ascontiguousarray(b_s, np.int64)
    return lib().or_sank_elt_distance(len(a_s), _ptr(tcm, i64p), _ptr(a_s, i64p),
                                      _ptr(b_s, i64p))
