"""Generates tests/golden/dos_golden.npz from the REFERENCE's own compiled C
kernels (oracle/_ref/libporef.so, built by oracle/build_ref.sh from the
reference sources).  The deltaw policy and cost-matrix tables (OCaml in the
reference) come from the oracle's restatement; every DP output below is the
reference C code's.

Run where the reference sources are present:
    python tests/golden/make_golden.py
"""
import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402
from poyd_gb300 import synth  # noqa: E402

LINEAR = [(1, 2), (1, 1), (3, 1)]
AFFINE = [(2, 1, 1), (3, 1, 5), (1, 2, 3)]


def P(a):
    return a.ctypes.data_as(O.u8p)


def pairs():
    rng = np.random.default_rng(2024)
    A, B = synth.pair_batch(99, 30, lmin=1, lmax=420)
    g = synth.with_gap
    for n1, n2 in [(0, 0), (0, 7), (3, 0), (1, 1), (60, 140), (140, 60), (33, 31), (250, 90)]:
        A.append(g(synth.random_dna(rng, n1, 0.1)))
        B.append(g(synth.random_dna(rng, n2, 0.1)))
    a = synth.random_dna(rng, 200)
    b = a.copy()
    b[::9] = 16
    A.append(g(a))
    B.append(g(b))
    return A, B


def pack(list_of_arrays):
    lens = np.array([len(x) for x in list_of_arrays], np.int32)
    data = np.concatenate(list_of_arrays) if len(list_of_arrays) else np.zeros(0, np.uint8)
    return data.astype(np.uint8), lens


def main():
    O.build_ref()
    R = O.ref()
    assert R is not None, "compiled reference not available"
    A, B = pairs()
    out = {}
    out["a_data"], out["a_len"] = pack(A)
    out["b_data"], out["b_len"] = pack(B)
    for model in LINEAR:
        m = O.cm_dna(model[0], model[1], -1)
        rc = R.ref_cm_new(C.byref(m))
        tag = "lin_%d_%d" % model
        costs, costs_dos, al_a, al_b, anc, mwg = [], [], [], [], [], []
        for a, b in zip(A, B):
            for explicit, sink in ((None, costs), (max(abs(len(a) - len(b)), 8), costs_dos)):
                dw = O.deltaw(a, b, m, explicit)
                if len(a) >= len(b):
                    sink.append(R.ref_simple_2(P(a), len(a), P(b), len(b), rc, dw))
                else:
                    sink.append(R.ref_simple_2(P(b), len(b), P(a), len(a), rc, dw))
            dw = O.deltaw(a, b, m)
            cap = len(a) + len(b) + 2
            o1, o2 = np.zeros(cap, np.uint8), np.zeros(cap, np.uint8)
            n = C.c_int()
            R.ref_align_2(P(a), len(a), P(b), len(b), rc, dw, P(o1), P(o2), C.byref(n))
            ra, rb = o1[:n.value].copy(), o2[:n.value].copy()
            al_a.append(ra)
            al_b.append(rb)
            t = np.zeros(len(ra) + 2, np.uint8)
            k = R.ref_ancestor_2(P(ra), P(rb), len(ra), rc, P(t))
            anc.append(t[:k].copy())
            k = R.ref_median_2_with_gaps(P(ra), P(rb), len(ra), rc, P(t))
            mwg.append(t[:k].copy())
        out[tag + "_cost"] = np.array(costs, np.int32)
        out[tag + "_cost_dos"] = np.array(costs_dos, np.int32)
        for nm, lst in (("al_a", al_a), ("al_b", al_b), ("anc", anc), ("mwg", mwg)):
            out[tag + "_" + nm], out[tag + "_" + nm + "_len"] = pack(lst)
        R.ref_cm_free(rc)
    for model in AFFINE:
        m = O.cm_dna(*model)
        rc = R.ref_cm_new(C.byref(m))
        tag = "aff_%d_%d_%d" % model
        cost_nobt, cost_bt, med, mwg, ri, rj = [], [], [], [], [], []
        for a, b in zip(A, B):
            cost_nobt.append(R.ref_cost_affine_3(P(a), len(a), P(b), len(b), rc))
            cap = len(a) + len(b) + 3
            bufs = [np.zeros(cap, np.uint8) for _ in range(4)]
            lm, lw, lr = C.c_int(), C.c_int(), C.c_int()
            cost_bt.append(R.ref_align_affine_3(P(a), len(a), P(b), len(b), rc, P(bufs[0]),
                                                C.byref(lm), P(bufs[1]), C.byref(lw),
                                                P(bufs[2]), P(bufs[3]), C.byref(lr)))
            med.append(bufs[0][:lm.value].copy())
            mwg.append(bufs[1][:lw.value].copy())
            ri.append(bufs[2][:lr.value].copy())
            rj.append(bufs[3][:lr.value].copy())
        out[tag + "_cost"] = np.array(cost_nobt, np.int32)
        out[tag + "_cost_bt"] = np.array(cost_bt, np.int32)
        for nm, lst in (("median", med), ("mwg", mwg), ("resi", ri), ("resj", rj)):
            out[tag + "_" + nm], out[tag + "_" + nm + "_len"] = pack(lst)
        R.ref_cm_free(rc)
    # Fitch (NonaddCS8) vectors
    rng = np.random.default_rng(7)
    L = 2000
    nodes = rng.integers(1, 256, size=(6, L)).astype(np.uint8)
    nodes[:, ::3] = (1 << rng.integers(0, 8, size=(6, (L + 2) // 3))).astype(np.uint8)
    out["fitch_nodes"] = nodes
    med = np.zeros(L, np.uint8)
    out["fitch_cost01"] = np.array([R.ref_nonadd8_median(P(nodes[0]), P(nodes[1]), L, P(med))])
    out["fitch_median01"] = med.copy()
    out["fitch_dist"] = np.array([[R.ref_nonadd8_distance(P(nodes[i]), P(nodes[j]), L)
                                   for j in range(6)] for i in range(6)], np.int64)
    F = np.zeros(L, np.uint8)
    R.ref_nonadd8_median_3(P(nodes[2]), P(nodes[3]), P(nodes[4]), P(nodes[5]), L, P(F))
    out["fitch_median3"] = F
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "dos_golden.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
