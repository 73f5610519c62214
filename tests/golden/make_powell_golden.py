"""Generates tests/golden/powell_golden.npz from the REFERENCE's own compiled
powell_3D_align (ukkCommon.c, ukk.checkp.c in oracle/_ref/libporef.so, built
by oracle/build_ref.sh from the reference sources): seeded triples, the
reference's costs and its aligned rows, for three (mm, go, ge) settings.

Run where the reference sources are present:
    python tests/golden/make_powell_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402
from poyd_gb300 import synth  # noqa: E402

# (mm, go, ge): DNA sub 1 / indel 2 linear, sub 1 / indel 1 with opening 2,
# sub 2 / indel 1 with opening 3
PARAMS = [(1, 0, 2), (1, 2, 1), (2, 3, 1)]


def triples():
    T = synth.triple_batch(77, 60, lmin=0, lmax=160)
    T += synth.triple_batch(78, 12, lmin=0, lmax=12, sub=(0.3, 0.6), indel=(0.1, 0.3))
    g = synth.with_gap
    rng = np.random.default_rng(5)
    for n in [(0, 0, 0), (0, 0, 5), (4, 0, 0), (0, 3, 0), (1, 1, 1), (30, 2, 30), (90, 40, 60)]:
        T.append(tuple(g(synth.random_dna(rng, k, 0.05)) for k in n))
    return T


def pack(arrs):
    lens = np.array([len(x) for x in arrs], np.int32)
    data = np.concatenate(arrs).astype(np.uint8) if arrs else np.zeros(0, np.uint8)
    return data, lens


def main():
    O.build_ref()
    assert O.ref() is not None, "compiled reference not available"
    T = triples()
    out = {}
    for q, name in enumerate("abc"):
        out[name + "_data"], out[name + "_len"] = pack([t[q] for t in T])
    for mm, go, ge in PARAMS:
        key = "%d_%d_%d" % (mm, go, ge)
        costs, rows = [], [[], [], []]
        for t in T:
            c, ra, rb, rc = O.powell_3d(*t, mm, go, ge, reference=True)
            costs.append(c)
            for q, r in enumerate((ra, rb, rc)):
                rows[q].append(r)
        out["cost_" + key] = np.array(costs, np.int32)
        for q, name in enumerate("abc"):
            out["al%s_%s_data" % (name, key)], out["al%s_%s_len" % (name, key)] = pack(rows[q])
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "powell_golden.npz")
    np.savez_compressed(path, **out)
    print(path, len(T), "triples", os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
