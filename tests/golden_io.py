"""Reader for tests/golden/dos_golden.npz (made by tests/golden/make_golden.py
from the reference's compiled C kernels)."""
import os

import numpy as np

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "dos_golden.npz")
LINEAR = [(1, 2), (1, 1), (3, 1)]
AFFINE = [(2, 1, 1), (3, 1, 5), (1, 2, 3)]


def unpack(data, lens):
    out, o = [], 0
    for n in lens:
        out.append(data[o:o + n])
        o += n
    return out


def load():
    z = np.load(PATH)
    g = {k: z[k] for k in z.files}
    g["A"] = unpack(g["a_data"], g["a_len"])
    g["B"] = unpack(g["b_data"], g["b_len"])
    return g


def seqs(g, key):
    return unpack(g[key], g[key + "_len"])
