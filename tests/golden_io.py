"""Readers for the golden fixtures: tests/golden/dos_golden.npz (made by
tests/golden/make_golden.py from the reference's compiled C kernels) and
tests/golden/tree_golden.tar.gz (the reference's tree-level test inputs,
packed by tests/golden/make_tree_golden.py)."""
import os
import tarfile
import tempfile

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


TREE_ARCHIVE = os.path.join(os.path.dirname(PATH), "tree_golden.tar.gz")
_tree_dir = None


def tree_golden_dir() -> str:
    """A directory holding the reference's tree-level test inputs (1.fas ..
    13.fas, their trees, cc*/cnc*.costs, polymorphic.ss, cost_tests),
    extracted once per process."""
    global _tree_dir
    if _tree_dir is None:
        d = tempfile.mkdtemp(prefix="poyd_tree_golden_")
        with tarfile.open(TREE_ARCHIVE, "r:gz") as t:
            for m in t.getmembers():
                assert m.isfile() and "/" not in m.name and not m.name.startswith(".")
                with open(os.path.join(d, m.name), "wb") as f:
                    f.write(t.extractfile(m).read())
        _tree_dir = d
    return _tree_dir


def static_poly_cost(d: str) -> int:
    """The expected static_poly.poy cost, read from cost_tests."""
    line = [x for x in open(os.path.join(d, "cost_tests")) if "static_poly.poy" in x][0]
    return int(line.split("-cost")[1].split()[0])
