"""Final states of the non-DO characters (the uppass of
``assign_final_states``, allDirChar.ml:1377-1428) through the search module
over the oracle backend (CPU).

Pin: with a 0/1 matrix a Sankoff character is a Fitch character, and the
states whose final e is 0 (the states of a most parsimonious
reconstruction, Goloboff 1998) are the Fitch final state set of
NonaddCS.median_3 (nonaddCSc.c:472-544).  On the reference's own
static_poly data (test/polymorphic.ss, 131 taxa, polymorphic and missing
cells) both characterisations must agree at every vertex."""
import os

import numpy as np

from oracle import oracle as O
from poyd_gb300 import formats, search, simulate
from tests import golden_io
from tests.oracle_backend import OracleBackend

D = golden_io.tree_golden_dir()


def test_sankoff_unit_matrix_finals_equal_fitch_finals():
    h = formats.read_hennig(os.path.join(D, "polymorphic.ss"))
    t = formats.parse_tree(h.trees[0], h.names)
    F, _, _ = h.fitch_matrix()
    n, k = len(h.names), 8
    bit = (F[:, :, None] >> np.arange(k)) & 1
    sank = np.where(bit == 1, 0, simulate.SANK_INF).astype(np.int32)
    data = simulate.Dataset(names=h.names, seqs=[np.array([16], np.uint8)] * n, fitch=F,
                            fitch_states=np.array([len(h.observed(c)) for c in
                                                   np.flatnonzero(~h.additive)], np.int64),
                            sank=sank, sank_tcm=(1 - np.eye(k)).astype(np.int32))
    fc = search.final_cost(t, OracleBackend(data, O.cm_dna(1, 2, -1)), states=True)
    finals = fc.finals[0]
    assert len(finals) == 2 * n - 2
    for v, (f, e, best) in finals.items():
        zero = ((e == 0).astype(np.int64) << np.arange(k)).sum(axis=1)
        assert np.array_equal(zero, f.astype(np.int64)), v


def test_final_states_on_a_simulated_tree():
    """Every vertex gets a final state; Fitch finals are non-empty subsets
    of the 8-bit lanes, every Sankoff final has a zero-cost state and a
    best state, and a leaf's Fitch final lies within its observed set."""
    data = simulate.simulate(9, 14, 60, n_fitch=30, n_sank=6)
    be = OracleBackend(data, O.cm_dna(1, 2, -1))
    t, _ = search.wagner(data.n_taxa, be)
    fc = search.final_cost(t, be, states=True)
    finals = fc.finals[0]
    assert len(finals) == 2 * data.n_taxa - 2
    for v, (f, e, best) in finals.items():
        assert np.all(f != 0)
        assert np.all((e == 0).any(axis=1)) and np.all(best != 0)
        if v < data.n_taxa:
            assert np.all((f & ~data.fitch[v]) == 0), v
