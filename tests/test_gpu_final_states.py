"""Final states of the non-DO characters on the GB300 kernels (NonaddCS
median_3 and the SankCS median_3 kernel) equal the oracle's, vertex by
vertex, after the best rooting of a mixed DO + Fitch + Sankoff tree
(``assign_final_states``, allDirChar.ml:1377-1428); and the 0/1-matrix
Sankoff finals equal the Fitch finals on the reference's static_poly data."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from poyd_gb300 import align, formats, search, simulate
from tests import golden_io
from tests.oracle_backend import OracleBackend

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [3, 17])
def test_mixed_tree_final_states_match_oracle(seed):
    data = simulate.simulate(seed, 24, 150, n_fitch=60, n_sank=12)
    ob = OracleBackend(data, O.cm_dna(1, 2, -1))
    t, _ = search.wagner(data.n_taxa, ob)
    want = search.final_cost(t, ob, states=True)
    gb = search.GpuBackend(data, align.CostMatrix.default())
    got = search.final_cost(t, gb, states=True)
    assert got.cost == want.cost and got.root_edge == want.root_edge
    fw, fg = want.finals[0], got.finals[0]
    assert sorted(fw) == sorted(fg) and len(fg) == 2 * data.n_taxa - 2
    for v in fw:
        for x, y in zip(fw[v], fg[v]):
            assert np.array_equal(np.asarray(x), np.asarray(y)), v


def test_static_poly_unit_sankoff_finals_equal_fitch_on_gpu():
    d = golden_io.tree_golden_dir()
    h = formats.read_hennig(os.path.join(d, "polymorphic.ss"))
    t = formats.parse_tree(h.trees[0], h.names)
    F, _, _ = h.fitch_matrix()
    n, k = len(h.names), 8
    bit = (F[:, :, None] >> np.arange(k)) & 1
    sank = np.where(bit == 1, 0, simulate.SANK_INF).astype(np.int32)
    data = simulate.Dataset(names=h.names, seqs=[np.array([16], np.uint8)] * n, fitch=F,
                            fitch_states=np.array([len(h.observed(c)) for c in
                                                   np.flatnonzero(~h.additive)], np.int64),
                            sank=sank, sank_tcm=(1 - np.eye(k)).astype(np.int32))
    fc = search.final_cost(t, search.GpuBackend(data, align.CostMatrix.default()), states=True)
    for v, (f, e, best) in fc.finals[0].items():
        zero = ((e == 0).astype(np.int64) << np.arange(k)).sum(axis=1)
        assert np.array_equal(zero, f.astype(np.int64)), v
