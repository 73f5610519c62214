"""The reference's own whole-tree cost tests through the CUDA path.

test/cost_tests:7-14 score test/1.fas .. 13.fas (every '#' fragment a DO
character) on fixed trees under four models and compare the reported tree
cost with cc*.costs, and with cnc*.costs under ``weightfactor:-1``;
test/cost_tests:17 (static_poly.poy) scores the Hennig matrix
polymorphic.ss.  Here every DO median, root median, single assignment and
distance is computed by the GB300 kernels (search.GpuBackend): 52 trees,
their 52 weight -1 twins, and static_poly's non-additive part on Fitch
kernels and on Sankoff kernels under a 0/1 matrix.  The inputs are the
reference's files, packed into tests/golden/tree_golden.tar.gz."""
import os

import numpy as np
import pytest

from poyd_gb300 import align, formats, search, simulate
from tests import golden_io
from tests.test_tree_golden import _static_cost, _static_cost_fitch_only

pytestmark = pytest.mark.gpu

D = golden_io.tree_golden_dir()
MODELS = {"cc": ((1, 2, None), "tree"), "cc1": ((1, 1, None), "1.tree"),
          "cc2": ((2, 1, 1), "2.tree"), "cc3": ((3, 1, 5), "3.tree")}


@pytest.mark.parametrize("model", sorted(MODELS))
def test_golden_tree_costs_on_gpu(model):
    (sub, indel, go), suffix = MODELS[model]
    cm = align.CostMatrix.dna(sub, indel, go)
    gold = [int(x) for x in open(os.path.join(D, model + ".costs")).read().split()]
    neg = [int(x) for x in open(os.path.join(D, "cn" + model[1:] + ".costs")).read().split()]
    assert len(gold) == 13 and len(neg) == 13
    got, got_neg = [], []
    for f in range(1, 14):
        fas = os.path.join(D, "%d.fas" % f)
        frags = formats.fasta_fragments(fas)
        t = formats.parse_tree(open(fas + "." + suffix).read(), frags[0].names)
        bes = [search.GpuBackend(ds, cm) for ds in frags]
        got.append(search.final_cost(t, bes, 1).cost)
        got_neg.append(search.final_cost(t, bes, -1).cost)
    assert got == gold
    assert got_neg == neg


def _hennig():
    h = formats.read_hennig(os.path.join(D, "polymorphic.ss"))
    return h, formats.parse_tree(h.trees[0], h.names)


def test_static_poly_fitch_on_gpu():
    """static_poly.poy's non-additive characters on the Fitch kernels: the
    downpass, the best rooting and the reported cost all give the expected
    cost less its additive part (1298 - 20)."""
    h, t = _hennig()
    want = golden_io.static_poly_cost(D)
    additive = _static_cost(h, h.trees[0]) - _static_cost_fitch_only(h, h.trees[0])
    F, _, _ = h.fitch_matrix()
    n = len(h.names)
    data = simulate.Dataset(names=h.names, seqs=[np.array([16], np.uint8)] * n, fitch=F,
                            fitch_states=np.array([len(h.observed(c)) for c in
                                                   np.flatnonzero(~h.additive)], np.int64),
                            sank=np.zeros((n, 0, 4), np.int32), sank_tcm=np.zeros((4, 4), np.int32))
    be = search.GpuBackend(data, align.CostMatrix.default())
    assert search.downpass(t, be).total == want - additive
    assert search.root_costs(t, be).best()[0] == want - additive
    assert search.final_cost(t, be).cost == want - additive


def test_static_poly_sankoff_on_gpu():
    """The same characters as 8-state Sankoff characters under a 0/1 matrix
    (Sankoff is then Fitch) on the Sankoff kernels: the same cost."""
    h, t = _hennig()
    F, _, _ = h.fitch_matrix()
    n, k = len(h.names), 8
    bit = (F[:, :, None] >> np.arange(k)) & 1
    sank = np.where(bit == 1, 0, simulate.SANK_INF).astype(np.int32)
    data = simulate.Dataset(names=h.names, seqs=[np.array([16], np.uint8)] * n,
                            fitch=np.zeros((n, 0), np.uint8), fitch_states=np.zeros(0, np.int64),
                            sank=sank, sank_tcm=(1 - np.eye(k)).astype(np.int32))
    be = search.GpuBackend(data, align.CostMatrix.default())
    want = _static_cost_fitch_only(h, h.trees[0])
    assert search.downpass(t, be).total == want
    assert search.final_cost(t, be).cost == want
