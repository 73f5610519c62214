"""Tree-level parity: the reference's own whole-tree cost tests.

test/cost_tests:11-12 read each of test/1.fas .. 13.fas (every
'#'-separated fragment a DO character), read a fixed tree
(test/N.fas.tree for cc.poy with the default sub 1 / indel 2 matrix,
test/N.fas.1.tree for cc1.poy after ``transform (tcm:(1,1))``) and compare
the diagnosed tree cost with test/cc.costs and test/cc1.costs.  Here the
same files are diagnosed with the all-rootings diagnosis over the oracle's
DO medians (the backend the CUDA kernels match bit for bit): the cost of
the best rooting, summed over the fragments with one root for all, must
equal the golden cost.  The files are read where the reference tree is
present and the test skips elsewhere; nothing of them is stored here.

The affine models (cc2.poy, cc3.poy) are not covered: there the reported
cost comes from the final-state assignment (``assign_single``), which is
not restated."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from poyd_gb300 import formats, search, simulate
from tests.oracle_backend import OracleBackend

REF_TEST = os.environ.get("POYD_REFERENCE_TEST", "/root/reference/test")
have_ref = os.path.exists(os.path.join(REF_TEST, "cc.costs"))

MODELS = {"cc": ((1, 2, -1), "tree"), "cc1": ((1, 1, -1), "1.tree")}


def tree_cost(fas, tree_file, om):
    frags = formats.fasta_fragments(fas)
    names = frags[0].names
    t = formats.parse_tree(open(tree_file).read(), names)
    total = None
    for ds in frags:
        rc = search.root_costs(t, OracleBackend(ds, om))
        total = rc.costs if total is None else total + rc.costs
    return int(total.min())


@pytest.mark.skipif(not have_ref, reason="reference test files not present")
@pytest.mark.parametrize("model", sorted(MODELS))
def test_golden_tree_costs(model):
    (sub, indel, go), suffix = MODELS[model]
    om = O.cm_dna(sub, indel, go)
    gold = [int(x) for x in open(os.path.join(REF_TEST, model + ".costs")).read().split()]
    got = []
    for f in range(1, len(gold) + 1):
        fas = os.path.join(REF_TEST, "%d.fas" % f)
        got.append(tree_cost(fas, fas + "." + suffix, om))
    assert got == gold


def test_rooted_downpass_is_one_rooting():
    """The downpass total of a rooted tree is the root cost of the edge
    joining the root's two children."""
    data = simulate.simulate(3, 12, 120, 20, 4)
    be = OracleBackend(data, O.cm_dna(1, 2, -1))
    t, diag = search.wagner(data.n_taxa, be)
    rc = search.root_costs(t, be)
    a, b = sorted(int(x) for x in t.kids[t.root])
    k = [i for i, e in enumerate(rc.edges.tolist()) if e == [a, b]]
    assert len(k) == 1
    assert int(rc.costs[k[0]]) == diag.total
    assert len(rc.edges) == 2 * data.n_taxa - 3
    assert rc.best()[0] == int(rc.costs.min()) <= diag.total


def test_formats():
    assert formats.encode_dna("ACgt-N r").tolist() == [16, 1, 2, 4, 8, 15, 5]
    assert formats.encode_dna("A-C", remove_gaps=False).tolist() == [16, 1, 16, 2]
    with pytest.raises(ValueError):
        formats.encode_dna("AZ")
    names = ["t1", "t2", "t3", "t4"]
    t = formats.parse_tree("(t1 ((t2 t3) t4))[12.]", names)
    assert t.newick() == "(0,((1,2),3));"
    assert formats.parse_tree("((t1,t2),(t3,t4));", names).newick() == "((0,1),(2,3));"
    with pytest.raises(ValueError):
        formats.parse_tree("(t1 (t2 t1))", names)
    part = formats.parse_tree("(t1 (t2 t4))", names)
    assert sorted(part.nodes())[:3] == [0, 1, 3] and not part.in_tree[2]
    assert search.Tree.min_codes(t)[t.root] == 0
