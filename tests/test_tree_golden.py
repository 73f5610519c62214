"""Tree-level parity: the reference's own whole-tree cost tests.

test/cost_tests:11-14 read each of test/1.fas .. 13.fas (every
'#'-separated fragment a DO character), read a fixed tree and compare the
tree cost poy_test reports (``Ptree.get_cost `Adjusted``, poy_test.ml:43)
with a golden file:

  cc.poy   default matrix (sub 1, indel 2)          N.fas.tree    cc.costs
  cc1.poy  transform (tcm:(1,1))                     N.fas.1.tree  cc1.costs
  cc2.poy  transform (tcm:(2,1), gap_opening:1)      N.fas.2.tree  cc2.costs
  cc3.poy  transform (tcm:(3,1), gap_opening:5)      N.fas.3.tree  cc3.costs

and cnc*.poy repeat them with ``weightfactor:-1`` added (cnc*.costs).

Here the same files go through ``search.final_cost`` (best rooting, then
single-state assignment and the edge-distance sum) over the oracle's DO
medians, the backend the CUDA kernels match bit for bit.  The files are
read where the reference tree is present and the test skips elsewhere;
nothing of them is stored here."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from poyd_gb300 import formats, search, simulate
from tests.oracle_backend import OracleBackend

REF_TEST = os.environ.get("POYD_REFERENCE_TEST", "/root/reference/test")
have_ref = os.path.exists(os.path.join(REF_TEST, "cc.costs"))

MODELS = {"cc": ((1, 2, -1), "tree"), "cc1": ((1, 1, -1), "1.tree"),
          "cc2": ((2, 1, 1), "2.tree"), "cc3": ((3, 1, 5), "3.tree")}


def diagnose(fas, tree_file, om, weight=1):
    frags = formats.fasta_fragments(fas)
    t = formats.parse_tree(open(tree_file).read(), frags[0].names)
    return search.final_cost(t, [OracleBackend(ds, om) for ds in frags], weight)


@pytest.mark.skipif(not have_ref, reason="reference test files not present")
@pytest.mark.parametrize("model", sorted(MODELS))
def test_golden_tree_costs(model):
    (sub, indel, go), suffix = MODELS[model]
    om = O.cm_dna(sub, indel, go)
    gold = [int(x) for x in open(os.path.join(REF_TEST, model + ".costs")).read().split()]
    neg = [int(x) for x in open(os.path.join(REF_TEST, "cn" + model[1:] + ".costs")).read().split()]
    got, got_neg = [], []
    for f in range(1, len(gold) + 1):
        fas = os.path.join(REF_TEST, "%d.fas" % f)
        got.append(diagnose(fas, fas + "." + suffix, om).cost)
        if f <= 2:   # weightfactor -1 on the small datasets; it scales every cost
            got_neg.append(diagnose(fas, fas + "." + suffix, om, -1).cost)
    assert got == gold
    assert got_neg == neg[:len(got_neg)]
    assert [-c for c in got] == neg


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
    fc = search.final_cost(t, be)
    assert fc.root_cost == rc.best()[0]


def test_closest_rules():
    """DOS.to_single's cases: identical sequences (gap bits cleared, no
    alignment), an all-gap node (returned as is), an all-gap parent
    (replaced by the node) and ambiguity resolved towards the parent."""
    m = O.cm_dna(1, 2, -1)
    s = np.array([16, 1, 17, 4], np.uint8)
    assert O.closest(s, s, m).tolist() == [16, 1, 1, 4]
    assert O.closest(np.array([16, 1], np.uint8), np.array([16, 16], np.uint8), m).tolist() == [16, 16]
    assert O.closest(np.array([16], np.uint8), np.array([16, 5, 2], np.uint8), m).tolist() == [16, 1, 2]
    assert O.closest(np.array([16, 4, 2], np.uint8), np.array([16, 5, 2], np.uint8), m).tolist() == [16, 4, 2]
    assert O.closest(np.array([16, 1, 2], np.uint8), np.array([16, 15, 2], np.uint8), m).tolist() == [16, 1, 2]


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


def _rooted_on(adj, n, u, v):
    """A Tree over the unrooted adjacency `adj`, rooted on edge (u, v)."""
    t = search.Tree(n)
    nxt = [n]

    def build(x, frm):
        if x < n:
            return x
        kids = [build(c, x) for c in adj[x] if c != frm]
        w = nxt[0]
        nxt[0] += 1
        t.kids[w] = kids
        t.parent[kids[0]] = t.parent[kids[1]] = w
        return w

    a, b = build(u, v), build(v, u)
    r = nxt[0]
    t.kids[r] = (a, b)
    t.parent[a] = t.parent[b] = r
    t.parent[r] = -1
    t.root = r
    t.free = []
    t.in_tree[t.nodes()] = True
    return t


def test_root_costs_equal_downpass_of_every_rooting():
    """Each edge's root cost equals the ordinary downpass total of the tree
    rooted on that edge (Fitch and Sankoff characters included)."""
    data = simulate.simulate(4, 9, 90, 12, 3)
    om = O.cm_dna(1, 2, -1)
    t, _ = search.wagner(data.n_taxa, OracleBackend(data, om))
    rc = search.root_costs(t, OracleBackend(data, om))
    adj = search.unrooted_adjacency(t)
    for (u, v), c in zip(rc.edges.tolist(), rc.costs.tolist()):
        T = _rooted_on(adj, t.n, u, v)
        assert search.downpass(T, OracleBackend(data, om)).total == c, (u, v)
