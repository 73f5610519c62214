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
the reference's own, packed unchanged into tests/golden/tree_golden.tar.gz
by tests/golden/make_tree_golden.py; tests/test_gpu_tree_golden.py runs
them through the CUDA path."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from poyd_gb300 import formats, search, simulate
from tests import golden_io
from tests.oracle_backend import OracleBackend

REF_TEST = golden_io.tree_golden_dir()

MODELS = {"cc": ((1, 2, -1), "tree"), "cc1": ((1, 1, -1), "1.tree"),
          "cc2": ((2, 1, 1), "2.tree"), "cc3": ((3, 1, 5), "3.tree")}


def diagnose(fas, tree_file, om, weight=1):
    frags = formats.fasta_fragments(fas)
    t = formats.parse_tree(open(tree_file).read(), frags[0].names)
    return search.final_cost(t, [OracleBackend(ds, om) for ds in frags], weight)


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


def _static_cost(h, tree_text):
    """Whole-tree cost of a Hennig matrix's static characters on a fixed
    tree: the oracle's Fitch medians (nonaddCSc.c:422-462) for the
    non-additive characters plus, for the additive ones, the interval rule
    of add_item (add.c:559-600) restated here as a test helper (additive
    characters are not on the GPU path).  Both totals are root-invariant."""
    F, _, w = h.fitch_matrix()
    assert (w == 1).all()
    lo, hi, _ = h.additive_intervals()
    t = formats.parse_tree(tree_text, h.names)
    total = 0
    state = {}
    for v in t.nodes()[::-1]:   # reversed preorder: children before parents
        if v < t.n:
            state[v] = (F[v], lo[v].astype(np.int64), hi[v].astype(np.int64))
            continue
        a, b = (state[int(k)] for k in t.kids[v])
        c, med = O.nonadd_median(a[0], b[0])
        lo_v, hi_v = np.maximum(a[1], b[1]), np.minimum(a[2], b[2])
        gap = lo_v > hi_v
        total += c + int((lo_v - hi_v)[gap].sum())
        state[v] = (med, np.where(gap, hi_v, lo_v), np.where(gap, lo_v, hi_v))
    return total


def test_static_poly_cost():
    """test/cost_tests' static_poly.poy: the Hennig matrix
    test/polymorphic.ss (non-additive characters with polymorphic and
    missing cells, two additive characters) on the tree its tread gives;
    the expected cost is read from test/cost_tests."""
    want = golden_io.static_poly_cost(REF_TEST)
    h = formats.read_hennig(os.path.join(REF_TEST, "polymorphic.ss"))
    assert len(h.trees) == 1
    assert _static_cost(h, h.trees[0]) == want


def test_read_hennig(tmp_path):
    p = tmp_path / "m.ss"
    p.write_text("xread\n'title; with a semicolon'\n5 4\n"
                 "a 0 1 2 [01] ?\nb 1 1 0 2 A\nc 0.0-0 V\nd 1 [1 2] 1 3 0\n;\n"
                 "cc - 0.2;\ncc + 3 ] 4;\nccode /3 1.;\n"
                 "cn {0 first x y ;\n"
                 "tread (a (b (c d)))*(0 (3 (1 2)));\nproc/;\n")
    h = formats.read_hennig(str(p))
    assert h.names == ["a", "b", "c", "d"]
    assert h.cells[:, 3].tolist() == [0b11, 0b100, 0b1, 0b1000]
    assert h.cells[2].tolist() == [1, 1, 0, 1, 1 << 31]
    assert h.cells[3, 1] == 0b110 and h.cells[1, 4] == 1 << 10
    assert h.additive.tolist() == [False, False, False, True, True]
    assert h.active.tolist() == [True, True, True, True, False]
    assert h.weight.tolist() == [1, 3, 3, 3, 3]
    assert h.trees[1].split() == ["(a", "(d", "(b", "c)))"]
    F, cols, w = h.fitch_matrix()
    assert cols.tolist() == [0, 1, 2] and w.tolist() == [1, 3, 3]
    # character 2 observes states {0, 1, 2}: bit i is its i-th state
    # (c is missing there, so it holds all three)
    assert F[:, 2].tolist() == [0b100, 0b001, 0b111, 0b010]
    assert F[:, 1].tolist() == [0b010, 0b010, 0b001, 0b110]
    lo, hi, acols = h.additive_intervals()
    assert acols.tolist() == [3] and lo[:, 0].tolist() == [0, 2, 0, 3]
    assert hi[:, 0].tolist() == [1, 2, 0, 3]


def _sankoff_tree_cost(t, leaves, tcm):
    """Root cost of a Sankoff downpass (the oracle's elt_median,
    sankCS.ml:302-338) with leaf cost vectors leaves[v] [n_chars, k]."""
    s = {}
    for v in t.nodes()[::-1]:
        if v < t.n:
            s[v] = leaves[v]
            continue
        a, b = (s[int(k)] for k in t.kids[v])
        s[v] = np.array([O.sank_elt_median(tcm, a[c], b[c])[0] for c in range(len(a))])
    return int(s[t.root].min(axis=1).sum())


def test_static_poly_cost_through_sankoff():
    """Sankoff with a 0/1 matrix is Fitch, and with |i - j| costs it is the
    additive rule: the Sankoff oracle on polymorphic.ss, non-additive
    characters under the unit matrix and additive ones under the linear
    matrix (a cell's leaf vector 0 on its states, infinite elsewhere), must
    give the same whole-tree cost as the reference's static_poly test."""
    want = golden_io.static_poly_cost(REF_TEST)
    h = formats.read_hennig(os.path.join(REF_TEST, "polymorphic.ss"))
    t = formats.parse_tree(h.trees[0], h.names)
    k = 8
    F, _, _ = h.fitch_matrix()
    lo, hi, _ = h.additive_intervals()
    bit = (F[:, :, None] >> np.arange(k)) & 1
    unit = np.where(bit == 1, 0, O.SANK_INF).astype(np.int64)
    st = np.arange(k)
    inside = (st >= lo[:, :, None]) & (st <= hi[:, :, None])
    ordered = np.where(inside, 0, O.SANK_INF).astype(np.int64)
    tcm_unit = 1 - np.eye(k, dtype=np.int64)
    tcm_lin = np.abs(st[:, None] - st[None, :]).astype(np.int64)
    got = (_sankoff_tree_cost(t, unit, tcm_unit) + _sankoff_tree_cost(t, ordered, tcm_lin))
    assert got == want


def test_static_poly_fitch_through_the_search_module():
    """The search module's own accounting (downpass, best rooting, reported
    cost) over polymorphic.ss's non-additive characters, with an empty DO
    character beside them, gives the static_poly cost less its additive
    part."""
    want = golden_io.static_poly_cost(REF_TEST)
    h = formats.read_hennig(os.path.join(REF_TEST, "polymorphic.ss"))
    t = formats.parse_tree(h.trees[0], h.names)
    F, _, _ = h.fitch_matrix()
    n = len(h.names)
    data = simulate.Dataset(names=h.names, seqs=[np.array([16], np.uint8)] * n, fitch=F,
                            fitch_states=np.array([len(h.observed(c)) for c in
                                                   np.flatnonzero(~h.additive)], np.int64),
                            sank=np.zeros((n, 0, 4), np.int32), sank_tcm=np.zeros((4, 4), np.int32))
    additive = _static_cost(h, h.trees[0]) - _static_cost_fitch_only(h, h.trees[0])
    be = OracleBackend(data, O.cm_dna(1, 2, -1))
    assert search.downpass(t, be).total == want - additive
    assert search.root_costs(t, be).best()[0] == want - additive
    assert search.final_cost(t, be).cost == want - additive


def _static_cost_fitch_only(h, tree_text):
    F, _, _ = h.fitch_matrix()
    t = formats.parse_tree(tree_text, h.names)
    total, state = 0, {}
    for v in t.nodes()[::-1]:
        if v < t.n:
            state[v] = F[v]
            continue
        c, state[v] = O.nonadd_median(*(state[int(k)] for k in t.kids[v]))
        total += c
    return total


def test_static_poly_sankoff_through_the_search_module():
    """The same characters as Sankoff characters under a 0/1 matrix (which
    makes Sankoff equal Fitch) through the search module: the same cost."""
    h = formats.read_hennig(os.path.join(REF_TEST, "polymorphic.ss"))
    t = formats.parse_tree(h.trees[0], h.names)
    F, _, _ = h.fitch_matrix()
    n, k = len(h.names), 8
    bit = (F[:, :, None] >> np.arange(k)) & 1
    sank = np.where(bit == 1, 0, simulate.SANK_INF).astype(np.int32)
    data = simulate.Dataset(names=h.names, seqs=[np.array([16], np.uint8)] * n,
                            fitch=np.zeros((n, 0), np.uint8), fitch_states=np.zeros(0, np.int64),
                            sank=sank, sank_tcm=(1 - np.eye(k)).astype(np.int32))
    be = OracleBackend(data, O.cm_dna(1, 2, -1))
    want = _static_cost_fitch_only(h, h.trees[0])
    assert search.downpass(t, be).total == want
    assert search.final_cost(t, be).cost == want


def test_hennig_fitch_groups_by_state_count(tmp_path):
    """Characters of 2-8, 9-16 and 17-32 observed states go to 8-, 16- and
    32-bit lanes; one-state characters are left out; the grouped Fitch cost
    on a tree equals a direct per-character Fitch over the raw state sets."""
    rng = np.random.default_rng(21)
    sym = formats.HENNIG_STATES
    n_taxa, spans = 24, [3, 12, 20, 1, 2, 32]   # states per character
    rows = []
    for t in range(n_taxa):
        cells = []
        for c, k in enumerate(spans):
            # each state appears somewhere: taxon t takes state t mod k, some
            # taxa a polymorphic pair, one a missing cell
            s = {(t + c) % k}
            if t % 4 == 1 and k > 1:
                s.add((t + 3) % k)
            cells.append("?" if t == 7 and c == 1 else
                         sym[s.pop()] if len(s) == 1 else "[" + "".join(sym[x] for x in s) + "]")
        rows.append("t%d %s" % (t, " ".join(cells)))
    p = tmp_path / "g.ss"
    p.write_text("xread\n%d %d\n%s\n;\ncc - .;\ncc + 4;\n" % (len(spans), n_taxa, "\n".join(rows)))
    h = formats.read_hennig(str(p))
    obs = [len(h.observed(c)) for c in range(len(spans))]
    g = h.fitch_groups()
    want_w = {c: (8 if k <= 8 else 16 if k <= 16 else 32) for c, k in enumerate(obs)
              if k >= 2 and c != 4}
    got_w = {int(c): w for w, (_, cols, _) in g.items() for c in cols}
    assert got_w == want_w and sorted(g) == [8, 16, 32]
    t = search.Tree(n_taxa)
    order = list(rng.permutation(n_taxa))
    t.start(int(order[0]), int(order[1]))
    for x in order[2:]:
        t.insert(int(x), int(rng.choice([v for v in t.nodes()])))
    grouped = 0
    for w, (M, _, _) in g.items():
        state = {}
        for v in t.nodes()[::-1]:
            if v < t.n:
                state[v] = M[v]
                continue
            c, state[v] = O.nonadd_median_w(*(state[int(k)] for k in t.kids[v]), w)
            grouped += c
    direct = 0
    for c in want_w:
        full = sum(1 << s for s in h.observed(c))
        st = {}
        for v in t.nodes()[::-1]:
            if v < t.n:
                st[v] = int(h.cells[v, c]) or full
                continue
            a, b = (st[int(k)] for k in t.kids[v])
            st[v] = a & b if a & b else a | b
            direct += not (a & b)
    assert grouped == direct > 0
