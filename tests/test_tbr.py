"""TBR (tbr_join re-rooting, ptree.ml:1178-1217) on the oracle backend:
re-rooting keeps the unrooted tree, every re-rooted clade's score is the
distance its re-diagnosed root median gives, and a TBR pass only accepts
moves whose exact cost is lower."""
import numpy as np

from oracle import oracle as O
from poyd_gb300 import search, simulate
from tests.oracle_backend import OracleBackend


def _setup(seed=5, n=12, length=120):
    data = simulate.simulate(seed, n, length, 16, 3)
    be = OracleBackend(data, O.cm_dna(1, 2, -1))
    t, diag = search.wagner(data.n_taxa, be)
    return data, be, t, diag


def _ancestors(t, v):
    out = set()
    while t.parent[v] >= 0:
        v = t.parent[v]
        out.add(int(v))
    return out


def _clade_splits(t, s):
    """Bipartitions of the clade under s taken as an unrooted tree."""
    leaves = frozenset(x for x in t.subtree(s) if x < t.n)
    out = set()
    for v in t.subtree(s):
        if v == s:
            continue
        below = frozenset(x for x in t.subtree(v) if x < t.n)
        other = leaves - below
        if len(below) > 1 and len(other) > 1:
            out.add(min(below, other, key=min))
    return out


def test_reroot_keeps_the_clade_and_moves_its_attachment():
    """Re-rooting changes where the clade joins the rest of the tree (the
    point of a TBR move), not the clade itself or anything outside it."""
    data, be, t, _ = _setup()
    done = 0
    for s in t.nodes():
        if s < t.n or t.parent[s] < 0:
            continue
        for u in t.subtree(s):
            if u == s or t.parent[u] == s:
                continue
            T = t.copy()
            T.reroot(s, u)
            assert sorted(T.nodes()) == sorted(t.nodes())
            assert set(T.subtree(s)) == set(t.subtree(s))
            assert _clade_splits(T, s) == _clade_splits(t, s)
            assert set(T.kids[s].tolist()) == {u, int(t.parent[u])}
            outside = [v for v in t.nodes() if v not in set(t.subtree(s))]
            for v in outside:
                assert T.parent[v] == t.parent[v]
            done += 1
    assert done > 0


def test_rerooted_scores_match_rediagnosis():
    data, be, t, _ = _setup(seed=6)
    diag = search.downpass(t, be)
    S, U, E, score, dclade = search.tbr_candidates(t, be, diag)
    assert len(S) == len(U) == len(E) == len(score) == len(dclade)

    def clade_cost(tree, d, s):
        return sum(d.do_cost[v] + d.fitch_cost[v] for v in tree.subtree(s) if v >= tree.n)
    rng = np.random.default_rng(0)
    idx = [i for i in range(len(S)) if U[i] >= 0 and int(E[i]) not in _ancestors(t, int(S[i]))]
    assert idx
    for i in rng.choice(idx, size=min(12, len(idx)), replace=False):
        s, u, e = int(S[i]), int(U[i]), int(E[i])
        T = t.copy()
        T.reroot(s, u)
        be2 = OracleBackend(data, O.cm_dna(1, 2, -1))
        d2 = search.downpass(T, be2)
        assert int(be2.distances([s], [e])[0]) == int(score[i]), (s, u, e)
        assert clade_cost(T, d2, s) - clade_cost(t, diag, s) == int(dclade[i]), (s, u)
    # the clade's own rooting scores as SPR does
    j = [i for i in range(len(S)) if U[i] < 0]
    assert not dclade[j].any()
    be.ensure_nodes(2 * t.n)
    assert np.array_equal(score[j], be.distances(S[j], E[j]))


def test_tbr_pass_lowers_or_keeps_cost():
    data, be, t, diag = _setup(seed=7, n=14)
    st = search.tbr_pass(t, be, max_moves=8, diag=diag)
    assert st.candidates > 0
    assert st.cost_after <= st.cost_before
    assert search.downpass(t, be).total == st.cost_after
    assert sorted(v for v in t.nodes() if v < t.n) == list(range(t.n))


def test_join_distance_of_an_empty_sequence_is_zero():
    """A join with an all-gap sequence costs nothing on the DO character
    (the join cost's missing distance, Node.Standard.distance 0.)."""
    data = simulate.simulate(9, 6, 80, 10, 2)
    data.seqs[2] = np.array([16], np.uint8)
    be = OracleBackend(data, O.cm_dna(1, 2, -1))
    full = be.distances([2, 0], [0, 1])
    fitch_sank = [O.nonadd_distance(be.fitch[2], be.fitch[0]) +
                  int(sum(O.sank_elt_distance(be.tcm, be.sank[2][c], be.sank[0][c])
                          for c in range(be.ns)))]
    assert int(full[0]) == fitch_sank[0]
    assert int(full[1]) > 0


def test_tbr_candidate_enumeration():
    """Every clade (parent not the root) appears with its own rooting and
    with each re-rooting below its children, joined to every node outside
    it except its parent (and, for its own rooting, its sibling)."""
    data, be, t, diag = _setup(seed=8, n=10, length=60)
    S, U, E, score, dclade = search.tbr_candidates(t, be, diag)
    nodes = set(t.nodes())
    want = set()
    for s in nodes:
        p = t.parent[s]
        if p < 0 or t.parent[p] < 0:
            continue
        inside = set(t.subtree(s))
        sib = int(t.kids[p][0] if t.kids[p][1] == s else t.kids[p][1])
        reroots = [-1] + [u for u in inside if u != s and t.parent[u] != s]
        for u in reroots:
            for e in nodes - inside - {int(p)}:
                if u < 0 and e == sib:
                    continue
                want.add((s, u, e))
    got = set(zip(S.tolist(), U.tolist(), E.tolist()))
    assert len(got) == len(S) and got == want


def test_either_empty_matches_a_sort():
    """The GPU backend's all-gap test per pair asks once per distinct node
    and agrees with the sort-based formulation."""
    rng = np.random.default_rng(3)
    empty_nodes = set(rng.choice(300, 40, replace=False).tolist())
    asked = []

    def empty(v):
        asked.append(v.copy())
        return np.array([int(x) in empty_nodes for x in v], bool)
    for n in (0, 1, 17, 5000):
        a = rng.integers(0, 300, n)
        b = rng.integers(0, 300, n)
        asked.clear()
        got = search.either_empty(a, b, 300, empty)
        u, inv = np.unique(np.concatenate([a, b]).astype(np.int64), return_inverse=True)
        e = np.array([int(x) in empty_nodes for x in u], bool)[inv]
        assert np.array_equal(got, e[:n] | e[n:])
        if n:
            assert len(asked) == 1 and np.array_equal(asked[0], u)
        else:
            assert not asked
