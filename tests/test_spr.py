"""SPR (single_spr_round, ptree.ml:1142-1169) on the oracle backend: the
candidate enumeration against its definition, and a pass that only
accepts moves whose exact re-diagnosed cost is lower."""
import numpy as np

from oracle import oracle as O
from poyd_gb300 import learned, search, simulate
from tests.oracle_backend import OracleBackend


def test_spr_candidate_enumeration():
    """Every pruned subtree (parent not the root) joined to every node
    outside it except its parent and sibling, subtrees in ascending order
    and join nodes ascending within each."""
    for n, seed in ((3, 1), (4, 2), (9, 3), (30, 4)):
        t = learned.random_tree(n, seed)
        S, E = search.spr_candidates(t)
        want = []
        for s in sorted(t.nodes()):
            p = t.parent[s]
            if p < 0 or t.parent[p] < 0:
                continue
            inside = set(t.subtree(s))
            sib = int(t.kids[p][0] if t.kids[p][1] == s else t.kids[p][1])
            want += [(s, e) for e in sorted(t.nodes()) if e not in inside and e not in (p, sib)]
        assert list(zip(S.tolist(), E.tolist())) == want, n


def test_spr_pass_lowers_or_keeps_cost():
    data = simulate.simulate(7, 14, 120, 16, 3)
    be = OracleBackend(data, O.cm_dna(1, 2, -1))
    t = learned.random_tree(data.n_taxa, 11)
    st = search.spr_pass(t, be, max_moves=8)
    assert st.candidates == len(search.spr_candidates(learned.random_tree(data.n_taxa, 11))[0])
    assert st.moves_accepted > 0 and st.cost_after < st.cost_before
    assert search.downpass(t, be).total == st.cost_after
    assert sorted(v for v in t.nodes() if v < t.n) == list(range(t.n))


def test_distinct_nodes_matches_unique():
    rng = np.random.default_rng(5)
    for n in (0, 1, 50, 100000):
        ids = rng.integers(0, 700, n)
        assert np.array_equal(search.distinct_nodes(ids, 700), np.unique(ids))
    assert search.distinct_nodes(np.zeros(0, np.int64), 10).dtype == np.int64


def test_overlay_evaluation_equals_tree_copies():
    """SPR trials applied as overlays over the base tree (evaluate_trials'
    fast path) give the totals and recomputed nodes of the same trials
    applied to tree copies (the path TBR moves take; (s, e, -1) is an SPR
    move written as TBR without re-rooting), single moves and pairs."""
    data = simulate.simulate(4, 18, 60, 8, 2)
    be = OracleBackend(data, O.cm_dna(1, 2, -1))
    t = learned.random_tree(data.n_taxa, 5)
    diag = search.downpass(t, be)
    S, E = search.spr_candidates(t)
    rng = np.random.default_rng(0)
    pick = rng.choice(len(S), size=12, replace=False)
    moves = [(int(S[i]), int(E[i])) for i in pick]
    trials = [[m] for m in moves]
    for a in moves[:4]:
        tg = t.copy()
        tg.insert(a[0], a[1], tg.prune(a[0]))
        trials += [[a, b] for b in moves[4:] if search._valid_move(tg, *b)]
    d1, d2 = {}, {}
    r1 = search.evaluate_trials(t, be, diag, trials, d1)
    be.release_nodes(2 * t.n)
    r2 = search.evaluate_trials(t, be, diag, [[(s, e, -1) for s, e in tr] for tr in trials], d2)
    be.release_nodes(2 * t.n)
    assert np.array_equal(r1, r2) and len(trials) > 12
    assert d1 == d2
