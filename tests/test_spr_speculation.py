"""The SPR pass's speculative rounds (each round also evaluates every move
after the best-scored one) accept exactly the moves of the plain greedy
rounds: the same final tree, cost and number of accepted moves, on the
oracle backend."""
import numpy as np
import pytest

from oracle import oracle as O
from poyd_gb300 import learned, search, simulate
from tests.oracle_backend import OracleBackend


def greedy_pass(t, be, max_moves):
    """The pass without speculation: candidate scores, the best-scored
    move per pruned subtree, then rounds of exact evaluation accepting the
    best improving move."""
    diag = search.downpass(t, be)
    S, E = search.spr_candidates(t)
    score = be.distances(S, E)
    subs = search.distinct_nodes(S, len(t.parent))
    cur = np.zeros(len(t.parent), np.int64)
    p = t.parent[subs]
    sib = np.where(t.kids[p, 0] == subs, t.kids[p, 1], t.kids[p, 0])
    cur[subs] = be.distances(subs, sib)
    gain = cur[S] - score
    pos = np.nonzero(gain > 0)[0]
    order = pos[np.lexsort((E[pos], S[pos], -gain[pos]))]
    moves, seen = [], set()
    for i in order:
        if len(moves) >= max_moves:
            break
        if int(S[i]) not in seen:
            seen.add(int(S[i]))
            moves.append((int(S[i]), int(E[i])))
    best, accepted = diag.total, 0
    while moves:
        detail = {}
        totals = search.evaluate_moves(t, be, diag, moves, detail)
        k = int(np.argmin(totals))
        if totals[k] >= best:
            be.release_nodes(2 * t.n)
            break
        s, e = moves.pop(k)
        t.insert(s, e, t.prune(s))
        search.commit_move(be, diag, detail[k], totals[k])
        be.release_nodes(2 * t.n)
        best, accepted = int(totals[k]), accepted + 1
        moves = [(a, b) for a, b in moves if search._valid_move(t, a, b)]
    return best, accepted


@pytest.mark.parametrize("seed", [3, 7, 12, 21])
def test_speculative_pass_accepts_the_greedy_moves(seed):
    data = simulate.simulate(seed, 16, 90, 12, 2)
    t1 = learned.random_tree(data.n_taxa, seed + 100)
    t2 = t1.copy()
    be1 = OracleBackend(data, O.cm_dna(1, 2, -1))
    be2 = OracleBackend(data, O.cm_dna(1, 2, -1))
    st = search.spr_pass(t1, be1, max_moves=8)
    cost, accepted = greedy_pass(t2, be2, 8)
    assert (st.cost_after, st.moves_accepted) == (cost, accepted)
    assert np.array_equal(t1.parent, t2.parent) and np.array_equal(t1.kids, t2.kids)
    assert search.downpass(t1, be1).total == cost
