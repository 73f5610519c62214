"""Learned join proposal: trained on exact deltas logged by the plain
search, the network (a) ranks the truly best joins far better than an
untrained network or chance, and (b) lets a best-first search reach the
cost of a full exhaustive pass with at least 3x fewer exact DP
evaluations, every accepted tree being re-diagnosed exactly."""
import numpy as np
import pytest
import torch

from poyd_gb300 import align, learned, search, simulate

pytestmark = pytest.mark.gpu


def _recall(pred, delta, frac=0.05):
    k = max(1, int(frac * len(pred)))
    best = set(np.argsort(delta, kind="stable")[:k].tolist())
    top = np.argsort(pred, kind="stable")[:k]
    return len(best.intersection(top.tolist())) / k


@pytest.fixture(scope="module")
def trained():
    data = simulate.simulate(21, 64, 240, n_fitch=120, n_sank=12)
    be = search.GpuBackend(data, align.CostMatrix.default())
    Xs, ys = [], []
    for seed in range(8):  # the exact search logs its own training pairs
        t = learned.random_tree(data.n_taxa, 100 + seed)
        search.downpass(t, be)
        X, y = learned.log_pass(t, be)
        Xs.append(X)
        ys.append(y)
    X, y = torch.cat(Xs), torch.cat(ys)
    prop = learned.Proposal(seed=0)
    prop.fit(X, y, epochs=40, batch=1024, lr=1e-3)
    return data, be, prop, X


def test_ranking_gain(trained):
    data, be, prop, X = trained
    t = learned.random_tree(data.n_taxa, 999)
    search.downpass(t, be)
    Xt, yt = learned.log_pass(t, be)
    d = yt.cpu().numpy()
    r_trained = _recall(prop.predict(Xt).cpu().numpy(), d)
    r_untrained = []
    for seed in (5, 6, 7):
        u = learned.Proposal(seed=seed)
        u.mu, u.sd = prop.mu, prop.sd
        r_untrained.append(_recall(u.predict(Xt).cpu().numpy(), d))
    assert r_trained >= 0.3, r_trained
    assert r_trained >= 2 * float(np.mean(r_untrained)), (r_trained, r_untrained)


def test_best_first_search_needs_fewer_exact_evaluations(trained):
    data, be, prop, _ = trained
    t_plain = learned.random_tree(data.n_taxa, 4242)
    S, _ = search.spr_candidates(t_plain)
    st = search.spr_pass(t_plain, be, max_moves=8)
    target = st.cost_after
    exact_plain = len(S)
    stats = {}
    sc = learned.learned_scorer(prop, be, frac=0.05, stats=stats)
    t = learned.random_tree(data.n_taxa, 4242)
    costs = []
    for _ in range(6):
        s2 = search.spr_pass(t, be, max_moves=8, scorer=sc)
        costs.append(s2.cost_after)
        if s2.cost_after <= target:
            break
    assert costs[-1] <= target, (costs, target)
    assert costs[-1] == search.downpass(t, be).total
    assert 3 * stats["exact"] <= exact_plain, (stats, exact_plain)
