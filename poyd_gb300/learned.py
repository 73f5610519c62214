"""Learned join proposal for the SPR candidate pass.

A small MLP (poyd_gb300.mlp) predicts, from cheap features, how much a
candidate join (pruned subtree s onto the edge above e) changes the cost
relative to s's current attachment.  The exact search logs its own
(candidate, exact delta) pairs for training; at search time the network
orders all candidates, only the best-predicted fraction is scored with the
exact DP, and the exact downpass alone decides whether a tree is
accepted.  When a learned pass accepts nothing, an exhaustive pass is the
fallback, so the search stops at the same kind of local optimum.

Features (32, computed on the device): clade sizes, depths, sequence and
median lengths (s, e, their parents), Fitch distances and bitset summaries
(s-e, s-parent(e), s-sibling, ambiguity), Sankoff distances, the exact
current attachment distance of s, and a few products.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np
import torch

from . import native, search
from .mlp import MLP

NFEAT = 32
_POPC = torch.tensor([bin(i).count("1") for i in range(256)], dtype=torch.float32)


def node_info(t: search.Tree, be):
    """Subtree sizes, depths, parents (a root is its own) and siblings of
    every node (cached per tree state; do not modify the arrays)."""
    return t._memo("node_info", lambda: _node_info(t))


def _node_info(t: search.Tree):
    n_nodes = len(t.parent)
    parent, kids, n = t.parent.tolist(), t.kids.tolist(), t.n
    size = [0.0] * n_nodes
    depth = [0.0] * n_nodes
    sib = list(range(n_nodes))
    order = t.nodes()
    for v in order:  # preorder: parents first
        p = parent[v]
        if p >= 0:
            depth[v] = depth[p] + 1
            a, b = kids[p]
            sib[v] = a if b == v else b
    for v in order[::-1]:
        size[v] = 1.0 if v < n else size[kids[v][0]] + size[kids[v][1]]
    par = np.where(t.parent >= 0, t.parent, np.arange(n_nodes))
    return (np.array(size, np.float32), np.array(depth, np.float32), par,
            np.array(sib, np.int64))


def _as_idx(be, x):
    """Node ids as a device int32 tensor (host arrays are uploaded once)."""
    if isinstance(x, torch.Tensor):
        return x.to(device=be.dev, dtype=torch.int32)
    return torch.from_numpy(np.ascontiguousarray(x, np.int32)).to(be.dev)


def _fitch_dist(be, a, b):
    ia, ib = _as_idx(be, a), _as_idx(be, b)
    n = int(ia.numel())
    if not be.nf or n == 0:
        return torch.zeros(n, dtype=torch.float32, device=be.dev)
    out = torch.empty(n, dtype=torch.int64, device=be.dev)
    native.check(native.lib().poyd_nonadd8_distance_batch(
        C.c_void_p(be.fitch.data_ptr()), C.c_int64(be.stride), be.nf, n, C.c_void_p(ia.data_ptr()),
        C.c_void_p(ib.data_ptr()), C.c_void_p(out.data_ptr()),
        C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    return out.to(torch.float32)


def _sank_dist(be, a, b):
    ia, ib = _as_idx(be, a), _as_idx(be, b)
    n = int(ia.numel())
    if not be.ns or n == 0:
        return torch.zeros(n, dtype=torch.float32, device=be.dev)
    out = torch.empty(n, dtype=torch.int64, device=be.dev)
    native.check(native.lib().poyd_sank_distance_batch(
        C.c_void_p(be.sank.data_ptr()), be.ns, be.k, C.c_void_p(be.tcm.data_ptr()), n,
        C.c_void_p(ia.data_ptr()), C.c_void_p(ib.data_ptr()), C.c_void_p(out.data_ptr()),
        C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    return out.to(torch.float32)


def features(t: search.Tree, be, S: np.ndarray, E: np.ndarray, cur: dict) -> torch.Tensor:
    """[len(S), 32] fp32 features of candidate joins (S[i] onto the edge above E[i])."""
    dev = be.dev
    size, depth, par, sib = node_info(t, be)
    T = lambda x: torch.from_numpy(np.ascontiguousarray(x, np.float32)).to(dev)
    I = lambda x: torch.from_numpy(np.ascontiguousarray(x, np.int64)).to(dev)
    L = T(be.len)
    nf, ns = max(be.nf, 1), max(be.ns, 1)
    amb = (_POPC.to(dev)[be.fitch[:, :be.nf].long()].mean(dim=1) if be.nf
           else torch.zeros(len(be.len), device=dev))
    # the candidates are uploaded once; parents, siblings and attachment
    # costs are gathered on the device from per-node tables
    s32, e32 = _as_idx(be, S), _as_idx(be, E)
    s, e = s32.long(), e32.long()
    par_t, sib_t = I(par), I(sib)
    pe, ps, sb = par_t[e], par_t[s], sib_t[s]
    fse = _fitch_dist(be, s32, e32) / nf * 10
    fspe = _fitch_dist(be, s32, pe) / nf * 10
    fsib = _fitch_dist(be, s32, sb) / nf * 10
    sse = _sank_dist(be, s32, e32) / ns
    ssib = _sank_dist(be, s32, sb) / ns
    curs = T(cur.astype(np.float32))[s]
    size_t, depth_t = T(size), T(depth)
    f = [
        torch.log1p(size_t[s]), torch.log1p(size_t[e]),
        torch.full_like(fse, float(np.log(t.n))),
        depth_t[s] / 10, depth_t[e] / 10,
        L[s] / 1000, L[e] / 1000, (L[e] - L[s]) / 100, (L[e] - L[s]).abs() / 100,
        (L[pe] - L[e]) / 100, (L[ps] - L[s]) / 100,
        fse, fspe, fse - fspe, amb[s], amb[e], sse,
        (s < t.n).float(), (e < t.n).float(),
        curs / L[s].clamp(min=1), curs / 1000, fsib, fse - fsib, ssib, sse - ssib,
        (pe == e).float(),
        fse * L[s] / 1000, (fse - fsib) * amb[s], (sse - ssib) * L[s] / 1000,
        torch.log1p(size_t[e]) - torch.log1p(size_t[s]), (depth_t[e] - depth_t[s]) / 10,
        (fse - fsib) * (L[e] - L[s]).abs() / 100,
    ]
    X = torch.stack(f, dim=1)
    assert X.shape[1] == NFEAT
    return X


def current_attachment(t: search.Tree, be, S: np.ndarray) -> np.ndarray:
    """Exact distance of every pruned subtree to its current sibling, indexed by node id."""
    cur = np.zeros(len(t.parent), np.int64)
    subs = search.distinct_nodes(S, len(t.parent))
    if len(subs):
        _, _, _, sib = node_info(t, be)
        cur[subs] = be.distances(subs, sib[subs])
    return cur


class Proposal:
    """MLP + feature standardisation; predicts delta = (score - current) / 100."""

    def __init__(self, seed: int = 0, device="cuda"):
        self.net = MLP(seed=seed, device=device)
        self.mu = None
        self.sd = None

    def fit(self, X: torch.Tensor, y: torch.Tensor, epochs=4, batch=4096, lr=1e-3, seed=0):
        self.mu = X.mean(dim=0)
        self.sd = X.std(dim=0).clamp(min=1e-3)
        Z = ((X - self.mu) / self.sd).contiguous()
        return self.net.fit(Z, y.contiguous(), epochs=epochs, batch=batch, lr=lr, seed=seed)

    def predict(self, X: torch.Tensor) -> torch.Tensor:
        Z = ((X - self.mu) / self.sd).contiguous()
        return self.net.predict(Z)


def log_pass(t: search.Tree, be):
    """Features and exact deltas of every candidate of one pass (training data)."""
    S, E = search.spr_candidates(t)
    cur = current_attachment(t, be, S)
    X = features(t, be, S, E, cur)
    score = be.distances(S, E)
    delta = torch.from_numpy(
        (score - cur[S]).astype(np.float32) / 100.0
    ).to(be.dev)
    return X, delta


def learned_scorer(prop: Proposal, be, frac: float = 0.03, min_k: int = 64, stats=None):
    """scorer for search.spr_pass: exact scores for the best-predicted
    fraction of candidates, a large sentinel for the rest."""

    def scorer(t, S, E, cur=None):
        if cur is None:
            cur = current_attachment(t, be, S)
        X = features(t, be, S, E, cur)
        pred = prop.predict(X)
        k = min(len(S), max(min_k, int(frac * len(S))))
        # best-predicted first, ties by candidate index (a stable sort on
        # the device; only the chosen indices come back)
        top = torch.sort(pred, stable=True).indices[:k].cpu().numpy()
        out = np.full(len(S), np.iinfo(np.int64).max // 4, np.int64)
        out[top] = be.distances(S[top], E[top])
        if stats is not None:
            stats["exact"] = stats.get("exact", 0) + k
            stats["candidates"] = stats.get("candidates", 0) + len(S)
        return out

    return scorer


def run_search(t: search.Tree, be, scorer=None, max_passes: int = 30, max_moves: int = 16,
               fallback: bool = True, times=None):
    """SPR passes until a pass accepts nothing (with an exhaustive fallback
    pass when `scorer` is the learned proposal).  Returns (history, seconds);
    `times` (a list) receives the elapsed seconds after every pass."""
    hist = []
    t0 = time.perf_counter()
    diag = None

    def mark(st):
        hist.append(st.cost_after)
        if times is not None:
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)

    for _ in range(max_passes):
        st = search.spr_pass(t, be, max_moves=max_moves, scorer=scorer, diag=diag)
        diag = st.diag
        mark(st)
        if st.moves_accepted == 0:
            if scorer is not None and fallback:
                st = search.spr_pass(t, be, max_moves=max_moves, diag=diag)
                diag = st.diag
                mark(st)
                if st.moves_accepted == 0:
                    break
            else:
                break
    torch.cuda.synchronize()
    return hist, time.perf_counter() - t0


def random_tree(n: int, seed: int) -> search.Tree:
    """A seeded random rooted binary tree (Yule topology, random labels)."""
    from .simulate import yule_tree
    parent = yule_tree(np.random.default_rng(seed), n)
    t = search.Tree(n)
    kids = [[] for _ in range(len(parent))]
    for v, p in enumerate(parent):
        if p >= 0:
            kids[p].append(v)
    for v in range(n, len(parent)):
        t.kids[v] = kids[v]
    t.parent[:len(parent)] = parent
    t.root = len(parent) - 1
    t.free = []
    t.in_tree[:len(parent)] = True
    return t
