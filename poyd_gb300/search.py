"""Candidate-pass driver: Wagner build and SPR passes whose every candidate
join is scored in one batch on the device.

This is the caller side of the hot path (the search-loop integration of
the batched scorer).  The reference evaluates one candidate per call from
``single_spr_round`` (ptree.ml:1120-1176) and ``make_wagner_tree``
(ptree.ml:941-1030) through ``AllDirChar.cost_fn`` -> ``Node.distance``
(node.ml:914-947); here the candidates of a whole pass are collected and
scored together, per character type:

* DO sequences: ``DOS.distance`` (cost_2 with deltaw = max(|la-lb|, 8),
  seqCS.ml:819-867) and ``DOS.median`` (seqCS.ml:747-776) for the downpass;
* non-additive characters: ``NonaddCS8.distance`` / ``median``
  (nonaddCS.ml:119-130);
* Sankoff characters: ``SankCS.distance`` / ``median`` (sankCS.ml:340-377).

The tree is rooted (POY diagnoses from a handle); a node's data is its
downpass (preliminary) median.  A candidate join of subtree ``s`` on the
edge above node ``e`` is scored by the distance between s's data and e's
data -- the quantity ``cost_fn`` adds for a join -- and the exact tree cost
after a join is recomputed by a full batched downpass, which alone decides
acceptance.  Batching a pass changes which improving tree is found first
(the reference accepts sequentially), not the cost of any tree.

:func:`root_costs` diagnoses a tree as the reference reports it: the tree
cost under every rooting (every directed subtree median, then every
edge's root median, batched), the reported cost being the cheapest.

Backends: :class:`GpuBackend` runs the CUDA kernels; the oracle backend in
tests/ implements the same interface on the CPU restatement, so a search
driven through either yields identical trees, costs and node medians.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import align, native
from .simulate import Dataset


# ---------------------------------------------------------------------------
# Tree
# ---------------------------------------------------------------------------
class Tree:
    """Rooted binary tree over leaves 0..n-1; internal ids from n upward."""

    def __init__(self, n_leaves: int):
        self.n = n_leaves
        cap = 2 * n_leaves
        self.parent = -np.ones(cap, dtype=np.int64)
        self.kids = -np.ones((cap, 2), dtype=np.int64)
        self.root = -1
        self.free = list(range(2 * n_leaves - 2, n_leaves - 1, -1))
        self.in_tree = np.zeros(cap, dtype=bool)

    def copy(self) -> "Tree":
        t = Tree.__new__(Tree)
        t.n = self.n
        t.parent = self.parent.copy()
        t.kids = self.kids.copy()
        t.root = self.root
        t.free = list(self.free)
        t.in_tree = self.in_tree.copy()
        return t

    def _new_internal(self) -> int:
        return self.free.pop()

    def start(self, a: int, b: int):
        w = self._new_internal()
        self.kids[w] = (a, b)
        self.parent[a] = self.parent[b] = w
        self.parent[w] = -1
        self.root = w
        self.in_tree[[a, b, w]] = True

    def insert(self, t: int, e: int, w: int | None = None) -> int:
        """Join node t on the edge above e through a new internal node w."""
        if w is None:
            w = self._new_internal()
        p = self.parent[e]
        self.kids[w] = (e, t)
        self.parent[w] = p
        self.parent[e] = w
        self.parent[t] = w
        if p < 0:
            self.root = w
        else:
            k = self.kids[p]
            k[0 if k[0] == e else 1] = w
        self.in_tree[[t, w]] = True
        return w

    def prune(self, s: int) -> int:
        """Detach the subtree under s; returns its freed parent node."""
        p = self.parent[s]
        assert p >= 0, "cannot prune the root"
        o = self.kids[p][0] if self.kids[p][1] == s else self.kids[p][1]
        g = self.parent[p]
        self.parent[o] = g
        if g < 0:
            self.root = o
        else:
            k = self.kids[g]
            k[0 if k[0] == p else 1] = o
        self.parent[p] = -1
        self.parent[s] = -1
        self.kids[p] = (-1, -1)
        self.in_tree[p] = False
        return p

    def reroot(self, s: int, u: int):
        """Re-roots the subtree under s on the edge above u (u inside it,
        u's parent not s): s keeps its id and becomes the midpoint of that
        edge, the path from u's parent up to s is reversed and s's old
        other child hangs from the path's top.  ``Tree_Ops.reroot_fn`` on
        a clade (ptree.ml:1179-1181)."""
        path = [u]
        while self.parent[path[-1]] != s:
            path.append(int(self.parent[path[-1]]))
        assert len(path) >= 2, "u must lie below a child of s"
        top = path[-1]
        sib = int(self.kids[s][0] if self.kids[s][1] == top else self.kids[s][1])
        other = []
        for j in range(1, len(path)):
            k = self.kids[path[j]]
            other.append(int(k[0] if k[1] == path[j - 1] else k[1]))
        self.kids[s] = (path[0], path[1])
        self.parent[path[0]] = s
        self.parent[path[1]] = s
        for j in range(1, len(path)):
            nxt = path[j + 1] if j + 1 < len(path) else sib
            self.kids[path[j]] = (other[j - 1], nxt)
            self.parent[other[j - 1]] = path[j]
            self.parent[nxt] = path[j]

    def _memo(self, name, fn):
        """fn() cached until the tree's root or children change (compared
        exactly; trees are also built by writing the arrays directly)."""
        key = (int(self.root), self.kids.tobytes())
        memo = self.__dict__.setdefault("_cache", {})
        hit = memo.get(name)
        if hit is not None and hit[0] == key:
            return hit[1]
        val = fn()
        memo[name] = (key, val)
        return val

    def nodes(self):
        """Preorder (a node before its children, the second child first).
        The list is shared by later calls on the same tree: do not modify it."""
        def walk():
            kids, n = self.kids.tolist(), self.n
            out, stack = [], [int(self.root)]
            while stack:
                v = stack.pop()
                out.append(v)
                if v >= n:
                    stack.extend(kids[v])
            return out
        return self._memo("nodes", walk)

    def subtree(self, s: int):
        out, stack = [], [s]
        while stack:
            v = stack.pop()
            out.append(v)
            if v >= self.n:
                stack.extend(self.kids[v])
        return out

    def min_codes(self) -> np.ndarray:
        """Smallest leaf id under every node (POY's ``min_child_code``,
        node.ml:674; a leaf's is its own taxon code)."""
        def compute():
            kids, n = self.kids.tolist(), self.n
            mc = list(range(len(self.parent)))
            for v in self.nodes()[::-1]:
                if v >= n:
                    a, b = kids[v]
                    mc[v] = min(mc[a], mc[b])
            return np.array(mc, np.int64)
        return self._memo("min_codes", compute).copy()

    def levels(self):
        """Internal nodes grouped by height (all children before parents)."""
        kids, n = self.kids.tolist(), self.n
        h = {}
        order = self.nodes()[::-1]
        for v in order:
            if v < n:
                h[v] = 0
            else:
                a, b = kids[v]
                h[v] = 1 + max(h[a], h[b])
        groups = {}
        for v in order:
            if v >= self.n:
                groups.setdefault(h[v], []).append(v)
        return [sorted(groups[k]) for k in sorted(groups)]

    def newick(self, names=None) -> str:
        def rec(v):
            if v < self.n:
                return names[v] if names else str(v)
            a, b = self.kids[v]
            return "(%s,%s)" % (rec(a), rec(b))
        return rec(self.root) + ";"


# ---------------------------------------------------------------------------
# GPU backend
# ---------------------------------------------------------------------------
def distinct_nodes(ids, n_slots: int) -> np.ndarray:
    """The distinct node ids among `ids`, ascending (what np.unique gives),
    from a mark array over the n_slots node ids instead of a sort: the
    candidate lists of a pass name each node many times."""
    seen = np.zeros(n_slots, bool)
    seen[np.asarray(ids, np.int64)] = True
    return np.flatnonzero(seen)


def either_empty(a, b, n_slots: int, empty) -> np.ndarray:
    """Per pair whether node a_i or b_i is all gaps.  ``empty(v)`` answers
    for an ascending array of distinct node ids and is asked once per node
    the pairs name, found with a mark array over the n_slots node ids
    rather than a sort of the 2n ids."""
    a = np.asarray(a, np.int64)
    b = np.asarray(b, np.int64)
    seen = np.zeros(n_slots, bool)
    seen[a] = True
    seen[b] = True
    u = np.flatnonzero(seen)
    e = np.zeros(n_slots, bool)
    if len(u):
        e[u] = empty(u)
    return e[a] | e[b]


def _p(t):
    return C.c_void_p(t.data_ptr())


class GpuBackend:
    """Node data resident in HBM: DO medians in a byte pool, Fitch rows,
    Sankoff cost vectors; every batch is a few kernel launches."""

    def __init__(self, data: Dataset, cm: align.CostMatrix, device="cuda"):
        self.dev = torch.device(device)
        self.cm = cm
        self.n = data.n_taxa
        n_nodes = 2 * self.n
        self.nf = data.fitch.shape[1]
        self.stride = max(16, (self.nf + 15) // 16 * 16)
        self.ns, self.k = data.sank.shape[1], data.sank.shape[2]
        fit = np.zeros((n_nodes, self.stride), np.uint8)
        fit[:self.n, :self.nf] = data.fitch
        self.fitch = torch.from_numpy(fit).to(self.dev)
        sk = np.zeros((n_nodes, max(self.ns, 1), self.k), np.int32)
        sk[:self.n, :self.ns] = data.sank
        self.sank = torch.from_numpy(sk).to(self.dev)
        self.tcm = torch.from_numpy(np.ascontiguousarray(data.sank_tcm, np.int32)).to(self.dev)
        total = sum(len(s) for s in data.seqs)
        # the level engine leaves each median inside its four-sequence
        # result slot (about 8x a sequence's bytes); compaction reclaims
        # the rest
        self.pool = torch.zeros(max(64 << 20, 64 * total), dtype=torch.uint8, device=self.dev)
        self.off = np.zeros(n_nodes, np.int64)
        self.len = np.zeros(n_nodes, np.int32)
        self.top = 0
        for v, s in enumerate(data.seqs):
            self._put(v, torch.from_numpy(np.asarray(s, np.uint8)).to(self.dev))
        self.stats = {"median_pairs": 0, "distance_pairs": 0, "do_cells": 0}

    # -- sequence pool -------------------------------------------------------
    def _reserve(self, nbytes: int) -> int:
        if self.top + nbytes > self.pool.numel():
            self._compact(extra=nbytes)
        o = self.top
        self.top += nbytes
        return o

    def _compact(self, extra: int = 0):
        """Moves every live sequence to the front of a fresh pool with room
        for `extra` more bytes (one gather on the device)."""
        live = np.flatnonzero(self.len > 0)
        ln = self.len[live].astype(np.int64)
        top = int(ln.sum())
        newpool = torch.zeros(max(2 * (top + extra), self.pool.numel()), dtype=torch.uint8,
                              device=self.dev)
        if top:
            dst = np.cumsum(ln) - ln
            src = np.repeat(self.off[live] - dst, ln) + np.arange(top, dtype=np.int64)
            newpool[:top] = self.pool[torch.from_numpy(src).to(self.dev)]
            self.off[live] = dst
        self.pool, self.top = newpool, top

    def _put(self, v: int, seq: torch.Tensor):
        o = self._reserve(seq.numel())
        self.pool[o:o + seq.numel()] = seq
        self.off[v], self.len[v] = o, seq.numel()

    def _batch(self, a, b) -> align.PairBatch:
        t = lambda x, dt: torch.from_numpy(np.ascontiguousarray(x, dt)).to(self.dev)
        return align.PairBatch(self.pool, t(self.off[a], np.int64), t(self.len[a], np.int32),
                               t(self.off[b], np.int64), t(self.len[b], np.int32))

    # -- batched operations -------------------------------------------------
    def medians(self, a: np.ndarray, b: np.ndarray, out: np.ndarray):
        """Downpass medians of (a_i, b_i) into nodes out_i; returns the DO
        and Fitch costs of each median (numpy int64)."""
        return self.median_levels([(a, b, out)])[0]

    def median_levels(self, levels):
        """Several dependent levels of downpass medians in one call of the
        level engine (``poyd_median_levels``): `levels` lists (a, b, out)
        node-id arrays; a level's inputs are existing nodes or outputs of
        earlier levels.  Returns [(DO costs, Fitch costs)] per level."""
        sizes = [len(lv[0]) for lv in levels]
        n = int(sum(sizes))
        if n == 0:
            return [(np.zeros(0, np.int64), np.zeros(0, np.int64)) for _ in levels]
        start = np.zeros(len(levels) + 1, np.int32)
        start[1:] = np.cumsum(sizes)
        cat = lambda k: np.ascontiguousarray(np.concatenate(
            [np.asarray(lv[k], np.int64) for lv in levels]).astype(np.int32))
        A, B, O = cat(0), cat(1), cat(2)
        costs = np.zeros(2 * n, np.int64)
        st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        L = native.lib()
        for attempt in range(2):
            store = native.PoydNodeStore(
                pool=self.pool.data_ptr(), pool_size=self.pool.numel(),
                fitch=self.fitch.data_ptr(), fitch_stride=self.stride, fitch_len=self.nf,
                sank_nchar=self.ns, sank=self.sank.data_ptr(), sank_tcm=self.tcm.data_ptr(),
                sank_k=self.k, pad=0)
            top, need = C.c_int64(self.top), C.c_int64(0)
            rc = L.poyd_median_levels(self.cm.ref, C.byref(store), len(self.len),
                                      self.off.ctypes.data, self.len.ctypes.data, len(levels),
                                      start.ctypes.data, A.ctypes.data, B.ctypes.data,
                                      O.ctypes.data, C.byref(top), C.byref(need),
                                      costs.ctypes.data, st)
            if rc == native.ESPACE and attempt == 0:
                self._compact(extra=int(need.value))
                continue
            native.check(rc)
            break
        self.top = int(top.value)
        self.stats["median_pairs"] += n
        c = costs.reshape(n, 2)
        return [(c[start[l]:start[l + 1], 0].copy(), c[start[l]:start[l + 1], 1].copy())
                for l in range(len(levels))]

    def _store(self, res: align.AlignResult, out, extra=None):
        """Moves each pair's fourth output sequence (the median, or the
        single sequence of ``closest``) into the pool as node out_i; one
        transfer brings the lengths, the costs and `extra` to the host.
        Returns (costs, extra) as numpy int64."""
        n = len(out)
        ln = res.out_len.view(-1, 2)[:, 1].to(torch.int64)
        parts = [ln, res.cost.to(torch.int64)] + ([extra] if extra is not None else [])
        host = torch.cat(parts).cpu().numpy()
        lens, cost = host[:n], host[n:2 * n]
        if n and lens.min() < 0:
            raise native.PoydError(-3, "traceback failed (code %d)" % int(lens.min()))
        src = res.out_off + 4 * res.cap - ln
        total = int(lens.sum())
        dst_off = self._reserve(total) + np.cumsum(lens) - lens
        seg = torch.repeat_interleave(torch.arange(n, device=self.dev), ln)
        starts = torch.cumsum(ln, 0) - ln
        pos = torch.arange(total, device=self.dev) - starts[seg]
        dst = torch.from_numpy(dst_off).to(self.dev)
        self.pool[dst[seg] + pos] = res.out[src[seg] + pos]
        self.off[out], self.len[out] = dst_off, lens.astype(np.int32)
        return cost, (host[2 * n:] if extra is not None else None)

    def singles(self, parent: np.ndarray, node: np.ndarray, out: np.ndarray):
        """Final-state sequences: out_i = closest(parent_i, node_i)
        (``DOS.to_single``); Fitch and Sankoff rows are not assigned."""
        if len(out) == 0:
            return
        self._store(align.closest(self._batch(parent, node), self.cm, dos_empty=True), out)

    def _empty(self, v: np.ndarray) -> np.ndarray:
        """Whether each node's sequence is all gaps (``Sequence.is_empty``)."""
        v = np.asarray(v, np.int64)
        ln = self.len[v].astype(np.int64)
        t = lambda x: torch.from_numpy(np.ascontiguousarray(x)).to(self.dev)
        seg = torch.repeat_interleave(torch.arange(len(v), device=self.dev), t(ln))
        pos = torch.arange(int(ln.sum()), device=self.dev) - t(np.cumsum(ln) - ln)[seg]
        idx = t(self.off[v])[seg] + pos
        nongap = torch.zeros(len(v), dtype=torch.int64, device=self.dev).index_add_(
            0, seg, (self.pool[idx] != self.cm.gap).to(torch.int64))
        return (nongap == 0).cpu().numpy()

    def do_distances(self, a: np.ndarray, b: np.ndarray) -> np.ndarray:
        """``DOS.distance`` (seqCS.ml:819-867) alone between nodes a_i, b_i,
        with missing distance 0 where either is all gaps."""
        a = np.asarray(a, np.int64)
        b = np.asarray(b, np.int64)
        do, _ = align.cost_2(self._batch(a, b), self.cm, deltaw="dos")
        e = either_empty(a, b, len(self.len), self._empty)
        do = do.to(torch.int64).cpu().numpy()
        do[e] = 0
        return do

    def rebind_nodes(self, dst: np.ndarray, src: np.ndarray):
        """Nodes dst take over the medians computed into nodes src (the
        scratch slots of an evaluated move)."""
        dst = np.asarray(dst, np.int64)
        src = np.asarray(src, np.int64)
        self.off[dst], self.len[dst] = self.off[src], self.len[src]
        d = torch.from_numpy(dst).to(self.dev)
        s = torch.from_numpy(src).to(self.dev)
        if self.nf:
            self.fitch[d] = self.fitch[s]
        if self.ns:
            self.sank[d] = self.sank[s]

    def distances(self, a: np.ndarray, b: np.ndarray) -> np.ndarray:
        """Candidate-join distance d(a_i, b_i) = DOS.distance + Fitch + Sankoff,
        with the join cost's missing distance 0 for an all-gap sequence
        (``Node.Standard.distance 0.``, allDirChar.ml:1305-1316)."""
        n = len(a)
        st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        L = native.lib()
        ia = torch.from_numpy(np.asarray(a, np.int32)).to(self.dev)
        ib = torch.from_numpy(np.asarray(b, np.int32)).to(self.dev)
        do, cells = align.cost_2(self._batch(a, b), self.cm, deltaw="dos", band_cells=True)
        tot = do.to(torch.int64)
        e = either_empty(a, b, len(self.len), self._empty)
        if e.any():
            tot = tot * torch.from_numpy((~e).astype(np.int64)).to(self.dev)
        if self.nf:
            fd = torch.empty(n, dtype=torch.int64, device=self.dev)
            native.check(L.poyd_nonadd8_distance_batch(_p(self.fitch), C.c_int64(self.stride), self.nf,
                                                       n, _p(ia), _p(ib), _p(fd), st))
            tot = tot + fd
        if self.ns:
            sd = torch.empty(n, dtype=torch.int64, device=self.dev)
            native.check(L.poyd_sank_distance_batch(_p(self.sank), self.ns, self.k, _p(self.tcm), n,
                                                    _p(ia), _p(ib), _p(sd), st))
            tot = tot + sd
        self.stats["distance_pairs"] += n
        self.stats["do_cells"] += int(cells.sum().item())
        return tot.cpu().numpy()

    def ensure_nodes(self, n_nodes: int):
        """Room for node ids < n_nodes (scratch ids of move evaluation)."""
        have = self.fitch.shape[0]
        if n_nodes <= have:
            return
        grow = max(n_nodes, 2 * have)
        f = torch.zeros((grow, self.stride), dtype=torch.uint8, device=self.dev)
        f[:have] = self.fitch
        sk = torch.zeros((grow,) + tuple(self.sank.shape[1:]), dtype=torch.int32, device=self.dev)
        sk[:have] = self.sank
        self.fitch, self.sank = f, sk
        self.off = np.concatenate([self.off, np.zeros(grow - have, np.int64)])
        self.len = np.concatenate([self.len, np.zeros(grow - have, np.int32)])

    def release_nodes(self, first: int):
        """Forget scratch node ids >= first (their pool bytes are reclaimed
        at the next compaction)."""
        self.len[first:] = 0

    def sank_costs(self, vs) -> np.ndarray:
        """Sankoff root costs of several nodes, one read-back."""
        vs = np.asarray(vs, np.int64)
        if not self.ns or len(vs) == 0:
            return np.zeros(len(vs), np.int64)
        s = self.sank[torch.from_numpy(vs).to(self.dev)]
        c = torch.clamp(s.min(dim=2).values, max=native.SANK_INF).to(torch.int64).sum(dim=1)
        return c.cpu().numpy()

    def sank_cost(self, v: int) -> int:
        if not self.ns:
            return 0
        s = self.sank[v]
        return int(torch.clamp(s.min(dim=1).values, max=native.SANK_INF).to(torch.int64).sum().item())

    # -- final states of the non-DO characters (uppass) ---------------------
    def final_slots(self, n_slots: int, fitch_base: int):
        """Room for n_slots final states: Fitch finals in node rows
        fitch_base + slot (the median_3 kernel reads ancestors from the node
        rows), Sankoff finals (e rows, best-state bits) in their own arrays."""
        self.ensure_nodes(fitch_base + n_slots)
        self.fin_base = fitch_base
        if self.ns:
            self.fin_e = torch.zeros((n_slots, self.ns, self.k), dtype=torch.int32, device=self.dev)
            self.fin_best = torch.zeros((n_slots, self.ns), dtype=torch.int32, device=self.dev)

    def final_root(self, node: int, slot: int):
        """The root's final: its preliminary state (a median's final is its
        preliminary, node.ml:270-290); a Sankoff root's best states are its
        cheapest states (elt_median_3 takes them when none are set,
        sankCS.ml:423-436)."""
        if self.nf:
            self.fitch[self.fin_base + slot] = self.fitch[node]
        if self.ns:
            s = self.sank[node, :self.ns]
            mn = s.min(dim=1, keepdim=True).values
            self.fin_e[slot] = torch.where(s >= native.SANK_INF, native.SANK_INF, s - mn)
            bits = (s == mn).to(torch.int32) << torch.arange(self.k, device=self.dev, dtype=torch.int32)
            self.fin_best[slot] = bits.sum(dim=1).to(torch.int32)

    def final_states(self, anc, node, left, right, out):
        """Finals of slots out_i from the ancestors' finals (slots anc_i), the
        nodes' preliminary states and their children's (node ids; a leaf
        passes itself): NonaddCS median_3 (nonaddCSc.c:472-544) and SankCS
        median_3 (sankCS.ml:402-452), as node.ml's cs_median_3 (459-486)."""
        n = len(out)
        if n == 0:
            return
        st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        L = native.lib()
        t = lambda x: torch.from_numpy(np.ascontiguousarray(x, np.int32)).to(self.dev)
        ia, inode, il, ir = t(anc), t(node), t(left), t(right)
        io = torch.from_numpy(np.asarray(out, np.int64)).to(self.dev)
        if self.nf:
            tmp = torch.empty((n, self.stride), dtype=torch.uint8, device=self.dev)
            native.check(L.poyd_nonadd8_median_3_batch(
                _p(self.fitch), C.c_int64(self.stride), self.nf, n, _p(ia + self.fin_base),
                _p(inode), _p(il), _p(ir), _p(tmp), st))
            self.fitch[io + self.fin_base] = tmp
        if self.ns:
            e = torch.empty((n, self.ns, self.k), dtype=torch.int32, device=self.dev)
            b = torch.empty((n, self.ns), dtype=torch.int32, device=self.dev)
            native.check(L.poyd_sank_median_3_batch(
                _p(self.sank), _p(self.fin_e), _p(self.fin_best), self.ns, self.k, _p(self.tcm),
                n, _p(ia), _p(inode), _p(il), _p(ir), _p(e), _p(b), st))
            self.fin_e[io] = e
            self.fin_best[io] = b

    def node_final(self, slot: int):
        """(Fitch final row, Sankoff final e rows, best-state bits) of a slot."""
        f = self.fitch[self.fin_base + slot, :self.nf].cpu().numpy() if self.nf else \
            np.zeros(0, np.uint8)
        if self.ns:
            return f, self.fin_e[slot].cpu().numpy(), self.fin_best[slot].cpu().numpy()
        return f, np.zeros((0, self.k), np.int32), np.zeros(0, np.int32)

    def node_seq(self, v: int) -> np.ndarray:
        o, l = int(self.off[v]), int(self.len[v])
        return self.pool[o:o + l].cpu().numpy()

    def put_seqs(self, out, seqs):
        """Host sequences into the pool as nodes out_i (one upload)."""
        out = np.asarray(out, np.int64)
        lens = np.array([len(x) for x in seqs], np.int64)
        if not len(out):
            return
        dst = self._reserve(int(lens.sum()))
        self.pool[dst:dst + int(lens.sum())] = torch.from_numpy(
            np.concatenate([np.asarray(x, np.uint8) for x in seqs])).to(self.dev)
        self.off[out] = dst + np.cumsum(lens) - lens
        self.len[out] = lens.astype(np.int32)

    def readjust(self, ch1, ch2, par, mine, out, mode: str = "three"):
        """``DOS.readjust`` (seqCS.ml:680-722) of nodes mine_i from their
        neighbours (ch1_i, ch2_i, par_i), the Iterative mode's ThreeD or
        ApproxD, into nodes out_i; returns (changed, costs)."""
        from . import iterative, three
        ch1, ch2, par, mine, out = (np.asarray(x, np.int64) for x in (ch1, ch2, par, mine, out))
        n = len(out)
        changed = np.zeros(n, bool)
        costs = np.zeros(n, np.int64)
        host = np.arange(n)
        if mode == "three" and n:
            # no empty neighbour: readjust_3d on the pool's own bytes, the
            # medians moved back into the pool on the device
            emp = self._empty(np.concatenate([ch1, ch2, par])).reshape(3, n).any(axis=0)
            dev = np.flatnonzero(~emp)
            host = np.flatnonzero(emp)
            if len(dev):
                t = lambda x, dt: torch.from_numpy(np.ascontiguousarray(x, dt)).to(self.dev)
                ids = (ch1[dev], ch2[dev], mine[dev], par[dev])
                batch = three.TripleBatch(self.pool, [t(self.off[x], np.int64) for x in ids],
                                          [t(self.len[x], np.int32) for x in ids])
                r = three.readjust_3d(batch, self.cm)
                c, ch = self._store(r, out[dev], r.changed.to(torch.int64))
                costs[dev], changed[dev] = c, ch.astype(bool)
        if len(host):
            items = [(self.node_seq(int(ch1[i])), self.node_seq(int(ch2[i])),
                      self.node_seq(int(par[i])), self.node_seq(int(mine[i]))) for i in host]
            res = iterative.dos_readjust(items, self.cm, mode)
            self.put_seqs(out[host], [x[1] for x in res])
            changed[host] = [x[0] for x in res]
            costs[host] = [x[2] for x in res]
        return changed, costs

    def node_fitch(self, v: int) -> np.ndarray:
        return self.fitch[v, :self.nf].cpu().numpy()

    def node_sank(self, v: int) -> np.ndarray:
        return self.sank[v, :self.ns].cpu().numpy()


# ---------------------------------------------------------------------------
# Diagnosis and search
# ---------------------------------------------------------------------------
@dataclass
class Diagnosis:
    do_cost: dict = field(default_factory=dict)
    fitch_cost: dict = field(default_factory=dict)
    total: int = 0


def _by_code(a, b, mc):
    """Median argument order of ``Node.cs_median`` (node.ml:344-349): the
    child holding the smaller taxon code first (DO medians break ties by
    argument order)."""
    a = np.asarray(a, np.int64)
    b = np.asarray(b, np.int64)
    sw = np.asarray(mc[a] > mc[b])
    return np.where(sw, b, a), np.where(sw, a, b)


def downpass(tree: Tree, be, nodes=None) -> Diagnosis:
    """Preliminary medians of every internal node, one batch per height."""
    d = Diagnosis()
    mc = tree.min_codes()
    levels = []
    for level in tree.levels():
        lv = np.array(level, np.int64)
        a, b = _by_code(tree.kids[lv, 0], tree.kids[lv, 1], mc)
        levels.append((a, b, lv))
    for (_, _, lv), (do, fi) in zip(levels, be.median_levels(levels)):
        for i, v in enumerate(lv.tolist()):
            d.do_cost[v] = int(do[i])
            d.fitch_cost[v] = int(fi[i])
    d.total = sum(d.do_cost.values()) + sum(d.fitch_cost.values()) + be.sank_cost(tree.root)
    return d


def wagner(n: int, be, order=None, log=None):
    """make_wagner_tree (ptree.ml:941-1030): add taxa one at a time at the
    edge whose join distance is smallest (ties: lowest node id)."""
    order = list(range(n)) if order is None else list(order)
    t = Tree(n)
    t.start(order[0], order[1])
    downpass(t, be)
    for x in order[2:]:
        cand = np.array(sorted(t.nodes()), np.int64)
        d = be.distances(np.full(len(cand), x, np.int64), cand)
        if log is not None:
            log.append((x, cand, d))
        e = int(cand[int(np.argmin(d))])
        t.insert(x, e)
        downpass(t, be)
    return t, downpass(t, be)


@dataclass
class PassStats:
    candidates: int = 0
    moves_tried: int = 0
    moves_accepted: int = 0
    cost_before: int = 0
    cost_after: int = 0
    seconds_scoring: float = 0.0
    seconds_total: float = 0.0
    diag: Diagnosis | None = None  # diagnosis of the tree after the pass


def euler(t: Tree):
    """Preorder entry / exit times: u is in subtree(v) iff tin[v] <= tin[u] < tout[v]
    (cached per tree state; do not modify the arrays)."""
    return t._memo("euler", lambda: _euler(t))


def _euler(t: Tree):
    cap, n = len(t.parent), t.n
    kids = t.kids.tolist()
    tin = [0] * cap
    tout = [0] * cap
    clock = 0
    stack = [(int(t.root), 0)]
    while stack:
        v, state = stack.pop()
        if state == 0:
            tin[v] = clock
            clock += 1
            stack.append((v, 1))
            if v >= n:
                a, b = kids[v]
                stack.append((b, 0))
                stack.append((a, 0))
        else:
            tout[v] = clock
    return np.array(tin, np.int64), np.array(tout, np.int64)


def spr_candidates(t: Tree):
    """Every (pruned subtree s, join edge e) of one SPR pass: s ranges over
    non-root nodes whose parent is not the root, e over the nodes left after
    pruning s, except s's old parent and sibling (the unchanged tree)."""
    nodes = np.array(sorted(t.nodes()), np.int64)
    par = t.parent
    pn = par[nodes]
    subs = nodes[(pn >= 0) & (par[np.maximum(pn, 0)] >= 0)]
    if len(subs) == 0:
        return np.zeros(0, np.int64), np.zeros(0, np.int64)
    tin, tout = euler(t)
    p = par[subs]
    sib = np.where(t.kids[p, 0] == subs, t.kids[p, 1], t.kids[p, 0])
    # one (subtree x node) mask; rows in subtree order, nodes ascending
    tn = tin[nodes][None, :]
    keep = ~((tn >= tin[subs][:, None]) & (tn < tout[subs][:, None]))
    keep &= (nodes[None, :] != p[:, None]) & (nodes[None, :] != sib[:, None])
    return np.repeat(subs, keep.sum(axis=1)), np.broadcast_to(nodes, keep.shape)[keep]


def spr_pass(t: Tree, be, max_moves: int = 16, scorer=None, log=None, diag=None):
    """One SPR pass: score every candidate join in one batch (or through
    `scorer`, which may score a subset), then try the best-scoring moves in
    order; a move is kept only if the exact re-diagnosed tree cost drops.
    `diag` may carry the current tree's diagnosis (a previous pass's
    `PassStats.diag`) to skip the initial downpass."""
    t0 = time.perf_counter()
    st = PassStats()
    diag = downpass(t, be) if diag is None else diag
    st.cost_before = diag.total
    S, E = spr_candidates(t)
    st.candidates = len(S)
    t1 = time.perf_counter()
    # the cost of each subtree where it is now: distance to its sibling
    subs = distinct_nodes(S, len(t.parent))
    cur = np.zeros(len(t.parent), np.int64)
    if len(subs):
        p = t.parent[subs]
        sib = np.where(t.kids[p, 0] == subs, t.kids[p, 1], t.kids[p, 0])
        cur[subs] = be.distances(subs, sib)
    # a scorer receives those attachment costs (indexed by node id) too
    score = be.distances(S, E) if scorer is None else scorer(t, S, E, cur)
    st.seconds_scoring = time.perf_counter() - t1
    if log is not None:
        log.append((t.copy(), S, E, score))
    gain = cur[S] - score
    # largest predicted gain first, ties by ids; only improving candidates
    # can become moves, so only they are sorted
    pos = np.nonzero(gain > 0)[0]
    order = pos[np.lexsort((E[pos], S[pos], -gain[pos]))]
    moves, seen = [], set()
    for i in order:
        if len(moves) >= max_moves:
            break
        s, e = int(S[i]), int(E[i])
        if s not in seen:
            seen.add(s)
            moves.append((s, e))
    # Rounds: the exact cost of every remaining move is computed in one
    # batched incremental diagnosis; the best improving move is applied and
    # the tree re-diagnosed; moves no longer valid are dropped.
    # The accepted move's recomputed medians become the tree's own (no
    # re-diagnosis per move); one full downpass at the end of the pass
    # checks the incremental totals.
    best = diag.total
    while moves:
        st.moves_tried += len(moves)
        detail = {}
        totals = evaluate_moves(t, be, diag, moves, detail)
        k = int(np.argmin(totals))
        if totals[k] >= best:
            be.release_nodes(2 * t.n)
            break
        s, e = moves.pop(k)
        t.insert(s, e, t.prune(s))
        commit_move(be, diag, detail[k], totals[k])
        be.release_nodes(2 * t.n)
        best = int(totals[k])
        st.moves_accepted += 1
        moves = [(a, b) for a, b in moves if _valid_move(t, a, b)]
    if st.moves_accepted:
        check = downpass(t, be)
        assert check.total == best, (check.total, best)
        diag = check
    st.cost_after = best
    st.diag = diag
    st.seconds_total = time.perf_counter() - t0
    return st


def tbr_candidates(t: Tree, be, diag: Diagnosis | None = None):
    """Every TBR candidate of one pass, scored in one batch: (pruned
    subtree s, re-root node u, join edge e, score, clade cost change).
    ``tbr_join`` (ptree.ml:1178-1217) breaks the edge above s and runs an
    SPR round of the clade for each of its re-rootings (``reroot_fn``),
    joining by the clade's root median.  Here, for every clade together:

    * the medians of the clade seen from inside, looking up towards s
      (up(w) = median(up(parent), sibling's downpass median)), one batch
      per depth below s;
    * the root median of every re-rooting on the edge above w
      (median(w's downpass median, up(w))), one batch;
    * the distance of every (re-rooted clade, join edge) pair, one batch.

    The clade cost change is the clade's own cost rooted on the edge above
    u (the costs of those medians plus the downpass costs below them)
    minus its cost as rooted now: a re-rooting changes it, a join does not.
    u = -1 is the clade's own rooting (plain SPR: its sibling edge is
    excluded).  Medians take their arguments in ``min_child_code`` order.
    Scratch node ids from 2 * t.n are released on return."""
    n = t.n
    diag = downpass(t, be) if diag is None else diag
    mc = t.min_codes()
    par = t.parent
    nodes = np.array(sorted(t.nodes()), np.int64)
    # downpass cost of every subtree (DO + Fitch)
    tot = np.zeros(len(par), np.int64)
    for v in t.nodes()[::-1]:
        if v >= n:
            a, b = t.kids[v]
            tot[v] = tot[a] + tot[b] + diag.do_cost[v] + diag.fitch_cost[v]
    subs = [int(v) for v in nodes if par[v] >= 0 and par[par[v]] >= 0]
    nxt = 2 * n
    cand = []        # (s, u, node holding the clade's root median, clade cost change)
    fronts = {}      # s -> [(node, id of up(node), min code of up(node), cost of up(node))]
    for s in subs:
        cand.append((s, -1, s, 0))
        if s >= n:
            k0, k1 = int(t.kids[s][0]), int(t.kids[s][1])
            fronts[s] = [(k0, k1, int(mc[k1]), int(tot[k1])), (k1, k0, int(mc[k0]), int(tot[k0]))]
    size = np.zeros(len(par), np.int64)  # nodes per subtree
    for v in t.nodes()[::-1]:
        size[v] = 1 if v < n else 1 + size[t.kids[v][0]] + size[t.kids[v][1]]
    # two medians (up, root) for every clade node below the clade's children
    be.ensure_nodes(nxt + sum(2 * (int(size[s]) - 3) for s in fronts))
    # The medians' node ids do not depend on their costs: every depth's up
    # medians and then all root medians are laid out first (ids in the
    # order depth by depth, each depth's up medians before its roots) and
    # computed in one call of dependent levels.  A front entry is (node,
    # id of up(node), min code of up(node), job computing up(node) or -1,
    # constant part of its cost); a job's cost below its median is its
    # entry's cost plus the sibling subtree's downpass cost.
    fronts = {s: [(u, up, upmc, -1, upc) for u, up, upmc, upc in f] for s, f in fronts.items()}
    levels = []      # per depth: (a, b, out) of the up medians
    jobs = []        # per up median: (parent job or -1, constant cost below it)
    roots = []       # (a, b, out, s, u, job of up(u))
    while fronts:
        lvl, entries = [], []
        for s, front in fronts.items():
            for u, upid, upmc, pj, pc in front:
                if u < n:
                    continue
                for w in (int(t.kids[u][0]), int(t.kids[u][1])):
                    x = int(t.kids[u][0] if t.kids[u][1] == w else t.kids[u][1])
                    lvl.append((upid, x, nxt) if upmc < mc[x] else (x, upid, nxt))
                    jobs.append((pj, pc + int(tot[x])))
                    entries.append((s, w, nxt, min(upmc, int(mc[x])), len(jobs) - 1))
                    nxt += 1
        if not lvl:
            break
        levels.append(np.array(lvl, np.int64))
        fronts = {}
        for s, w, wid, wmc, ji in entries:
            fronts.setdefault(s, []).append((w, wid, wmc, ji, 0))
            a, b = (w, wid) if mc[w] < wmc else (wid, w)
            roots.append((a, b, nxt, s, w, ji))
            nxt += 1
    if roots:
        r = np.array([x[:3] for x in roots], np.int64)
        res = be.median_levels([(j[:, 0], j[:, 1], j[:, 2]) for j in levels] +
                               [(r[:, 0], r[:, 1], r[:, 2])])
        upc = np.zeros(len(jobs), np.int64)
        k = 0
        for do, fi in res[:-1]:
            for i in range(len(do)):
                pj, pc = jobs[k]
                upc[k] = pc + (upc[pj] if pj >= 0 else 0) + int(do[i]) + int(fi[i])
                k += 1
        do, fi = res[-1]
        for i, (_, _, rid, s, w, ji) in enumerate(roots):
            below = int(tot[w]) + int(upc[ji])
            cand.append((s, w, rid, below + int(do[i]) + int(fi[i]) - int(tot[s])))
    # join edges: outside the clade, not its parent, not (own rooting) its
    # sibling; one (candidate x node) mask, rows in candidate order
    tin, tout = euler(t)
    cs, cu, cr, cd = (np.array([c[i] for c in cand], np.int64).reshape(-1) for i in range(4))
    p = par[cs]
    sib = np.where(t.kids[p, 0] == cs, t.kids[p, 1], t.kids[p, 0])
    tn = tin[nodes][None, :]
    keep = ~((tn >= tin[cs][:, None]) & (tn < tout[cs][:, None]))
    keep &= nodes[None, :] != p[:, None]
    keep &= ~((cu < 0)[:, None] & (nodes[None, :] == sib[:, None]))
    cnt = keep.sum(axis=1)
    S, U, R, D = (np.repeat(x, cnt) for x in (cs, cu, cr, cd))
    E = np.broadcast_to(nodes, keep.shape)[keep]
    score = be.distances(R, E) if len(S) else np.zeros(0, np.int64)
    be.release_nodes(2 * n)
    return S, U, E, score, D


def tbr_pass(t: Tree, be, max_moves: int = 16, log=None, diag=None):
    """One TBR pass: every (clade, re-rooting, join edge) candidate scored
    in one batch (:func:`tbr_candidates`), then the best-scoring move of
    each clade tried in order of predicted gain, as in :func:`spr_pass`: a
    move is kept only if the exact re-diagnosed tree cost drops."""
    t0 = time.perf_counter()
    st = PassStats()
    diag = downpass(t, be) if diag is None else diag
    st.cost_before = diag.total
    t1 = time.perf_counter()
    S, U, E, score, dclade = tbr_candidates(t, be, diag)
    st.candidates = len(S)
    subs = distinct_nodes(S, len(t.parent))
    cur = np.zeros(len(t.parent), np.int64)
    if len(subs):
        p = t.parent[subs]
        sib = np.where(t.kids[p, 0] == subs, t.kids[p, 1], t.kids[p, 0])
        cur[subs] = be.distances(subs, sib)
    st.seconds_scoring = time.perf_counter() - t1
    if log is not None:
        log.append((t.copy(), S, U, E, score))
    gain = cur[S] - score - dclade
    # largest predicted gain first, ties by ids; only improving candidates
    pos = np.nonzero(gain > 0)[0]
    order = pos[np.lexsort((U[pos], E[pos], S[pos], -gain[pos]))]
    moves, seen = [], set()
    for i in order:
        if len(moves) >= max_moves:
            break
        s, e, u = int(S[i]), int(E[i]), int(U[i])
        if s not in seen:
            seen.add(s)
            moves.append((s, e) if u < 0 else (s, e, u))
    best = diag.total
    while moves:
        st.moves_tried += len(moves)
        detail = {}
        totals = evaluate_moves(t, be, diag, moves, detail)
        k = int(np.argmin(totals))
        if totals[k] >= best:
            be.release_nodes(2 * t.n)
            break
        mv = moves.pop(k)
        if len(mv) > 2:
            t.reroot(mv[0], mv[2])
        w = t.prune(mv[0])
        t.insert(mv[0], mv[1], w)
        commit_move(be, diag, detail[k], totals[k])
        be.release_nodes(2 * t.n)
        best = int(totals[k])
        st.moves_accepted += 1
        moves = [m for m in moves if _valid_tbr_move(t, *m)]
    if st.moves_accepted:
        check = downpass(t, be)
        assert check.total == best, (check.total, best)
        diag = check
    st.cost_after = best
    st.diag = diag
    st.seconds_total = time.perf_counter() - t0
    return st


def _valid_tbr_move(t: Tree, s: int, e: int, u: int = -1) -> bool:
    if u < 0:
        return _valid_move(t, s, e)
    p = t.parent[s]
    if p < 0 or t.parent[p] < 0 or not t.in_tree[e]:
        return False
    inside = set(t.subtree(s))
    return e != p and e not in inside and u in inside and u != s and t.parent[u] != s


def _valid_move(t: Tree, s: int, e: int) -> bool:
    p = t.parent[s]
    if p < 0 or t.parent[p] < 0 or not t.in_tree[e]:
        return False
    sib = t.kids[p][0] if t.kids[p][1] == s else t.kids[p][1]
    return e != p and e != sib and e not in set(t.subtree(s))


def _heights(t: Tree) -> dict:
    """Height of every node of the tree (leaves 0); shared, do not modify."""
    def compute():
        kids, n = t.kids.tolist(), t.n
        h = {}
        for v in t.nodes()[::-1]:
            if v < n:
                h[v] = 0
            else:
                a, b = kids[v]
                h[v] = 1 + max(h[a], h[b])
        return h
    return t._memo("heights", compute)


def evaluate_moves(t: Tree, be, diag: Diagnosis, moves, detail=None) -> np.ndarray:
    """Exact total cost of the tree after each move, computed together.  A
    move (s, e) is SPR: s onto the edge above e; (s, e, u) is TBR: the
    subtree under s re-rooted on the edge above u first.  A move changes
    only the nodes whose children change (in a re-rooted subtree, the path
    from u's parent up to s) and the ancestors of the prune point and of
    the regraft point, so each trial recomputes just those nodes (into
    scratch node slots), and the dirty nodes of every trial at one height
    form one batch of medians.

    With `detail` (a dict), the scratch slots are kept and detail[m] lists
    (node, scratch slot, DO cost, Fitch cost) of trial m's recomputed nodes,
    for commit_move; the caller then releases the slots."""
    return evaluate_trials(t, be, diag, [[mv] for mv in moves], detail)


def _spr_overlay(par, kids, root, trial):
    """The parents and children a trial of SPR moves (s, e) changes, applied
    in order over the base tree's lists exactly as ``Tree.prune`` and
    ``Tree.insert`` would (the pruned parent node is the inserted one);
    returns (parent changes, children changes, root, prune and regraft
    points)."""
    P, K = {}, {}
    gp = lambda v: P[v] if v in P else par[v]
    gk = lambda v: K[v] if v in K else kids[v]
    starts = []
    for mv in trial:
        s, e = int(mv[0]), int(mv[1])
        p = gp(s)
        kp = gk(p)
        o = kp[0] if kp[1] == s else kp[1]
        g = gp(p)
        P[o] = g
        if g < 0:
            root = o
        else:
            kg = list(gk(g))
            kg[0 if kg[0] == p else 1] = o
            K[g] = kg
        P[p] = P[s] = -1
        K[p] = [-1, -1]
        q = gp(e)
        K[p] = [e, s]
        P[p], P[e], P[s] = q, p, p
        if q < 0:
            root = p
        else:
            kq = list(gk(q))
            kq[0 if kq[0] == e else 1] = p
            K[q] = kq
        starts += [g, p]
    return P, K, root, starts


def evaluate_trials(t: Tree, be, diag: Diagnosis, trials, detail=None) -> np.ndarray:
    """``evaluate_moves`` for trials of several moves applied in order (each
    in the tree the previous ones left): the dirty nodes are the ancestors,
    in the trial's final tree, of every move's prune and regraft points and
    re-rooted path nodes.  Trials of SPR moves only are applied as overlays
    of the changed parents and children over the base tree; TBR moves on a
    copy of the tree."""
    h_base = _heights(t)
    mcb = t.min_codes().tolist()
    base_sank = be.sank_cost(t.root)
    tid_next = 2 * t.n
    recs = {}      # level -> list of (trial, a_ref, b_ref, out_tid)
    old = np.zeros(len(trials), np.int64)
    roots = []
    spr_only = all(len(mv) == 2 for trial in trials for mv in trial)
    if spr_only:
        par_l = t._memo("parent_list", lambda: t.parent.tolist())
        kids_l = t._memo("kids_list", lambda: t.kids.tolist())
    for m, trial in enumerate(trials):
        if spr_only:
            P, K, root_m, starts = _spr_overlay(par_l, kids_l, int(t.root), trial)
            gp = lambda v, P=P: P[v] if v in P else par_l[v]
            gk = lambda v, K=K: K[v] if v in K else kids_l[v]
        else:
            T = t.copy()
            starts = []
            for mv in trial:
                s, e = int(mv[0]), int(mv[1])
                u = int(mv[2]) if len(mv) > 2 else -1
                if u >= 0:
                    T.reroot(s, u)
                    starts += [v for v in T.subtree(s)
                               if v >= T.n and set(T.kids[v].tolist()) != set(t.kids[v].tolist())]
                p = T.parent[s]
                starts.append(int(T.parent[p]))
                w = T.prune(s)
                T.insert(s, e, w)
                starts.append(int(w))
            gp = lambda v, T=T: int(T.parent[v])
            gk = lambda v, T=T: T.kids[v].tolist()
            root_m = int(T.root)
        # the dirty nodes with their depths in the trial tree: each walk up
        # from a start ends at the root or at a node already seen, whose
        # depth fixes the depths along the walk
        depth = {}
        for v in starts:
            chain = []
            while v >= 0 and v not in depth:
                chain.append(v)
                v = gp(v)
            d = depth[v] if v >= 0 else -1
            for x in reversed(chain):
                d += 1
                depth[x] = d
        h, tid, mc = {}, {}, {}   # heights, scratch ids, min codes of dirty nodes
        for v in sorted(depth, key=depth.__getitem__, reverse=True):  # children first
            a, b = gk(v)
            ha = h[a] if a in depth else h_base[a]
            hb = h[b] if b in depth else h_base[b]
            h[v] = 1 + (ha if ha > hb else hb)
        for v in sorted(depth, key=h.__getitem__):
            tid[v] = tid_next
            tid_next += 1
            a, b = gk(v)
            ca = mc[a] if a in depth else mcb[a]
            cb = mc[b] if b in depth else mcb[b]
            if ca > cb:
                a, b, ca = b, a, cb
            mc[v] = ca
            recs.setdefault(h[v], []).append((m, tid[a] if a in depth else a,
                                              tid[b] if b in depth else b, tid[v], v))
            old[m] += diag.do_cost[v] + diag.fitch_cost[v]
        roots.append(tid[root_m])
    be.ensure_nodes(tid_next)
    new = np.zeros(len(trials), np.int64)
    rs = [np.array(recs[lvl], np.int64) for lvl in sorted(recs)]
    for r, (do, fi) in zip(rs, be.median_levels([(r[:, 1], r[:, 2], r[:, 3]) for r in rs])):
        np.add.at(new, r[:, 0], do + fi)
        if detail is not None:
            for i in range(len(r)):
                detail.setdefault(int(r[i, 0]), []).append(
                    (int(r[i, 4]), int(r[i, 3]), int(do[i]), int(fi[i])))
    totals = diag.total - old + new - base_sank + be.sank_costs(roots)
    if detail is None:
        be.release_nodes(2 * t.n)
    return totals


def commit_move(be, diag: Diagnosis, rows, total: int):
    """Makes an evaluated move's recomputed medians the tree's own (the move
    must already be applied to the tree): each recomputed node takes over
    its scratch slot's medians and costs."""
    be.rebind_nodes([v for v, _, _, _ in rows], [tid for _, tid, _, _ in rows])
    for v, _, do, fi in rows:
        diag.do_cost[v] = do
        diag.fitch_cost[v] = fi
    diag.total = int(total)



# ---------------------------------------------------------------------------
# All-rootings diagnosis
# ---------------------------------------------------------------------------
@dataclass
class RootCosts:
    edges: np.ndarray   # [m, 2] undirected edges (u < v) of the unrooted tree
    costs: np.ndarray   # [m] tree cost when rooted on each edge

    def best(self):
        """(cost, edge) of the cheapest rooting (first edge on ties)."""
        k = int(np.argmin(self.costs))
        return int(self.costs[k]), (int(self.edges[k, 0]), int(self.edges[k, 1]))


def unrooted_adjacency(tree: Tree) -> dict:
    """Neighbours of every node of `tree` taken as unrooted: the root's
    two children are joined by one edge and the root itself dropped."""
    n = tree.n
    nodes = tree.nodes()
    adj = {v: [] for v in nodes}
    for v in nodes:
        if v >= n:
            for c in tree.kids[v]:
                adj[v].append(int(c))
                adj[int(c)].append(v)
    r = tree.root
    if r >= n:
        a, b = (int(x) for x in tree.kids[r])
        adj[a].remove(r)
        adj[b].remove(r)
        adj[a].append(b)
        adj[b].append(a)
        del adj[r]
    return adj


@dataclass
class _AllDir:
    adj: dict
    info: dict          # directed subtree (u seen from v) -> (height, min code, node id, children)
    edges: list         # undirected edges (u < v)
    root_ids: np.ndarray  # node id of each edge's root median
    do_cost: np.ndarray   # DO part of each rooting's cost
    other: np.ndarray     # Fitch + Sankoff part
    next_id: int          # first node id past the medians


def _all_directions(tree: Tree, be) -> _AllDir | None:
    n = tree.n
    adj = unrooted_adjacency(tree)
    if len(adj) < 2:
        return None
    info = {}
    nxt = 2 * n
    for u0 in adj:
        for v0 in adj[u0]:
            stack = [(u0, v0)]
            while stack:
                u, v = stack[-1]
                if (u, v) in info:
                    stack.pop()
                    continue
                if u < n:
                    info[(u, v)] = (0, u, u, None)
                    stack.pop()
                    continue
                kids = [(c, u) for c in adj[u] if c != v]
                todo = [k for k in kids if k not in info]
                if todo:
                    stack.extend(todo)
                    continue
                k1, k2 = kids
                if info[k1][1] > info[k2][1]:
                    k1, k2 = k2, k1
                info[(u, v)] = (1 + max(info[k1][0], info[k2][0]), info[k1][1], nxt, (k1, k2))
                nxt += 1
                stack.pop()
    edges = sorted({(min(u, v), max(u, v)) for u in adj for v in adj[u]})
    be.ensure_nodes(nxt + len(edges))
    cdo = {e: 0 for e, x in info.items() if x[3] is None}
    cfi = dict(cdo)
    levels = {}
    for e, x in info.items():
        if x[3] is not None:
            levels.setdefault(x[0], []).append(e)
    # every directed median, height by height, then the root median of
    # every edge: one call of dependent levels
    hs = sorted(levels)
    jobs = []
    for h in hs:
        es = levels[h]
        jobs.append((np.array([info[info[e][3][0]][2] for e in es], np.int64),
                     np.array([info[info[e][3][1]][2] for e in es], np.int64),
                     np.array([info[e][2] for e in es], np.int64)))
    ends = []
    for u, v in edges:
        d1, d2 = (u, v), (v, u)
        if info[d1][1] > info[d2][1]:
            d1, d2 = d2, d1
        ends.append((d1, d2))
    out = np.arange(nxt, nxt + len(edges), dtype=np.int64)
    jobs.append((np.array([info[d1][2] for d1, _ in ends], np.int64),
                 np.array([info[d2][2] for _, d2 in ends], np.int64), out))
    res = be.median_levels(jobs)
    for h, (do, fi) in zip(hs, res):
        for i, e in enumerate(levels[h]):
            k1, k2 = info[e][3]
            cdo[e] = cdo[k1] + cdo[k2] + int(do[i])
            cfi[e] = cfi[k1] + cfi[k2] + int(fi[i])
    bdo = [cdo[d1] + cdo[d2] for d1, d2 in ends]
    bfi = [cfi[d1] + cfi[d2] for d1, d2 in ends]
    do, fi = res[-1]
    other = np.array(bfi, np.int64) + fi
    if getattr(be, "ns", 0):
        other = other + be.sank_costs(out)
    return _AllDir(adj, info, edges, out, np.array(bdo, np.int64) + do, other,
                   nxt + len(edges))


def root_costs(tree: Tree, be) -> RootCosts:
    """The reference's tree diagnosis in its default cost mode: the median
    of every directed subtree -- both directions of every edge, children
    before parents, one batch per subtree height (``internal_downpass``,
    allDirChar.ml:722-786) -- then the root median on every edge, one
    batch (``refresh_all_edges``).  The reference roots the tree on the
    edge of lowest root cost (``pick_best_root`` with
    ``blindly_trust_downpass``, allDirChar.ml:791-869); ``RootCosts.best()``
    gives it.  Medians take their arguments in ``min_child_code`` order
    (node.ml:344-349).

    `be` may be a list of backends, one per character set (e.g. one per
    '#' fragment): their costs add up per rooting.  Scratch node ids from
    2 * tree.n hold the directed medians; they are released on return."""
    bes = list(be) if isinstance(be, (list, tuple)) else [be]
    tot = None
    for b in bes:
        D = _all_directions(tree, b)
        if D is None:
            return RootCosts(np.zeros((0, 2), np.int64), np.zeros(0, np.int64))
        b.release_nodes(2 * tree.n)
        tot = D.do_cost + D.other if tot is None else tot + D.do_cost + D.other
    return RootCosts(np.array(D.edges, np.int64).reshape(-1, 2), tot)


@dataclass
class FinalCost:
    cost: int           # the tree cost the reference reports
    root_edge: tuple    # (a, b): a on the handle's side
    root_cost: int      # the best rooting's downpass cost (pick_best_root)
    # with states=True: per backend, {vertex: (Fitch final row, Sankoff
    # final e rows, Sankoff best-state bits)} of the non-DO characters
    finals: list = field(default_factory=list)


def final_cost(tree: Tree, be, weight: int = 1, states: bool = False) -> FinalCost:
    """The tree cost the reference reports after a diagnosis
    (``Ptree.get_cost `Adjusted``, poy_test.ml:43): ``pick_best_root``
    (see :func:`root_costs`), then ``assign_single``
    (allDirChar.ml:288-404) and ``check_cost`` (allDirChar.ml:185-212).

    assign_single gives every node a single sequence from the root
    outwards: the root's is ``closest(root median, a's subtree median)``
    for the root edge (a, b), a on the handle's side; every node's is
    ``closest(parent's single, its subtree median seen from the parent)``
    (``DOS.to_single``, seqCS.ml:730-745), one batch per distance from the
    root.  check_cost sums ``DOS.distance`` between the single sequences
    of every edge and adds the rooting's non-DO (Fitch, Sankoff) cost.
    On the reference's test trees this equals the best rooting's cost for
    linear matrices and differs (by up to a few percent, either way) for
    affine ones.

    The tree's own root plays the handle: an edge is oriented from the
    parent, the root's two children from the first.  Among rootings of
    equal cost the first edge in (u, v) order is taken.

    `weight` is the characters' weight factor (``transform
    (weightfactor:w)``; node costs are ``weight * cost``, node.ml:350-357).
    The root is chosen by absolute cost (allDirChar.ml:794), so the
    rooting and the single sequences do not depend on it and it scales
    every cost.

    With `states`, the non-DO characters' final states are assigned too
    (``assign_final_states``, allDirChar.ml:1377-1428) and returned in
    ``FinalCost.finals``; they do not change the cost."""
    bes = list(be) if isinstance(be, (list, tuple)) else [be]
    Ds = [_all_directions(tree, b) for b in bes]
    if Ds[0] is None:
        return FinalCost(0, (), 0)
    tot = sum(D.do_cost + D.other for D in Ds)
    k = int(np.argmin(tot))
    D = Ds[0]
    u, v = D.edges[k]
    if tree.parent[v] == u:
        a, b = u, v
    elif tree.parent[u] == v:
        a, b = v, u
    else:
        a, b = (int(x) for x in tree.kids[tree.root])
    cost = 0
    finals = []
    for B, D in zip(bes, Ds):
        cost += _assign_single_cost(B, D, k, a, b)
        if states:
            finals.append(_assign_final_states(B, D, k, a, b, tree.n))
        B.release_nodes(2 * tree.n)
    return FinalCost(weight * cost, (int(a), int(b)), weight * int(tot[k]), finals)


def _assign_final_states(be, D: _AllDir, k: int, a: int, b: int, n: int) -> dict:
    """assign_final_states (allDirChar.ml:1377-1428) for the non-DO
    characters, from root edge k = (a, b): the root median's final is its
    preliminary; a and b, then every vertex away from them, take
    median_3(parent's final, own preliminary state seen from the parent,
    the two children's preliminary states seen from it) -- a leaf passes
    itself as both children -- one batch per distance from the root.
    Returns {vertex: (Fitch row, Sankoff e rows, Sankoff best bits)}."""
    if not (getattr(be, "nf", 0) or getattr(be, "ns", 0)):
        return {}
    root_slot = 2 * n - 1               # vertex ids stop at 2n - 2
    be.final_slots(2 * n, D.next_id + 2 + 2 * n)
    be.final_root(int(D.root_ids[k]), root_slot)
    front = [(a, b, root_slot), (b, a, root_slot)]
    done = []
    while front:
        anc = np.array([f[2] for f in front], np.int64)
        node, left, right = [], [], []
        for c, p, _ in front:
            x = D.info[(c, p)]
            node.append(x[2])
            if x[3] is None:  # a leaf: median_3 par cur cur cur
                left.append(x[2])
                right.append(x[2])
            else:
                left.append(D.info[x[3][0]][2])
                right.append(D.info[x[3][1]][2])
        out = np.array([c for c, _, _ in front], np.int64)
        be.final_states(anc, np.array(node), np.array(left), np.array(right), out)
        done.extend(out.tolist())
        front = [(x, c, c) for c, p, _ in front for x in D.adj[c] if x != p]
    return {int(v): be.node_final(int(v)) for v in done}


def _assign_single_cost(be, D: _AllDir, k: int, a: int, b: int) -> int:
    """assign_single from root edge k = (a, b) and check_cost, one
    backend's characters."""
    single, _ = _assign_singles(be, D, k, a, b)
    ea = np.array([single[x] for x, _ in D.edges], np.int64)
    eb = np.array([single[y] for _, y in D.edges], np.int64)
    return int(be.do_distances(ea, eb).sum()) + int(D.other[k])


def _assign_singles(be, D: _AllDir, k: int, a: int, b: int):
    """assign_single (allDirChar.ml:288-404) from root edge k = (a, b):
    {vertex: node id of its single sequence} and the next free node id."""
    nxt = D.next_id
    be.ensure_nodes(nxt + 1 + len(D.adj))
    root = nxt
    nxt += 1
    be.singles(np.array([D.root_ids[k]]), np.array([D.info[(a, b)][2]]), np.array([root]))
    single = {}
    front = [(a, b, root), (b, a, root)]
    while front:
        par = np.array([f[2] for f in front], np.int64)
        mine = np.array([D.info[(c, p)][2] for c, p, _ in front], np.int64)
        out = np.arange(nxt, nxt + len(front), dtype=np.int64)
        nxt += len(front)
        be.singles(par, mine, out)
        nf = []
        for (c, p, _), o in zip(front, out):
            single[c] = int(o)
            nf.extend((x, c, int(o)) for x in D.adj[c] if x != p)
        front = nf
    return single, nxt


@dataclass
class AdjustResult:
    cost: int           # check_cost of the accepted tree (DO edge distances + non-DO root cost)
    initial_cost: int   # the same before adjusting (final_cost's)
    passes: int         # accepted passes
    changes: int        # vertex readjustments that changed a sequence, accepted passes
    calls: int          # batched readjust calls (one per level and pass)
    seqs: dict = field(default_factory=dict)   # vertex -> adjusted DO sequence


def adjust_order(tree: Tree, adj: dict):
    """The interior vertices of the unrooted tree in post-order (children
    before parents) with their neighbours (ch1, ch2, parent) in the
    reference's positional order (``Tree.Interior (_, a, b, c)`` ->
    ``adjust_node a b c``, allDirChar.ml:532-545): the neighbour towards
    the handle first, then the two others.  The tree's root is dropped and
    its first child plays the handle, with the root's second child as the
    neighbour in front of it (visited as its last child)."""
    n = tree.n
    r = int(tree.root)
    top, other = (int(x) for x in tree.kids[r])
    up = {}
    for v in adj:
        if v == top:
            up[v] = other
        elif int(tree.parent[v]) == r:
            up[v] = top
        else:
            up[v] = int(tree.parent[v])
    # post-order from the handle: its own children, then the other side of
    # the root edge, then the handle
    order = []
    stack = [(top, False)]
    while stack:
        v, done = stack.pop()
        if done:
            if v >= n:
                order.append(v)
            continue
        stack.append((v, True))
        kids = [x for x in adj[v] if x != up[v]] + ([other] if v == top else [])
        for x in reversed(kids):
            stack.append((x, False))
    nbrs = {v: (up[v],) + tuple(x for x in adj[v] if x != up[v]) for v in order}
    return order, nbrs


def adjust_levels(order, adj):
    """Batches of the sequential order that keep its results: a vertex
    reads its neighbours' sequences, so of two adjacent vertices the one
    earlier in the order must run first (it reads the later one's old
    sequence, the later one reads its new one).  Level = 1 + the highest
    level of an earlier adjacent vertex; vertices of a level are pairwise
    non-adjacent."""
    pos = {v: i for i, v in enumerate(order)}
    lvl = {}
    for v in order:
        lvl[v] = 1 + max([lvl[u] for u in adj[v] if u in pos and pos[u] < pos[v]], default=-1)
    out = [[] for _ in range(1 + max(lvl.values(), default=-1))]
    for v in order:
        out[lvl[v]].append(v)
    return out


def adjust_tree(tree: Tree, be, mode: str = "three", max_count: int | None = None,
                batched: bool = True) -> AdjustResult:
    """``AllDirChar.adjust_tree`` (allDirChar.ml:488-668) of the Iterative
    cost modes for the DO characters of one backend, after the default
    diagnosis (``pick_best_root`` and ``assign_single``, see
    :func:`final_cost`): passes over the interior vertices in post-order,
    each vertex's sequence re-estimated from its three neighbours' current
    ones by ``DOS.readjust`` (mode "three": ``readjust_3d``; "approx":
    ``Sequence.readjust``).  A pass visits the vertices marked by the
    previous one (the first visits all); a changed vertex marks its three
    neighbours.  A pass is kept while something changed and the tree cost
    (``check_cost``: ``DOS.distance`` over every edge plus the rooting's
    non-DO cost) went down, at most `max_count` passes; otherwise the tree
    before it is returned.  The root recomputation of ``adjust_handle``
    leaves this cost unchanged for the DO part and is not done.

    With `batched`, the vertices of a pass run in the batches of
    :func:`adjust_levels` (the same results as one at a time)."""
    D = _all_directions(tree, be)
    if D is None:
        return AdjustResult(0, 0, 0, 0, 0)
    tot = D.do_cost + D.other
    k = int(np.argmin(tot))
    u, v = D.edges[k]
    if tree.parent[v] == u:
        a, b = u, v
    elif tree.parent[u] == v:
        a, b = v, u
    else:
        a, b = (int(x) for x in tree.kids[tree.root])
    single, nxt = _assign_singles(be, D, k, a, b)
    ea = np.array([x for x, _ in D.edges], np.int64)
    eb = np.array([y for _, y in D.edges], np.int64)
    other = int(D.other[k])

    def cost_of(cur):
        return int(be.do_distances(np.array([cur[x] for x in ea]),
                                   np.array([cur[y] for y in eb])).sum()) + other

    order, nbrs = adjust_order(tree, D.adj)
    groups = adjust_levels(order, D.adj) if batched else [[x] for x in order]
    cur = dict(single)
    prev = cost_of(cur)
    initial = prev
    affected = set(cur)
    count = max_count if max_count is not None else 1 << 30
    passes = changes = calls = 0
    while count > 0:
        new = dict(cur)
        marked, n_changed = set(), 0
        for g in groups:
            g = [x for x in g if x in affected]
            if not g:
                continue
            be.ensure_nodes(nxt + len(g))
            out = np.arange(nxt, nxt + len(g), dtype=np.int64)
            nxt += len(g)
            ch, _ = be.readjust([new[nbrs[x][0]] for x in g], [new[nbrs[x][1]] for x in g],
                                [new[nbrs[x][2]] for x in g], [new[x] for x in g], out, mode)
            calls += 1
            for x, o, c in zip(g, out, ch):
                if c:
                    new[x] = int(o)
                    marked.update(nbrs[x])
                    n_changed += 1
        if not n_changed:
            break
        c = cost_of(new)
        if c >= prev:
            break
        cur, prev, affected = new, c, marked
        passes += 1
        changes += n_changed
        count -= 1
    seqs = {x: np.asarray(be.node_seq(cur[x]), np.uint8).copy() for x in order}
    be.release_nodes(2 * tree.n)
    return AdjustResult(prev, initial, passes, changes, calls, seqs)
