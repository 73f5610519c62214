"""Seeded simulation of phylogenetic datasets (configs 0, 2, 3 and 4).

A random Yule tree; DNA evolved along it with Jukes-Cantor substitutions
(expected ``sub_per_branch`` substitutions per site per branch) and indels
at ``indel_rate`` per site with geometric lengths (mean 2); non-additive
characters with 2-8 states whose per-character state frequencies are drawn
from Dirichlet(0.5); Sankoff characters with 4 states observed at the
leaves and one random symmetric integer cost matrix (entries 1-5, zero
diagonal).  Every quantity comes from one numpy Generator seeded by the
caller.  Leaves carry POY encodings: DNA bitmasks with the leading gap,
one-bit Fitch state masks, Sankoff cost vectors (0 for the observed state,
infinity otherwise, sankCS.ml:34-67).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import synth

SANK_INF = 1 << 30


@dataclass
class Dataset:
    names: list
    seqs: list                     # uint8 arrays with the leading gap
    fitch: np.ndarray              # [n_taxa, n_fitch] uint8 state masks
    fitch_states: np.ndarray       # [n_fitch] number of states (2..8)
    sank: np.ndarray               # [n_taxa, n_sank, k] int32 leaf cost vectors
    sank_tcm: np.ndarray           # [k, k] int32
    true_parent: np.ndarray = field(default=None)  # generating tree (parent of each node)

    @property
    def n_taxa(self) -> int:
        return len(self.seqs)


def yule_tree(rng: np.random.Generator, n: int) -> np.ndarray:
    """Parent array of a rooted binary Yule tree: every step splits a
    uniformly chosen tip in two.  Leaves are 0..n-1 (labels in random
    order), internal nodes n..2n-2, the root 2n-2 (parent -1)."""
    par = [-1]
    tips = [0]
    while len(tips) < n:
        i = int(rng.integers(len(tips)))
        v = tips[i]
        a, b = len(par), len(par) + 1
        par += [v, v]
        tips[i] = a
        tips.append(b)
    internal = [v for v in range(len(par)) if v not in set(tips)]
    internal.sort(reverse=True)  # children were created after parents
    order = list(rng.permutation(tips))
    remap = {}
    for i, v in enumerate(order):
        remap[v] = i
    # internal nodes: root (0) last
    internal = [v for v in internal if v != 0] + [0]
    for i, v in enumerate(internal):
        remap[v] = n + i
    parent = -np.ones(2 * n - 1, dtype=np.int64)
    for v, p in enumerate(par):
        if p >= 0:
            parent[remap[v]] = remap[p]
    return parent


def _children(parent: np.ndarray):
    ch = [[] for _ in range(len(parent))]
    for v, p in enumerate(parent):
        if p >= 0:
            ch[p].append(v)
    return ch


def simulate(seed: int, n_taxa: int, seq_len: int, n_fitch: int = 0, n_sank: int = 0,
             sub_per_branch: float = 0.05, indel_rate: float = 0.01, k_sank: int = 4) -> Dataset:
    rng = np.random.default_rng(seed)
    parent = yule_tree(rng, n_taxa)
    ch = _children(parent)
    root = len(parent) - 1
    # JC: P(change) per site per branch for expected rate mu is
    # 3/4 (1 - exp(-4 mu / 3)); a changed site draws one of the 3 other bases
    p_change = 0.75 * (1.0 - np.exp(-4.0 * sub_per_branch / 3.0))
    seqs = {root: synth.random_dna(rng, seq_len)}
    fitch_states = rng.integers(2, 9, size=n_fitch)
    probs = [rng.dirichlet(np.full(k, 0.5)) for k in fitch_states]
    stack = [root]
    while stack:
        v = stack.pop()
        for c in ch[v]:
            s = seqs[v].copy()
            m = rng.random(len(s)) < p_change
            if m.any():
                shift = rng.integers(1, 4, size=int(m.sum()))
                idx = np.log2(s[m]).astype(np.int64)
                s[m] = synth.BASES[(idx + shift) % 4]
            s = synth.mutate(rng, s, 0.0, indel_rate)
            seqs[c] = s
            stack.append(c)
    fitch = np.zeros((n_taxa, n_fitch), dtype=np.uint8)
    for j, p in enumerate(probs):
        st = rng.choice(len(p), size=n_taxa, p=p)
        fitch[:, j] = (1 << st).astype(np.uint8)
    tcm = rng.integers(1, 6, size=(k_sank, k_sank))
    tcm = np.triu(tcm, 1)
    tcm = (tcm + tcm.T).astype(np.int32)
    sank = np.full((n_taxa, n_sank, k_sank), SANK_INF, dtype=np.int32)
    obs = rng.integers(0, k_sank, size=(n_taxa, n_sank))
    for t in range(n_taxa):
        sank[t, np.arange(n_sank), obs[t]] = 0
    names = ["t%d" % i for i in range(n_taxa)]
    return Dataset(names=names, seqs=[synth.with_gap(seqs[i]) for i in range(n_taxa)],
                   fitch=fitch, fitch_states=fitch_states, sank=sank, sank_tcm=tcm,
                   true_parent=parent)
