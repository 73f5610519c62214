"""Reading POY inputs: unaligned DNA FASTA files and parenthetical trees.

FASTA: every '#'-separated fragment of a taxon's sequence is its own
dynamic (DO) character (``split_frag``, parser.ml:262); residues are
encoded in POY's DNA bitmask alphabet (A=1, C=2, G=4, T=8, gap=16, IUPAC
codes the unions, alphabet.ml:143-175), gaps are dropped from unaligned
input and the leading gap is prepended (``process_sequence``,
parser.ml:273-287).

Trees: POY's parenthetical format, ``(a ((b c) d))`` with whitespace (or
commas) between siblings and an optional bracketed cost after the tree
(``[865.]``).  Taxon codes follow the order in which the FASTA file names
the taxa; they are the leaf ids of :class:`poyd_gb300.search.Tree`.
"""
from __future__ import annotations

import re

import numpy as np

from .simulate import SANK_INF, Dataset
from .synth import GAP

DNA = {"A": 1, "C": 2, "G": 4, "T": 8, "U": 8, "M": 3, "R": 5, "W": 9, "S": 6,
       "Y": 10, "K": 12, "V": 7, "H": 11, "D": 13, "B": 14, "N": 15, "X": 15, "-": GAP}


def encode_dna(text: str, remove_gaps: bool = True) -> np.ndarray:
    """One fragment as a uint8 sequence with the leading gap."""
    out = [GAP]
    for ch in text.upper():
        if ch.isspace():
            continue
        if ch not in DNA:
            raise ValueError("illegal DNA character %r" % ch)
        v = DNA[ch]
        if v == GAP and remove_gaps:
            continue
        out.append(v)
    return np.array(out, np.uint8)


def read_fasta(path: str):
    """(taxon names in file order, raw sequence text per taxon)."""
    names, seqs, cur = [], [], []
    with open(path) as f:
        for line in f:
            line = line.strip()
            if line.startswith(">"):
                if names:
                    seqs.append("".join(cur))
                names.append(line[1:].strip())
                cur = []
            elif line:
                cur.append(line)
    if names:
        seqs.append("".join(cur))
    return names, seqs


def fasta_fragments(path: str) -> list[Dataset]:
    """One dataset per '#'-separated fragment (every taxon must have the
    same number of fragments); each dataset holds that DO character only."""
    names, seqs = read_fasta(path)
    frags = [s.split("#") for s in seqs]
    k = {len(f) for f in frags}
    if len(k) != 1:
        raise ValueError("taxa differ in their number of '#' fragments")
    n = len(names)
    out = []
    for j in range(k.pop()):
        out.append(Dataset(names=list(names), seqs=[encode_dna(f[j]) for f in frags],
                           fitch=np.zeros((n, 0), np.uint8),
                           fitch_states=np.zeros(0, np.int64),
                           sank=np.full((n, 0, 4), SANK_INF, np.int32),
                           sank_tcm=np.zeros((4, 4), np.int32)))
    return out


def parse_tree(text: str, names):
    """A rooted binary :class:`Tree` from a parenthetical tree over `names`
    (a node with one child is skipped; more than two children is an
    error: POY's trees here are binary).  The tree may leave taxa out:
    they stay outside the tree (a one-taxon component, which adds no
    cost)."""
    from .search import Tree
    code = {nm: i for i, nm in enumerate(names)}
    text = re.sub(r"\[[^\]]*\]", " ", text)
    toks = re.findall(r"\(|\)|[^\s(),;]+", text)
    pos = 0

    def node():
        nonlocal pos
        if toks[pos] == "(":
            pos += 1
            kids = []
            while toks[pos] != ")":
                kids.append(node())
            pos += 1
            if len(kids) == 1:
                return kids[0]
            if len(kids) != 2:
                raise ValueError("tree node with %d children" % len(kids))
            return tuple(kids)
        t = toks[pos]
        pos += 1
        if t not in code:
            raise ValueError("unknown taxon %r" % t)
        return code[t]

    nested = node()
    t = Tree(len(names))
    seen = []

    def build(x):
        if isinstance(x, int):
            seen.append(x)
            return x
        a, b = build(x[0]), build(x[1])
        w = t._new_internal()
        t.kids[w] = (a, b)
        t.parent[a] = t.parent[b] = w
        return w

    r = build(nested)
    if len(set(seen)) != len(seen):
        raise ValueError("tree names a taxon twice")
    t.parent[r] = -1
    t.root = r
    t.in_tree[t.nodes()] = True
    return t
