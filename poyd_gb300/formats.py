"""Reading POY inputs: unaligned DNA FASTA files, Hennig86 matrices of
static characters and parenthetical trees.

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

Hennig86 (xread): the static characters' state sets per taxon, their
additive / non-additive, active and weight flags from ccode commands, and
the tread trees (:func:`read_hennig`).  The non-additive characters give
the 8-, 16- and 32-bit Fitch lanes of the GPU path
(:meth:`HennigMatrix.fitch_groups`).
"""
from __future__ import annotations

import re
from dataclasses import dataclass

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


# --------------------------------------------------------------------------
# Hennig86 / TNT files (xread, ccode, tread)
# --------------------------------------------------------------------------

# state symbols in order (hennig_upto, parser.ml:3813-3833)
HENNIG_STATES = "0123456789ABCDEFGHIJKLMNOPQRSTUV"


@dataclass
class HennigMatrix:
    """A Hennig86 file as POY reads it (Parser.Hennig.of_channel,
    parser.ml:3895-3990).

    ``cells[t][c]`` is the set of raw states of taxon t at character c as a
    bitmask over HENNIG_STATES (bit s = state s); 0 means missing ('?' or
    '-').  Every character starts additive, active and of weight 1
    (default_hennig, parser.ml:3790-3811) until a ccode command changes it
    (parser.ml:3929-3951)."""
    names: list
    cells: np.ndarray      # [n_taxa, n_chars] uint32 state masks, 0 = missing
    additive: np.ndarray   # [n_chars] bool
    active: np.ndarray     # [n_chars] bool
    weight: np.ndarray     # [n_chars] int64
    trees: list            # parenthetical tree texts, taxa by name

    def observed(self, c: int) -> list:
        """Raw states of character c seen in some taxon, ascending."""
        m = int(np.bitwise_or.reduce(self.cells[:, c])) if len(self.cells) else 0
        return [s for s in range(32) if m >> s & 1]

    def _fitch_masks(self, cols, dtype) -> np.ndarray:
        # bit i = the i-th observed state; a missing cell holds them all
        out = np.zeros((len(self.names), len(cols)), dtype)
        for j, c in enumerate(cols):
            obs = self.observed(c)
            full = (1 << max(len(obs), 1)) - 1
            for t in range(len(self.names)):
                m = int(self.cells[t, c])
                out[t, j] = full if m == 0 else sum(1 << i for i, s in enumerate(obs) if m >> s & 1)
        return out

    def fitch_matrix(self):
        """The active non-additive characters as 8-bit Fitch state masks:
        (uint8 [n_taxa, k] masks, int64 [k] character indices, int64 [k]
        weights).  As in POY's non-additive encoding, bit i stands for the
        i-th observed state of the character and a missing cell holds every
        observed state.  A character with more than 8 observed states does
        not fit the 8-bit lanes and raises ValueError (see fitch_groups)."""
        cols = [c for c in range(self.cells.shape[1]) if self.active[c] and not self.additive[c]]
        for c in cols:
            if len(self.observed(c)) > 8:
                raise ValueError("character %d has %d states; 8-bit lanes hold 8"
                                 % (c, len(self.observed(c))))
        cols = np.array(cols, np.int64)
        return self._fitch_masks(cols, np.uint8), cols, self.weight[cols]

    def fitch_groups(self) -> dict:
        """The active non-additive characters grouped by lane width the way
        POY groups them by observed states (data.ml:1962-1989): 2-8 states
        in 8-bit lanes, 9-16 in 16-bit, 17-32 in 32-bit; characters of 0 or 1
        observed state never cost anything and are left out.  Returns
        {width: (masks [n_taxa, k] of that width, int64 character indices,
        int64 weights)} for the widths present, for the nonadd8 / nonadd16 /
        nonadd32 batches."""
        groups = {8: [], 16: [], 32: []}
        for c in range(self.cells.shape[1]):
            if not self.active[c] or self.additive[c]:
                continue
            k = len(self.observed(c))
            if k >= 2:
                groups[8 if k <= 8 else 16 if k <= 16 else 32].append(c)
        dt = {8: np.uint8, 16: np.uint16, 32: np.uint32}
        return {w: (self._fitch_masks(cols, dt[w]), np.array(cols, np.int64),
                    self.weight[np.array(cols, np.int64)])
                for w, cols in groups.items() if cols}

    def additive_intervals(self):
        """The active additive characters as [min, max] state intervals:
        (uint8 [n_taxa, k] lows, uint8 [n_taxa, k] highs, int64 [k]
        character indices); a missing cell spans the observed states."""
        cols = [c for c in range(self.cells.shape[1]) if self.active[c] and self.additive[c]]
        lo = np.zeros((len(self.names), len(cols)), np.uint8)
        hi = np.zeros_like(lo)
        for j, c in enumerate(cols):
            obs = self.observed(c) or [0]
            for t in range(len(self.names)):
                m = int(self.cells[t, c])
                st = [s for s in range(32) if m >> s & 1] or obs
                lo[t, j], hi[t, j] = min(st), max(st)
        return lo, hi, np.array(cols, np.int64)


def _hennig_cell(tok: str) -> int:
    if tok in ("?", "-"):
        return 0
    m = 0
    for ch in tok.strip("[]"):
        if ch in " .":
            continue
        s = HENNIG_STATES.find(ch.upper())
        if s < 0:
            raise ValueError("illegal Hennig state %r" % ch)
        m |= 1 << s
    return m


def _hennig_ccode(body: str, flags, n_chars: int) -> None:
    """One ccode command: verbs '+' additive, '-' non-additive, '[' active,
    ']' inactive, '/w' weight w (default 1), '*' reset, each applying to the
    character ranges after it ('a.b'; a missing bound is 0 or the last
    character) (process_ccode, parser.ml:1209-1260)."""
    additive, active, weight = flags
    verbs = {}
    for tok in re.findall(r"/\s*\d*|[-+\[\]*]|\d*\.\d*|\d+", body):
        if tok[0] == "/":
            verbs["w"] = int(tok[1:].strip() or 1)
        elif tok == "+":
            verbs["add"] = True
        elif tok == "-":
            verbs["add"] = False
        elif tok == "[":
            verbs["act"] = True
        elif tok == "]":
            verbs["act"] = False
        elif tok == "*":
            verbs = {}
        else:
            a, dot, b = tok.partition(".")
            lo = int(a) if a else 0
            hi = (int(b) if b else n_chars - 1) if dot else lo
            for c in range(lo, min(hi, n_chars - 1) + 1):
                if "add" in verbs:
                    additive[c] = verbs["add"]
                if "act" in verbs:
                    active[c] = verbs["act"]
                if "w" in verbs:
                    weight[c] = verbs["w"]


def read_hennig(path: str) -> HennigMatrix:
    """Reads the xread matrix, ccode ('cc') commands and tread trees of a
    Hennig86 file; other commands (cn, proc, ...) are skipped.  In the
    matrix, spaces and '.' between cells are ignored and '[...]' is a
    polymorphic cell (read_data_xread, parser.ml:1365-1400).  Numeric taxon
    references in trees become taxon names (parser.ml:3952-3966)."""
    text = re.sub(r"'[^']*'", " ", open(path).read())  # titles and comments
    names, rows, trees = [], [], []
    flags = None
    n_chars = 0
    for m in re.finditer(r"[^;]*;", text, re.S):
        cmd = m.group(0)[:-1]
        cmd = re.sub(r"^[\s#$]+", "", cmd)
        word = re.match(r"[A-Za-z]*", cmd).group(0).lower()
        body = cmd[len(word):]
        if word == "xread":
            # the two counts come first
            head = re.match(r"\s*(\d+)\s+(\d+)", body)
            if not head:
                raise ValueError("xread without character and taxon counts")
            n_chars, n_taxa = int(head.group(1)), int(head.group(2))
            rest = body[head.end():]
            words = re.findall(r"\[[^\]]*\]|[^\s\[]+", rest)
            i = 0
            while i < len(words) and len(names) < n_taxa:
                names.append(words[i])
                i += 1
                cells = []
                while len(cells) < n_chars:
                    if i >= len(words):
                        raise ValueError("taxon %r has fewer than %d cells" % (names[-1], n_chars))
                    w = words[i]
                    i += 1
                    if w.startswith("["):
                        cells.append(_hennig_cell(w))
                    else:
                        cells.extend(_hennig_cell(ch) for ch in w if ch != ".")
                if len(cells) != n_chars:
                    raise ValueError("taxon %r has %d cells, not %d" % (names[-1], len(cells), n_chars))
                rows.append(cells)
            if len(names) != n_taxa:
                raise ValueError("xread names %d taxa, not %d" % (len(names), n_taxa))
            flags = (np.ones(n_chars, bool), np.ones(n_chars, bool), np.ones(n_chars, np.int64))
        elif word in ("cc", "ccode") and flags is not None:
            _hennig_ccode(body, flags, n_chars)
        elif word == "tread":
            for tree in body.split("*"):
                if tree.strip():
                    trees.append(re.sub(r"(?<![\w.])(\d+)(?![\w.])",
                                        lambda d: names[int(d.group(1))]
                                        if int(d.group(1)) < len(names) else d.group(1), tree))
    if flags is None:
        raise ValueError("no xread matrix in %s" % path)
    additive, active, weight = flags
    return HennigMatrix(names=names, cells=np.array(rows, np.uint32).reshape(len(names), n_chars),
                        additive=additive, active=active, weight=weight, trees=trees)
