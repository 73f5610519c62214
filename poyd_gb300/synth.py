"""Seeded synthetic inputs with the shapes of the benchmark workloads.

No public dataset is involved: every input is generated here from a seed.
Sequences use POY's DNA bitmask alphabet (A=1, C=2, G=4, T=8, gap=16;
IUPAC ambiguity codes are unions of these, alphabet.ml:143-175) and start with
the leading gap at position 0, as every POY sequence does.
"""
from __future__ import annotations

import numpy as np

GAP = 16
BASES = np.array([1, 2, 4, 8], dtype=np.uint8)
# non-empty subsets of {A, C, G, T} with more than one member (IUPAC codes)
AMBIG = np.array([v for v in range(1, 16) if bin(v).count("1") > 1], dtype=np.uint8)


def random_dna(rng: np.random.Generator, n: int, ambig_frac: float = 0.0) -> np.ndarray:
    """n residues (without the leading gap)."""
    s = BASES[rng.integers(0, 4, size=n)]
    if ambig_frac > 0 and n > 0:
        mask = rng.random(n) < ambig_frac
        s[mask] = AMBIG[rng.integers(0, len(AMBIG), size=int(mask.sum()))]
    return s


def mutate(rng: np.random.Generator, s: np.ndarray, sub: float, indel: float,
           mean_indel_len: float = 2.0) -> np.ndarray:
    """Jukes-Cantor-style substitutions plus insertions/deletions with
    geometric lengths (residues only, no leading gap)."""
    s = s.copy()
    n = len(s)
    if n and sub > 0:
        m = rng.random(n) < sub
        s[m] = BASES[rng.integers(0, 4, size=int(m.sum()))]
    if indel <= 0 or n == 0:
        return s
    out = []
    i = 0
    p = 1.0 / mean_indel_len
    ev = rng.random(n) < indel
    kind = rng.random(n) < 0.5
    lens = rng.geometric(p, size=n)
    while i < n:
        if ev[i]:
            if kind[i]:  # deletion
                i += int(lens[i])
                continue
            out.append(BASES[rng.integers(0, 4, size=int(lens[i]))])
        out.append(s[i:i + 1])
        i += 1
    return np.concatenate(out) if out else np.zeros(0, np.uint8)


def with_gap(s: np.ndarray) -> np.ndarray:
    return np.concatenate([np.array([GAP], np.uint8), np.asarray(s, np.uint8)])


def pair_batch(seed: int, n_pairs: int, lmin: int = 100, lmax: int = 5000,
               sub=(0.10, 0.30), indel=(0.02, 0.05), ambig: float = 0.05):
    """Independent DNA pairs: L1 ~ U[lmin, lmax]; the partner carries 10-30 %
    substitutions and 2-5 % indels; a fraction of positions in both become
    random IUPAC ambiguity masks.  Returns two lists of uint8 arrays with the
    leading gap."""
    rng = np.random.default_rng(seed)
    A, B = [], []
    for _ in range(n_pairs):
        n = int(rng.integers(lmin, lmax + 1))
        a = random_dna(rng, n)
        b = mutate(rng, a, float(rng.uniform(*sub)), float(rng.uniform(*indel)))
        if ambig > 0:
            for s in (a, b):
                m = rng.random(len(s)) < ambig
                s[m] = AMBIG[rng.integers(0, len(AMBIG), size=int(m.sum()))]
        A.append(with_gap(a))
        B.append(with_gap(b))
    return A, B


def _mutate_many(rng, base, pid, sub_rate, indel_rate, mean_len=2.0):
    """Vectorised mutate over a concatenation of sequences (pid = owner of
    each position): substitutions, then insertions before / deletions of
    geometric runs starting at event positions."""
    n = len(base)
    s = base.copy()
    m = rng.random(n) < sub_rate[pid]
    s[m] = BASES[rng.integers(0, 4, size=int(m.sum()))]
    ev = rng.random(n) < indel_rate[pid]
    is_del = ev & (rng.random(n) < 0.5)
    is_ins = ev & ~is_del
    ln = rng.geometric(1.0 / mean_len, size=n).astype(np.int64)
    # deletions: cover [i, i + len) but never past the owner's last position
    cover = np.zeros(n + 1, np.int64)
    di = np.nonzero(is_del)[0]
    ends = np.minimum(di + ln[di], n)
    # clip at the pair boundary
    last_of_pid = np.zeros(pid.max() + 2, np.int64)
    np.maximum.at(last_of_pid, pid, np.arange(n))
    ends = np.minimum(ends, last_of_pid[pid[di]] + 1)
    np.add.at(cover, di, 1)
    np.add.at(cover, ends, -1)
    keep = np.cumsum(cover[:-1]) == 0
    ins_len = np.where(is_ins, ln, 0)
    cnt = ins_len + keep
    src = np.repeat(np.arange(n), cnt)
    start = np.cumsum(cnt) - cnt
    rank = np.arange(len(src)) - start[src]
    out = np.where(rank < ins_len[src], BASES[rng.integers(0, 4, size=len(src))], s[src])
    return out.astype(np.uint8), pid[src]


def pair_batch_fast(seed: int, n_pairs: int, lmin: int = 100, lmax: int = 5000,
                    sub=(0.10, 0.30), indel=(0.02, 0.05), ambig: float = 0.05,
                    chunk: int = 4096):
    """Same distribution as :func:`pair_batch`, vectorised over chunks of
    pairs.  Returns the packed host form (seq, a_off, a_len, b_off, b_len) of
    align.PairBatch with a_i, b_i adjacent in seq."""
    rng = np.random.default_rng(seed)
    seqs, a_len, b_len = [], [], []
    for c0 in range(0, n_pairs, chunk):
        k = min(chunk, n_pairs - c0)
        L = rng.integers(lmin, lmax + 1, size=k)
        pid = np.repeat(np.arange(k), L)
        base = BASES[rng.integers(0, 4, size=len(pid))]
        srate = rng.uniform(*sub, size=k)
        irate = rng.uniform(*indel, size=k)
        part, ppid = _mutate_many(rng, base, pid, srate, irate)
        for arr in (base, part):
            m = rng.random(len(arr)) < ambig
            arr[m] = AMBIG[rng.integers(0, len(AMBIG), size=int(m.sum()))]
        lb = np.bincount(ppid, minlength=k)
        # interleave [gap, a_i, gap, b_i]
        la1, lb1 = L + 1, lb + 1
        tot = int(la1.sum() + lb1.sum())
        buf = np.empty(tot, np.uint8)
        sizes = np.empty(2 * k, np.int64)
        sizes[0::2], sizes[1::2] = la1, lb1
        starts = np.cumsum(sizes) - sizes
        buf[starts] = GAP
        a_pos = np.repeat(starts[0::2] + 1 - np.concatenate([[0], np.cumsum(L)[:-1]]), L) + \
            np.arange(len(base))
        buf[a_pos] = base
        b_pos = np.repeat(starts[1::2] + 1 - np.concatenate([[0], np.cumsum(lb)[:-1]]), lb) + \
            np.arange(len(part))
        buf[b_pos] = part
        seqs.append(buf)
        a_len.append(la1)
        b_len.append(lb1)
    seq = np.concatenate(seqs + [np.zeros(64, np.uint8)])
    a_len = np.concatenate(a_len).astype(np.int32)
    b_len = np.concatenate(b_len).astype(np.int32)
    sizes = np.empty(2 * n_pairs, np.int64)
    sizes[0::2], sizes[1::2] = a_len, b_len
    starts = np.cumsum(sizes) - sizes
    return [seq, starts[0::2].copy(), a_len, starts[1::2].copy(), b_len]


def triple_batch(seed: int, n: int, lmin: int = 50, lmax: int = 300,
                 sub=(0.05, 0.20), indel=(0.01, 0.04), ambig: float = 0.02):
    """Triples (child 1, child 2, parent) of a three-way alignment: three
    descendants of one random ancestor of length U[lmin, lmax], each with
    its own substitutions and indels, plus IUPAC ambiguity masks.  Returns a
    list of 3-tuples of uint8 arrays with the leading gap."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        anc = random_dna(rng, int(rng.integers(lmin, lmax + 1)))
        t = []
        for _k in range(3):
            s = mutate(rng, anc, float(rng.uniform(*sub)), float(rng.uniform(*indel)))
            if ambig > 0 and len(s):
                m = rng.random(len(s)) < ambig
                s[m] = AMBIG[rng.integers(0, len(AMBIG), size=int(m.sum()))]
            t.append(with_gap(s))
        out.append(tuple(t))
    return out
