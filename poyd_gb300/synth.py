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
