"""Input regimes shared by the oracle-vs-reference pins (CPU) and the GPU
parity tests, so both check the same pairs."""
import numpy as np

from poyd_gb300 import synth


def band_case(l1, l2, dw):
    """algn_fill_plane_2's band case (algn.c:880-937) for l1 >= l2: "full"
    (L1 >= 1.5 L2, or L1 - height <= 8), "narrow" (2 height < L1: extend
    right / left-right / extend left) or "rows" (extend right / full rows /
    extend left)."""
    width, height = min(50 + dw, l2), min((l1 - l2) + 50 + dw, l1)
    if np.float32(1.5) * np.float32(l2) <= np.float32(l1):
        return "full"
    if 2 * height < l1:
        return "narrow"
    return "full" if l1 - height <= 8 else "rows"


def config1_pairs(seed, n):
    """The batched-align_2 benchmark's regime: n pairs from its generator at
    1,500-5,000 bp (10-30 % substitutions, 2-5 % indels, 5 % IUPAC), then
    pairs that reach the other band cases at those lengths: a full plane by
    the length ratio, and gap-bearing sequences (their gap count widens
    deltaw) that take the full-rows branch and the L1 - height <= 8 full
    plane."""
    A, B = synth.pair_batch(seed, n, lmin=1500, lmax=5000)
    rng = np.random.default_rng(seed + 1)
    for k in range(4):
        a = synth.with_gap(synth.random_dna(rng, int(rng.integers(3000, 5000)), 0.05))
        keep = int(len(a) / (1.55 + 0.2 * k))
        A.append(a)
        B.append(synth.with_gap(synth.mutate(rng, a[1:keep].copy(), 0.2, 0.03)))
    for frac in (0.45, 0.55, 0.96, 0.99):
        a = synth.with_gap(synth.random_dna(rng, int(rng.integers(2000, 4000)), 0.05))
        b = synth.mutate(rng, a[1:].copy(), 0.15, 0.02)
        g = rng.random(len(b)) < frac
        b[g] = 16 | b[g]  # keep the base, add the gap bit (codes 17-31)
        A.append(a)
        B.append(synth.with_gap(b))
    return A, B
