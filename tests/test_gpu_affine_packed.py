"""The packed affine kernel (two pairs per lane group in 16-bit halves,
ranks folded into the values) against the 32-bit affine kernel
(POYD_AFF_PACKED=0) and the oracle: costs and every output byte, align
(bt) and cost (nobt), on config-1 pairs and under three affine models."""
import os

import numpy as np
import pytest
import torch

from oracle import oracle as O
from poyd_gb300 import align, synth

pytestmark = pytest.mark.gpu


def _run(batch, cm, packed, fn):
    old = os.environ.get("POYD_AFF_PACKED")
    os.environ["POYD_AFF_PACKED"] = "1" if packed else "0"
    try:
        return fn(batch, cm)
    finally:
        if old is None:
            os.environ.pop("POYD_AFF_PACKED")
        else:
            os.environ["POYD_AFF_PACKED"] = old


@pytest.mark.parametrize("model", [(1, 2, 3), (2, 1, 1), (3, 1, 5)])
def test_packed_affine_equals_32bit_and_oracle(model):
    host = synth.pair_batch_fast(7 + model[2], 2048, lmin=100, lmax=5000)
    batch = align.PairBatch.from_packed([torch.from_numpy(x) for x in host])
    cm = align.CostMatrix.dna(*model)
    al = lambda b, c: align.align_2(b, c, dos_empty=True).to_host()
    p, q = _run(batch, cm, True, al), _run(batch, cm, False, al)
    for i, (x, y) in enumerate(zip(p, q)):
        assert x["cost"] == y["cost"], i
        for k in ("a", "b", "median_wg", "median"):
            assert np.array_equal(x[k], y[k]), (i, k)
    cs = lambda b, c: align.cost_2(b, c)[0]
    assert torch.equal(_run(batch, cm, True, cs), _run(batch, cm, False, cs))
    om = O.cm_dna(*model)
    seq, ao, al_, bo, bl = host
    for i in range(0, 2048, 97):
        c, med, ra, rb, wg = O.dos_median(seq[ao[i]:ao[i] + al_[i]], seq[bo[i]:bo[i] + bl[i]], om)
        assert c == p[i]["cost"] and np.array_equal(med, p[i]["median"]), i
        assert np.array_equal(ra, p[i]["a"]) and np.array_equal(rb, p[i]["b"]), i


def test_packed_affine_small_and_ragged_batches():
    """Odd batch sizes (a lone pair in a lane group), length-1 and all-gap
    sequences, and unrelated pairs of very different lengths."""
    rng = np.random.default_rng(11)
    A, B = [], []
    for n in (1, 2, 3, 5, 40):
        for _ in range(n):
            la, lb = int(rng.integers(1, 300)), int(rng.integers(1, 3000))
            a = synth.with_gap(synth.random_dna(rng, la - 1, 0.05))
            b = synth.with_gap(synth.random_dna(rng, lb - 1, 0.05))
            if rng.random() < 0.1:
                a[1:] = 16
            A.append(a)
            B.append(b)
    batch = align.PairBatch.from_host(A, B)
    cm = align.CostMatrix.dna(1, 2, 3)
    al = lambda b, c: align.align_2(b, c, dos_empty=True).to_host()
    p, q = _run(batch, cm, True, al), _run(batch, cm, False, al)
    for x, y in zip(p, q):
        assert x["cost"] == y["cost"]
        for k in ("a", "b", "median_wg", "median"):
            assert np.array_equal(x[k], y[k])
