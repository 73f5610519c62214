"""The autotuner (poyd_autotune_batch): every launch variant it times gives
the default's results (it checks costs and lengths and fails otherwise), the
variant it keeps is used by later batches of the class, and those batches'
outputs equal the oracle's."""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import oracle as O
from poyd_gb300 import align, native, synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [12, 3000])
def test_autotune_keeps_results_and_records_a_variant(n):
    native.lib().poyd_autotune_clear()
    host = synth.pair_batch_fast(31 + n, n, lmin=100, lmax=1500)
    batch = align.PairBatch.from_packed([torch.from_numpy(x) for x in host])
    cm = align.CostMatrix.default()
    want = align.align_2(batch, cm, dos_empty=True).to_host()
    tuned = align.autotune(batch, cm, align=True, dos_empty=True, reps=1)
    assert len(tuned["tried"]) >= 2
    p, b, s = C.c_int32(), C.c_int32(), C.c_int32()
    assert native.lib().poyd_autotune_get(0, 1, tuned["lg_pairs"], tuned["lg_width"],
                                          C.byref(p), C.byref(b), C.byref(s)) == 1
    assert (p.value, b.value, s.value) == (tuned["packed"], tuned["blocks_per_sm"], tuned["solo"])
    got = align.align_2(batch, cm, dos_empty=True).to_host()
    for x, y in zip(want, got):
        assert x["cost"] == y["cost"]
        for k in ("a", "b", "median_wg", "median"):
            assert np.array_equal(x[k], y[k])
    # spot check against the oracle
    om = O.cm_dna(1, 2, -1)
    seq, ao, al, bo, bl = host
    for i in range(0, n, max(1, n // 8)):
        a = seq[ao[i]:ao[i] + al[i]]
        b_ = seq[bo[i]:bo[i] + bl[i]]
        c, med, _, _, _ = O.dos_median(a, b_, om)
        assert c == got[i]["cost"] and np.array_equal(med, got[i]["median"])
    native.lib().poyd_autotune_clear()


def test_autotune_cost_mode():
    native.lib().poyd_autotune_clear()
    host = synth.pair_batch_fast(5, 2000, lmin=100, lmax=2000)
    batch = align.PairBatch.from_packed([torch.from_numpy(x) for x in host])
    cm = align.CostMatrix.default()
    want, _ = align.cost_2(batch, cm, deltaw="dos")
    tuned = align.autotune(batch, cm, align=False, deltaw="dos", reps=1)
    assert len(tuned["tried"]) >= 2
    got, _ = align.cost_2(batch, cm, deltaw="dos")
    assert torch.equal(want, got)
    native.lib().poyd_autotune_clear()
