"""The oracle's batch checker (or_dos_median_check_many, used by bench.py to
verify the headline run's outputs) accepts slots that hold the oracle's own
results and flags a slot where one byte or one cost differs.  CPU only."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from poyd_gb300 import synth


def _slots(host, cm, model_affine):
    """Batched align_2 slots (four right-aligned sequences of cap bytes per
    pair) filled from the oracle's DOS.median."""
    seq, ao, al, bo, bl = host
    n = len(al)
    cap = ((al.astype(np.int64) + bl + 2 + 3) // 4) * 4
    off = np.zeros(n, np.int64)
    off[1:] = np.cumsum(4 * cap)[:-1]
    out = np.zeros(int((4 * cap).sum()), np.uint8)
    cost = np.zeros(n, np.int32)
    ln = np.zeros(2 * n, np.int32)
    for i in range(n):
        a = seq[ao[i]:ao[i] + al[i]]
        b = seq[bo[i]:bo[i] + bl[i]]
        c, med, ra, rb, wg = O.dos_median(a, b, cm)
        o, k = int(off[i]), int(cap[i])
        for j, x in enumerate((ra, rb, wg, med)):
            out[o + (j + 1) * k - len(x):o + (j + 1) * k] = x
        cost[i], ln[2 * i], ln[2 * i + 1] = c, len(ra), len(med)
    return cost, out, off, ln


@pytest.mark.parametrize("affine", [False, True])
def test_check_many_accepts_own_results_and_flags_one_byte(affine):
    host = synth.pair_batch_fast(5, 24, lmin=60, lmax=400)
    cm = O.cm_dna(1, 2, 3 if affine else -1)
    cost, out, off, ln = _slots(host, cm, affine)
    bad_out = out.copy()
    # one byte of pair 7's median with gaps, one cost of pair 11
    cap7 = ((int(host[2][7]) + int(host[4][7]) + 5) // 4) * 4
    bad_out[int(off[7]) + 4 * cap7 - 1 - cap7] ^= 1
    bad_cost = cost.copy()
    bad_cost[11] += 1
    keep = [cost, out, off, ln, bad_out, bad_cost]
    sets = (O.OrResultSet * 3)(
        O.OrResultSet(cost.ctypes.data, out.ctypes.data, off.ctypes.data, ln.ctypes.data),
        O.OrResultSet(cost.ctypes.data, bad_out.ctypes.data, off.ctypes.data, ln.ctypes.data),
        O.OrResultSet(bad_cost.ctypes.data, out.ctypes.data, off.ctypes.data, ln.ctypes.data))
    seq, ao, al, bo, bl = host
    idx = np.arange(len(al), dtype=np.int32)
    ocost = np.zeros(len(idx), np.int32)
    bad = np.zeros(len(idx), np.int32)
    cells = O.lib().or_dos_median_check_many(
        seq.ctypes.data, ao.ctypes.data, al.ctypes.data, bo.ctypes.data, bl.ctypes.data,
        idx.ctypes.data, len(idx), C.byref(cm), ocost.ctypes.data, 3,
        C.cast(sets, C.c_void_p), bad.ctypes.data)
    assert cells > 0 and len(keep) == 6
    assert np.array_equal(ocost, cost)
    assert np.nonzero(bad & 1)[0].tolist() == []
    assert np.nonzero(bad & 2)[0].tolist() == [7]
    assert np.nonzero(bad & 4)[0].tolist() == [11]
