"""Fitch on 16- and 32-bit state sets (NonaddCS16 / NonaddCS32) through
the CUDA kernels against the oracle, whose wide rules are pinned against
nonaddCSc.c built at CHARSIZE 16 / 32: distance, median (with the added
cost) and median_3, bit-exact, over ragged row lengths."""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import oracle as O
from poyd_gb300 import native

pytestmark = pytest.mark.gpu

DT = {16: np.uint16, 32: np.uint32}


def _sets(rng, shape, width):
    """Non-empty state sets of 1-3 states out of `width`."""
    out = np.zeros(shape, np.uint64)
    for _ in range(3):
        bit = rng.integers(0, width, shape).astype(np.uint64)
        out |= np.where(rng.random(shape) < 0.6, np.uint64(1) << bit, np.uint64(0))
    out[out == 0] = 1
    return out.astype(DT[width])


def _lib():
    L = C.CDLL(native.LIB_PATH)
    vp, i32, i64 = C.c_void_p, C.c_int32, C.c_int64
    for w in (16, 32):
        getattr(L, "poyd_nonadd%d_distance_batch" % w).argtypes = [vp, i64, i32, i32, vp, vp, vp, vp]
        getattr(L, "poyd_nonadd%d_median_batch" % w).argtypes = [vp, i64, i32, i32, vp, vp, vp, vp, vp]
        getattr(L, "poyd_nonadd%d_median_3_batch" % w).argtypes = [vp, i64, i32, i32, vp, vp, vp,
                                                                   vp, vp, vp]
    return L


def _p(t):
    return C.c_void_p(t.data_ptr())


@pytest.mark.parametrize("width", [16, 32])
def test_wide_fitch_matches_oracle(width):
    L = _lib()
    eb = width // 8
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(width)
    for length in (1, 3, 4, 5, 8, 9, 17, 257, 2000):
        n_nodes, n = 24, 150
        rows = _sets(rng, (n_nodes, length), width)
        stride = (length * eb + 15) // 16 * 16
        buf = rng.integers(0, 256, (n_nodes, stride), dtype=np.uint8)  # bytes past the rows
        buf[:, :length * eb] = rows.view(np.uint8).reshape(n_nodes, -1)
        dn = torch.from_numpy(buf).cuda()
        ai = rng.integers(0, n_nodes, n).astype(np.int32)
        bi = rng.integers(0, n_nodes, n).astype(np.int32)
        ci = rng.integers(0, n_nodes, n).astype(np.int32)
        di = rng.integers(0, n_nodes, n).astype(np.int32)
        da, db, dc, dd = (torch.from_numpy(x).cuda() for x in (ai, bi, ci, di))
        dist = torch.empty(n, dtype=torch.int64, device="cuda")
        out = torch.empty((n, stride), dtype=torch.uint8, device="cuda")
        added = torch.empty(n, dtype=torch.int64, device="cuda")
        out3 = torch.empty((n, stride), dtype=torch.uint8, device="cuda")
        assert getattr(L, "poyd_nonadd%d_distance_batch" % width)(
            _p(dn), stride, length, n, _p(da), _p(db), _p(dist), st) == 0
        assert getattr(L, "poyd_nonadd%d_median_batch" % width)(
            _p(dn), stride, length, n, _p(da), _p(db), _p(out), _p(added), st) == 0
        assert getattr(L, "poyd_nonadd%d_median_3_batch" % width)(
            _p(dn), stride, length, n, _p(da), _p(db), _p(dc), _p(dd), _p(out3), st) == 0
        torch.cuda.synchronize()
        dist, added = dist.cpu().numpy(), added.cpu().numpy()
        med = out.cpu().numpy()[:, :length * eb].copy().view(DT[width])
        med3 = out3.cpu().numpy()[:, :length * eb].copy().view(DT[width])
        for k in range(n):
            a, b = rows[ai[k]], rows[bi[k]]
            assert dist[k] == O.nonadd_distance_w(a, b, width), (length, k)
            c, m = O.nonadd_median_w(a, b, width)
            assert added[k] == c and np.array_equal(med[k], m), (length, k)
            assert np.array_equal(med3[k], O.nonadd_median_3_w(a, b, rows[ci[k]], rows[di[k]],
                                                               width)), (length, k)


def test_wide_fitch_rejects_short_stride():
    L = _lib()
    buf = torch.zeros((2, 16), dtype=torch.uint8, device="cuda")
    idx = torch.zeros(1, dtype=torch.int32, device="cuda")
    dist = torch.empty(1, dtype=torch.int64, device="cuda")
    # 9 characters of 2 bytes need 32-byte rows
    assert L.poyd_nonadd16_distance_batch(_p(buf), 16, 9, 1, _p(idx), _p(idx), _p(dist),
                                          None) == -1
