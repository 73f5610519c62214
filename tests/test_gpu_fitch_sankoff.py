"""Fitch (NonaddCS8) and Sankoff kernels against the oracle (bit-exact)."""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import oracle as O
from poyd_gb300 import native
from tests import golden_io as G

pytestmark = pytest.mark.gpu


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _nodes(rng, n_nodes, length, stride):
    nodes = np.zeros((n_nodes, stride), np.uint8)
    states = rng.integers(2, 9, size=length)
    for v in range(n_nodes):
        pick = rng.integers(0, states)
        nodes[v, :length] = (1 << pick).astype(np.uint8)
        amb = rng.random(length) < 0.2
        nodes[v, :length][amb] |= (1 << rng.integers(0, states[amb])).astype(np.uint8)
    nodes[:, length:] = rng.integers(0, 256, size=(n_nodes, stride - length))  # junk padding
    return nodes


@pytest.mark.parametrize("length", [1, 15, 16, 17, 2000, 2047])
def test_fitch_distance_median(length):
    rng = np.random.default_rng(length)
    stride = (length + 15) // 16 * 16 + 16
    nodes = _nodes(rng, 40, length, stride)
    n = 300
    ai = rng.integers(0, 40, n).astype(np.int32)
    bi = rng.integers(0, 40, n).astype(np.int32)
    dn = torch.from_numpy(nodes).cuda()
    da, db = torch.from_numpy(ai).cuda(), torch.from_numpy(bi).cuda()
    dist = torch.empty(n, dtype=torch.int64, device="cuda")
    L = native.lib()
    assert L.poyd_nonadd8_distance_batch(C.c_void_p(dn.data_ptr()), C.c_int64(stride), length, n,
                                         C.c_void_p(da.data_ptr()), C.c_void_p(db.data_ptr()),
                                         C.c_void_p(dist.data_ptr()), _stream()) == 0
    out = torch.empty((n, stride), dtype=torch.uint8, device="cuda")
    added = torch.empty(n, dtype=torch.int64, device="cuda")
    assert L.poyd_nonadd8_median_batch(C.c_void_p(dn.data_ptr()), C.c_int64(stride), length, n,
                                       C.c_void_p(da.data_ptr()), C.c_void_p(db.data_ptr()),
                                       C.c_void_p(out.data_ptr()), C.c_void_p(added.data_ptr()),
                                       _stream()) == 0
    dist, out, added = dist.cpu().numpy(), out.cpu().numpy(), added.cpu().numpy()
    for k in range(n):
        a, b = nodes[ai[k], :length], nodes[bi[k], :length]
        assert dist[k] == O.nonadd_distance(a, b)
        c, med = O.nonadd_median(a, b)
        assert added[k] == c and np.array_equal(out[k, :length], med)


def test_fitch_median3_and_golden():
    g = G.load()
    nodes = g["fitch_nodes"]
    length = nodes.shape[1]
    stride = (length + 15) // 16 * 16
    buf = np.zeros((nodes.shape[0], stride), np.uint8)
    buf[:, :length] = nodes
    dn = torch.from_numpy(buf).cuda()
    L = native.lib()
    idx = lambda *v: torch.tensor(v, dtype=torch.int32, device="cuda")
    out = torch.empty((1, stride), dtype=torch.uint8, device="cuda")
    a, p, d1, d2 = idx(2), idx(3), idx(4), idx(5)
    assert L.poyd_nonadd8_median_3_batch(C.c_void_p(dn.data_ptr()), C.c_int64(stride), length, 1,
                                         *[C.c_void_p(x.data_ptr()) for x in (a, p, d1, d2)],
                                         C.c_void_p(out.data_ptr()), _stream()) == 0
    assert np.array_equal(out.cpu().numpy()[0, :length], g["fitch_median3"])
    dist = torch.empty(36, dtype=torch.int64, device="cuda")
    ai = torch.arange(36, dtype=torch.int32, device="cuda") // 6
    bi = torch.arange(36, dtype=torch.int32, device="cuda") % 6
    assert L.poyd_nonadd8_distance_batch(C.c_void_p(dn.data_ptr()), C.c_int64(stride), length, 36,
                                         C.c_void_p(ai.data_ptr()), C.c_void_p(bi.data_ptr()),
                                         C.c_void_p(dist.data_ptr()), _stream()) == 0
    assert np.array_equal(dist.cpu().numpy().reshape(6, 6), g["fitch_dist"])


@pytest.mark.parametrize("k", [2, 4, 5, 8])
def test_sankoff_median_distance(k):
    rng = np.random.default_rng(k)
    tcm = rng.integers(1, 6, size=(k, k))
    tcm = np.minimum(tcm, tcm.T)
    np.fill_diagonal(tcm, 0)
    nchar, n_nodes, n = 200, 30, 120
    INF = native.SANK_INF
    nodes = rng.integers(0, 12, size=(n_nodes, nchar, k)).astype(np.int32)
    leaf = rng.random((n_nodes, nchar, k)) < 0.5
    nodes[leaf] = INF
    nodes[:, :, 0][leaf.all(axis=2)] = 0  # at least one finite state
    ai = rng.integers(0, n_nodes, n).astype(np.int32)
    bi = rng.integers(0, n_nodes, n).astype(np.int32)
    dn = torch.from_numpy(nodes).cuda()
    dt = torch.from_numpy(tcm.astype(np.int32)).cuda()
    da, db = torch.from_numpy(ai).cuda(), torch.from_numpy(bi).cuda()
    s = torch.empty((n, nchar, k), dtype=torch.int32, device="cuda")
    e, beta = torch.empty_like(s), torch.empty_like(s)
    dist = torch.empty(n, dtype=torch.int64, device="cuda")
    L = native.lib()
    ptr = lambda t: C.c_void_p(t.data_ptr())
    assert L.poyd_sank_median_batch(ptr(dn), nchar, k, ptr(dt), n, ptr(da), ptr(db), ptr(s),
                                    ptr(e), ptr(beta), _stream()) == 0
    assert L.poyd_sank_distance_batch(ptr(dn), nchar, k, ptr(dt), n, ptr(da), ptr(db), ptr(dist),
                                      _stream()) == 0
    s, e, beta, dist = (x.cpu().numpy() for x in (s, e, beta, dist))
    big = O.SANK_INF

    def to_ocaml(x):
        x = x.astype(np.int64)
        x[x >= INF] = big
        return x

    for q in range(n):
        tot = 0.0
        for ch in range(nchar):
            a_s, b_s = to_ocaml(nodes[ai[q], ch]), to_ocaml(nodes[bi[q], ch])
            c, ee, bb = O.sank_elt_median(tcm, a_s, b_s)
            inf_c = c >= big
            assert np.array_equal(s[q, ch] >= INF, inf_c)
            assert np.array_equal(s[q, ch][~inf_c], c[~inf_c])
            inf_e = ee >= big
            assert np.array_equal(e[q, ch] >= INF, inf_e)
            assert np.array_equal(e[q, ch][~inf_e], ee[~inf_e])
            assert np.array_equal(np.minimum(beta[q, ch], INF), np.where(bb >= big, INF, bb))
            tot += O.sank_elt_distance(tcm, a_s, b_s)
        assert dist[q] == tot
