"""poyd_cost_2_batch_noalloc: the batched cost_2 for callers that cannot
allocate device memory (an OCaml C stub inside a host that owns the CUDA
memory pool, a service with a fixed device-memory budget).

It must return exactly the costs of the allocating entry point
(poyd_cost_2_batch) -- integer costs, so the tolerance is zero -- on two
calls in a row, since the calls share one fixed device scratch array that
keeps the previous call's contents.  This file is collected last on
purpose, and passes alone or after the rest of the suite."""
import ctypes as C

import numpy as np
import pytest
import torch

from poyd_gb300 import align, native, synth

pytestmark = pytest.mark.gpu


def _noalloc(batch, cm, policy, out):
    L = native.lib()
    f = L.poyd_cost_2_batch_noalloc
    f.restype = C.c_int
    f.argtypes = [C.POINTER(native.PoydCM), C.c_int32] + [C.c_void_p] * 5 + \
        [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]
    return f(cm.ref, batch.n, batch.seq.data_ptr(), batch.a_off.data_ptr(),
             batch.a_len.data_ptr(), batch.b_off.data_ptr(), batch.b_len.data_ptr(), policy,
             None, out.data_ptr(), C.c_void_p(torch.cuda.current_stream().cuda_stream))


def test_noalloc_matches_allocating_entry_point_twice():
    torch.cuda.set_device(0)
    A, B = synth.pair_batch(4242, 300, lmin=1, lmax=3000)
    rng = np.random.default_rng(1)
    A.append(synth.with_gap(synth.random_dna(rng, 40)))
    B.append(synth.with_gap(synth.random_dna(rng, 400)))  # full-plane band
    batch = align.PairBatch.from_host(A, B)
    cm = align.CostMatrix.default()
    for policy, dw in ((native.DELTAW_DEFAULT, None), (native.DELTAW_DOS_DISTANCE, "dos")):
        expect, _ = align.cost_2(batch, cm, deltaw=dw)
        for call in range(2):
            out = torch.full((batch.n,), -7, dtype=torch.int32, device="cuda")
            rc = _noalloc(batch, cm, policy, out)
            assert rc == 0, native.lib().poyd_last_error()
            torch.cuda.synchronize()
            assert torch.equal(out, expect), (policy, call)


def test_noalloc_rejects_oversize_batch():
    n = 65537
    seq = torch.full((8,), 16, dtype=torch.uint8, device="cuda")
    off = torch.zeros(n, dtype=torch.int64, device="cuda")
    ln = torch.ones(n, dtype=torch.int32, device="cuda")
    batch = align.PairBatch(seq, off, ln, off, ln)
    out = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    rc = _noalloc(batch, align.CostMatrix.default(), native.DELTAW_DEFAULT, out)
    assert rc == -3  # POYD_ERANGE
    assert b"65536" in native.lib().poyd_last_error()
    assert int(out[0].item()) == -7


def test_noalloc_rejects_band_wider_than_scratch():
    """A pair whose band is wider than the 1,984 diagonals a fixed per-warp
    boundary row holds (here a full plane: 2,401 x 301 gives 2,701
    diagonals) is refused with POYD_ERANGE before the DP launch; the cost
    output is left as it was."""
    rng = np.random.default_rng(5)
    A = [synth.with_gap(synth.random_dna(rng, 60)), synth.with_gap(synth.random_dna(rng, 2400))]
    B = [synth.with_gap(synth.random_dna(rng, 50)), synth.with_gap(synth.random_dna(rng, 300))]
    batch = align.PairBatch.from_host(A, B)
    out = torch.full((batch.n,), -7, dtype=torch.int32, device="cuda")
    rc = _noalloc(batch, align.CostMatrix.default(), native.DELTAW_DEFAULT, out)
    assert rc == -3  # POYD_ERANGE
    assert b"1984" in native.lib().poyd_last_error()
    torch.cuda.synchronize()
    assert out.cpu().tolist() == [-7, -7]
