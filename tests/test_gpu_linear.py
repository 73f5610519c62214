"""Parity of the CUDA linear-gap path with the oracle (bit-exact)."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from poyd_gb300 import align, native, synth

pytestmark = pytest.mark.gpu

MODELS = [(1, 2), (1, 1), (3, 1), (2, 3)]


def _edge_pairs(rng):
    A, B = [], []
    g = synth.with_gap
    cases = [(0, 0), (0, 5), (5, 0), (1, 1), (2, 7), (40, 100), (100, 40), (64, 64),
             (63, 65), (31, 33), (200, 301), (301, 200), (1, 300), (150, 149), (500, 10)]
    for n1, n2 in cases:
        A.append(g(synth.random_dna(rng, n1, 0.1)))
        B.append(g(synth.random_dna(rng, n2, 0.1)))
    # all-ambiguous and gap-bearing inputs
    A.append(g(np.full(120, 15, np.uint8)))
    B.append(g(synth.random_dna(rng, 118)))
    a = synth.random_dna(rng, 300)
    b = a.copy()
    b[::7] = 16
    b[5:40] = 16
    A.append(g(a))
    B.append(g(b))
    a = synth.random_dna(rng, 257, 0.05)
    b = a.copy()
    b[rng.random(len(b)) < 0.3] = 31
    A.append(g(a))
    B.append(g(b))
    return A, B


def _random_pairs(seed, n, lmax):
    A, B = synth.pair_batch(seed, n, lmin=1, lmax=lmax)
    rng = np.random.default_rng(seed + 1)
    for _ in range(n // 4):
        A.append(synth.with_gap(synth.random_dna(rng, int(rng.integers(1, lmax)), 0.05)))
        B.append(synth.with_gap(synth.random_dna(rng, int(rng.integers(1, lmax)), 0.05)))
    return A, B


@pytest.mark.parametrize("model", MODELS)
def test_cost_2_matches_oracle(model):
    rng = np.random.default_rng(5)
    A, B = _random_pairs(100 + model[0], 60, 900)
    EA, EB = _edge_pairs(rng)
    A += EA
    B += EB
    cm = align.CostMatrix.dna(*model)
    om = O.cm_dna(model[0], model[1], -1)
    batch = align.PairBatch.from_host(A, B)
    for dw in (None, "dos"):
        cost, cells = align.cost_2(batch, cm, deltaw=dw, band_cells=True)
        cost = cost.cpu().numpy()
        cells = cells.cpu().numpy()
        for i, (a, b) in enumerate(zip(A, B)):
            explicit = None if dw is None else max(abs(len(a) - len(b)), 8)
            assert cost[i] == O.cost_2(a, b, om, explicit), (model, dw, i, len(a), len(b))
            d = O.deltaw(a, b, om, explicit)
            assert cells[i] == O.band_cells_linear(len(a), len(b), d)


def test_cost_2_explicit_deltaw():
    A, B = _random_pairs(7, 40, 600)
    cm = align.CostMatrix.default()
    om = O.cm_dna(1, 2, -1)
    rng = np.random.default_rng(0)
    dws = rng.integers(0, 120, len(A)).astype(np.int32)
    batch = align.PairBatch.from_host(A, B)
    cost, _ = align.cost_2(batch, cm, deltaw=torch.from_numpy(dws).cuda())
    cost = cost.cpu().numpy()
    for i, (a, b) in enumerate(zip(A, B)):
        assert cost[i] == O.cost_2(a, b, om, int(dws[i])), i


@pytest.mark.parametrize("model", MODELS)
def test_align_2_medians_match_oracle(model):
    rng = np.random.default_rng(9)
    A, B = _random_pairs(200 + model[1], 50, 800)
    EA, EB = _edge_pairs(rng)
    A += EA
    B += EB
    cm = align.CostMatrix.dna(*model)
    om = O.cm_dna(model[0], model[1], -1)
    res = align.align_2(align.PairBatch.from_host(A, B), cm).to_host()
    for i, (a, b) in enumerate(zip(A, B)):
        c, ra, rb = O.align_2(a, b, om)
        r = res[i]
        assert r["cost"] == c, (i, len(a), len(b))
        assert np.array_equal(r["a"], ra) and np.array_equal(r["b"], rb), (i, len(a), len(b))
        assert np.array_equal(r["median_wg"], O.median_2_with_gaps(ra, rb, om)), i
        assert np.array_equal(r["median"], O.ancestor_2(ra, rb, om)), i


def test_dos_median_empty_rule():
    rng = np.random.default_rng(3)
    g = synth.with_gap
    A = [g(np.zeros(0, np.uint8)), g(synth.random_dna(rng, 50)), np.array([16, 16, 16], np.uint8)]
    B = [g(synth.random_dna(rng, 40)), g(np.zeros(0, np.uint8)), g(synth.random_dna(rng, 30))]
    cm = align.CostMatrix.default()
    om = O.cm_dna(1, 2, -1)
    res = align.align_2(align.PairBatch.from_host(A, B), cm, dos_empty=True).to_host()
    for i, (a, b) in enumerate(zip(A, B)):
        c, med, ra, rb, wg = O.dos_median(a, b, om)
        assert res[i]["cost"] == c
        assert np.array_equal(res[i]["median"], med)


def test_full_size_properties():
    """Config-sized lengths (up to 5,000) through size-independent checks:
    the aligned pair re-scores to the DP cost (verify_2) and drops back to
    the inputs when gaps are removed."""
    A, B = synth.pair_batch(77, 48, lmin=3000, lmax=5000)
    cm = align.CostMatrix.default()
    om = O.cm_dna(1, 2, -1)
    res = align.align_2(align.PairBatch.from_host(A, B), cm).to_host()
    for i, (a, b) in enumerate(zip(A, B)):
        r = res[i]
        assert O.verify_2(r["a"], r["b"], om) == r["cost"]
        assert np.array_equal(r["a"][r["a"] != 16], a[a != 16])
        assert np.array_equal(r["b"][r["b"] != 16], b[b != 16])
    # and full oracle parity on every pair
    for i in range(48):
        c, med, ra, rb, wg = O.dos_median(A[i], B[i], om)
        r = res[i]
        assert r["cost"] == c and np.array_equal(r["a"], ra) and np.array_equal(r["b"], rb), i
        assert np.array_equal(r["median"], med) and np.array_equal(r["median_wg"], wg), i


def test_codes_above_31_rejected():
    """Element codes index 32-entry table rows: wider codes are refused before
    any DP launch (linear and affine)."""
    from poyd_gb300 import native
    rng = np.random.default_rng(9)
    a = synth.with_gap(synth.random_dna(rng, 50))
    b = synth.with_gap(synth.random_dna(rng, 50))
    b[10] = 40
    batch = align.PairBatch.from_host([a], [b])
    for cm in (align.CostMatrix.dna(1, 2), align.CostMatrix.dna(1, 2, gap_opening=3)):
        with pytest.raises(native.PoydError):
            align.cost_2(batch, cm)
        with pytest.raises(native.PoydError):
            align.align_2(batch, cm)
    ok = align.PairBatch.from_host([a], [synth.with_gap(synth.random_dna(rng, 50))])
    assert int(align.cost_2(ok, align.CostMatrix.dna(1, 2))[0].item()) >= 0


def test_packed_results_equal_slots():
    """AlignResult.pack() carries exactly the slot contents (aligned a, b,
    median with gaps, median per pair), DOS empty-rule pairs included."""
    rng = np.random.default_rng(21)
    A, B = _random_pairs(77, 40, 600)
    EA, EB = _edge_pairs(rng)
    A += EA
    B += EB
    g = synth.with_gap
    A.append(g(np.full(0, 16, np.uint8)))
    B.append(g(synth.random_dna(rng, 30)))
    cm = align.CostMatrix.dna(1, 2)
    res = align.align_2(align.PairBatch.from_host(A, B), cm, dos_empty=True)
    slots = res.to_host()
    packed = res.pack()
    assert packed.packed.numel() == sum(3 * len(r["a"]) + len(r["median"]) for r in slots)
    host = align.PackedAlignments(packed.cost.cpu(), packed.packed.cpu(), packed.out_len.cpu())
    for r, p in zip(slots, host.to_host()):
        assert r["cost"] == p["cost"]
        for k in ("a", "b", "median_wg", "median"):
            assert np.array_equal(r[k], p[k]), k


@pytest.mark.parametrize("pin,model,budget", [(True, (1, 2, None), None),
                                              (False, (1, 1, None), None),
                                              (True, (1, 2, None), 256 * 1024),
                                              (True, (2, 1, 1), None)])
def test_host_buffer_batch_matches_device_batch(pin, model, budget, monkeypatch):
    """poyd_align_2_host (slots in DP order, downloaded while the DP runs;
    several direction-matrix waves; affine) returns every pair's results as
    the device-resident batch does."""
    rng = np.random.default_rng(model[0] * 7 + model[1])
    A, B = _random_pairs(50 + model[1], 90, 900)
    EA, EB = _edge_pairs(rng)
    A += EA
    B += EB
    cm = align.CostMatrix.dna(*model)
    parts = align.PairBatch.pack_host(A, B, pin=pin)
    dev = align.align_2(align.PairBatch.from_host(A, B), cm, dos_empty=True).to_host()
    if budget:
        monkeypatch.setenv("POYD_DM_BUDGET_BYTES", str(budget))
    host = align.align_2_host(parts, cm, dos_empty=True)
    off = host.out_off.numpy()
    cap = host.cap.numpy()
    assert len(set(off.tolist())) == len(off)
    assert np.all(off % 4 == 0) and np.all(off + 4 * cap <= host.out.numel())
    for d, h in zip(dev, host.to_host()):
        assert d["cost"] == h["cost"]
        for k in ("a", "b", "median_wg", "median"):
            assert np.array_equal(d[k], h[k]), k


def test_host_buffer_batch_capacity_checked():
    A, B = _random_pairs(60, 20, 300)
    cm = align.CostMatrix.dna(1, 2)
    parts = align.PairBatch.pack_host(A, B)
    out = align.host_outputs(parts, pin=False)
    out["out"] = out["out"][:100]
    with pytest.raises(native.PoydError):
        align.align_2_host(parts, cm, out=out)
    ok = align.align_2_host(parts, cm)
    assert ok.cost.numel() == len(A)


def test_direction_matrix_waves_match_one_launch(monkeypatch):
    """A batch whose direction matrices exceed the device budget runs in
    waves of the longest-first order; the results are those of one launch."""
    A, B = _random_pairs(91, 80, 700)
    cm = align.CostMatrix.dna(1, 2)
    batch = align.PairBatch.from_host(A, B)
    ref = align.align_2(batch, cm, dos_empty=True).to_host()
    monkeypatch.setenv("POYD_DM_BUDGET_BYTES", str(256 * 1024))
    waved = align.align_2(batch, cm, dos_empty=True).to_host()
    monkeypatch.delenv("POYD_DM_BUDGET_BYTES")
    assert len(ref) == len(waved)
    for r, w in zip(ref, waved):
        assert r["cost"] == w["cost"]
        for k in ("a", "b", "median_wg", "median"):
            assert np.array_equal(r[k], w[k]), k
