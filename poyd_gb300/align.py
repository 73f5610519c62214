"""Host-side mirror of POY's ``Sequence.Align`` / ``DOS`` scoring interface
over the batched GB300 kernels.

The reference scores one pair per call (``Sequence.Align.cost_2``,
``align_2``, ``median_2`` ..., sequence.ml:453-1033; ``DOS.median`` /
``DOS.distance``, seqCS.ml:747-867).  Here the same functions take a
:class:`PairBatch` of device-resident pairs in the caller's argument order
and return device tensors; the single-pair forms are thin wrappers over a
batch of one.  Results are bit-identical to the reference's C kernels.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import native
from .native import PoydCM, check, lib


class CostMatrix:
    """``Cost_matrix.Two_D.m`` for the DNA bitmask alphabet (lcm 5)."""

    def __init__(self, cm: PoydCM):
        self._cm = cm

    @classmethod
    def dna(cls, sub: int = 1, indel: int = 2, gap_opening: int | None = None) -> "CostMatrix":
        """``of_transformations_and_gaps true 5 sub indel 31`` then, when
        gap_opening is given, ``set_affine (Affine gap_opening)``."""
        m = PoydCM()
        check(lib().poyd_cm_dna(C.byref(m), sub, indel, -1 if gap_opening is None else gap_opening))
        return cls(m)

    @classmethod
    def default(cls) -> "CostMatrix":
        """``Cost_matrix.Two_D.default`` (substitution 1, indel 2)."""
        return cls.dna(1, 2)

    @classmethod
    def of_matrix5(cls, mat, gap_opening: int | None = None) -> "CostMatrix":
        arr = np.ascontiguousarray(np.asarray(mat, dtype=np.int32).reshape(25))
        m = PoydCM()
        check(lib().poyd_cm_of_matrix5(C.byref(m), arr.ctypes.data,
                                       -1 if gap_opening is None else gap_opening))
        return cls(m)

    @property
    def gap(self) -> int:
        return self._cm.gap

    @property
    def affine(self) -> bool:
        return self._cm.cost_model == 1

    @property
    def gap_opening(self) -> int:
        return self._cm.gap_open

    def cost(self, a: int, b: int) -> int:
        return self._cm.cost[(a << 5) + b]

    def median(self, a: int, b: int) -> int:
        return self._cm.median[(a << 5) + b]

    def tables(self) -> dict:
        return {
            "cost": np.ctypeslib.as_array(self._cm.cost).copy(),
            "worst": np.ctypeslib.as_array(self._cm.worst).copy(),
            "prepend": np.ctypeslib.as_array(self._cm.prepend).copy(),
            "tail": np.ctypeslib.as_array(self._cm.tail).copy(),
            "median": np.ctypeslib.as_array(self._cm.median).copy(),
        }

    @property
    def ref(self):
        return C.byref(self._cm)


def _stream_handle(stream):
    if stream is None:
        stream = torch.cuda.current_stream()
    return C.c_void_p(stream.cuda_stream)


class PairBatch:
    """Pairs (a_i, b_i) packed in one device byte buffer.

    a and b are the caller's arguments in order; each sequence carries POY's
    leading gap at position 0."""

    def __init__(self, seq, a_off, a_len, b_off, b_len):
        self.seq, self.a_off, self.a_len, self.b_off, self.b_len = seq, a_off, a_len, b_off, b_len

    @property
    def n(self) -> int:
        return int(self.a_len.numel())

    @staticmethod
    def pack_host(a_list, b_list, pin: bool = False):
        """Host arrays for a batch: (seq, a_off, a_len, b_off, b_len)."""
        n = len(a_list)
        la = np.fromiter((len(x) for x in a_list), dtype=np.int32, count=n)
        lb = np.fromiter((len(x) for x in b_list), dtype=np.int32, count=n)
        # interleave a_i, b_i so that a pair's bytes are adjacent
        lens = np.empty(2 * n, dtype=np.int64)
        lens[0::2] = la
        lens[1::2] = lb
        offs = np.zeros(2 * n + 1, dtype=np.int64)
        np.cumsum(lens, out=offs[1:])
        seq = np.empty(int(offs[-1]) + 64, dtype=np.uint8)
        seq[int(offs[-1]):] = 0
        for i in range(n):
            seq[offs[2 * i]:offs[2 * i + 1]] = a_list[i]
            seq[offs[2 * i + 1]:offs[2 * i + 2]] = b_list[i]
        out = [seq, offs[0:-1:2].copy(), la, offs[1::2].copy(), lb]
        if pin:
            out = [torch.from_numpy(x).pin_memory() for x in out]
        return out

    @classmethod
    def from_host(cls, a_list, b_list, device="cuda") -> "PairBatch":
        parts = cls.pack_host(a_list, b_list)
        t = [torch.from_numpy(x).to(device) for x in parts]
        return cls(*t)

    @classmethod
    def from_packed(cls, parts, device="cuda", non_blocking=False) -> "PairBatch":
        t = [(x if torch.is_tensor(x) else torch.from_numpy(x)).to(device, non_blocking=non_blocking)
             for x in parts]
        return cls(*t)

    def out_layout(self):
        """Per-pair output slot offsets: 4 sequences of cap = la + lb + 2
        rounded up to a multiple of 4 (the library's slot_cap)."""
        cap = (self.a_len.to(torch.int64) + self.b_len.to(torch.int64) + 2 + 3) // 4 * 4
        sizes = 4 * cap
        off = torch.zeros_like(sizes)
        off[1:] = torch.cumsum(sizes, 0)[:-1]
        return off, int((off[-1] + sizes[-1]).item()) if self.n else 0, cap


def cost_2(batch: PairBatch, cm: CostMatrix, deltaw=None, band_cells: bool = False,
           stream=None):
    """Batched ``Sequence.Align.cost_2`` (sequence.ml:716-723).

    deltaw: None (the ``?deltaw``-less policy), ``"dos"`` (``DOS.distance``'s
    ``max(|la-lb|, 8)``), or an int32 device tensor of explicit values.
    Returns (cost int32 tensor, band-cells int64 tensor or None)."""
    dev = batch.seq.device
    cost = torch.empty(batch.n, dtype=torch.int32, device=dev)
    cells = torch.empty(batch.n, dtype=torch.int64, device=dev) if band_cells else None
    if deltaw is None:
        policy, dptr = native.DELTAW_DEFAULT, None
    elif isinstance(deltaw, str) and deltaw == "dos":
        policy, dptr = native.DELTAW_DOS_DISTANCE, None
    else:
        policy, dptr = native.DELTAW_EXPLICIT, deltaw.to(dev, torch.int32).contiguous()
    check(lib().poyd_cost_2_batch(
        cm.ref, batch.n, batch.seq.data_ptr(), batch.a_off.data_ptr(), batch.a_len.data_ptr(),
        batch.b_off.data_ptr(), batch.b_len.data_ptr(), policy,
        dptr.data_ptr() if dptr is not None else None, cost.data_ptr(),
        cells.data_ptr() if cells is not None else None, _stream_handle(stream)))
    return cost, cells


@dataclass
class AlignResult:
    """Device outputs of :func:`align_2` (right-aligned sequences, as the
    reference's ``seq`` prepend buffers hold them)."""

    cost: torch.Tensor      # int32 [n]
    out: torch.Tensor       # uint8 slots
    out_off: torch.Tensor   # int64 [n]
    out_len: torch.Tensor   # int32 [n, 2]: aligned length, median length
    cap: torch.Tensor       # int64 [n]
    band_cells: torch.Tensor | None

    def to_host(self):
        """List of dicts with numpy arrays: aligned a, aligned b, median with
        gaps, median, and the cost."""
        out = self.out.cpu().numpy()
        off = self.out_off.cpu().numpy()
        ln = self.out_len.view(-1, 2).cpu().numpy()
        if len(ln) and ln.min() < 0:
            raise native.PoydError(-3, "traceback left the band for pair(s) "
                                   f"{np.nonzero(ln[:, 0] < 0)[0][:8].tolist()}")
        cap = self.cap.cpu().numpy()
        cost = self.cost.cpu().numpy()
        res = []
        for i in range(len(cost)):
            c, o = int(cap[i]), int(off[i])
            n, nm = int(ln[i, 0]), int(ln[i, 1])
            res.append({
                "cost": int(cost[i]),
                "a": out[o + c - n:o + c].copy(),
                "b": out[o + 2 * c - n:o + 2 * c].copy(),
                "median_wg": out[o + 3 * c - n:o + 3 * c].copy(),
                "median": out[o + 4 * c - nm:o + 4 * c].copy(),
            })
        return res


    def pack(self, stream=None) -> "PackedAlignments":
        """The results packed back to back on the device (aligned a, aligned
        b, median with gaps, median per pair), ready for one download of
        only the bytes that hold results."""
        n = self.cost.numel()
        dev = self.cost.device
        ln = self.out_len.view(-1, 2).to(torch.int64)
        sizes = 3 * ln[:, 0] + ln[:, 1]
        off = torch.cumsum(sizes, 0) - sizes
        if n:
            total, lo = torch.stack([sizes.sum(), ln.min()]).cpu().tolist()
        else:
            total, lo = 0, 0
        if lo < 0:
            raise native.PoydError(-3, "traceback left the band for pair(s) "
                                   f"{torch.nonzero(ln[:, 0] < 0).flatten()[:8].tolist()}")
        packed = torch.empty(max(total, 16), dtype=torch.uint8, device=dev)
        a_len = (self.cap - 2).to(torch.int32)  # slot_cap(cap - 2, 0) == cap
        zeros = torch.zeros_like(a_len)
        check(lib().poyd_pack_alignments(
            n, self.out.data_ptr(), self.out_off.data_ptr(), a_len.data_ptr(), zeros.data_ptr(),
            self.out_len.data_ptr(), packed.data_ptr(), off.data_ptr(), _stream_handle(stream)))
        return PackedAlignments(self.cost, packed[:total], self.out_len)


@dataclass
class PackedAlignments:
    """Batched align_2 results packed back to back (see AlignResult.pack):
    pair i holds 3 * n_i + m_i bytes, n_i = out_len[2i], m_i = out_len[2i+1]."""

    cost: torch.Tensor     # int32 [n]
    packed: torch.Tensor   # uint8
    out_len: torch.Tensor  # int32 [n, 2]

    def to_host(self):
        """Same dicts as AlignResult.to_host, from the packed bytes (which may
        already be host tensors)."""
        buf = self.packed.cpu().numpy()
        ln = self.out_len.view(-1, 2).cpu().numpy().astype(np.int64)
        cost = self.cost.cpu().numpy()
        sizes = 3 * ln[:, 0] + ln[:, 1]
        off = np.cumsum(sizes) - sizes
        res = []
        for i in range(len(cost)):
            o, n, nm = int(off[i]), int(ln[i, 0]), int(ln[i, 1])
            res.append({
                "cost": int(cost[i]),
                "a": buf[o:o + n].copy(),
                "b": buf[o + n:o + 2 * n].copy(),
                "median_wg": buf[o + 2 * n:o + 3 * n].copy(),
                "median": buf[o + 3 * n:o + 3 * n + nm].copy(),
            })
        return res


def align_2(batch: PairBatch, cm: CostMatrix, dos_empty: bool = False,
            band_cells: bool = False, stream=None, layout=None) -> AlignResult:
    """Batched ``DOS.median`` pieces (seqCS.ml:747-776): ``align_2``,
    ``ancestor_2`` and ``median_2_with_gaps`` for the linear model, or
    ``align_affine_3`` for an affine matrix.  `layout` may bring the
    output layout (out_off, total, cap) the caller computed from host
    copies of the lengths, saving the device read-back of the total."""
    dev = batch.seq.device
    out_off, total, cap = batch.out_layout() if layout is None else layout
    out = torch.empty(max(total, 16), dtype=torch.uint8, device=dev)
    cost = torch.empty(batch.n, dtype=torch.int32, device=dev)
    out_len = torch.empty(2 * batch.n, dtype=torch.int32, device=dev)
    cells = torch.empty(batch.n, dtype=torch.int64, device=dev) if band_cells else None
    check(lib().poyd_align_2_batch(
        cm.ref, batch.n, batch.seq.data_ptr(), batch.a_off.data_ptr(), batch.a_len.data_ptr(),
        batch.b_off.data_ptr(), batch.b_len.data_ptr(), cost.data_ptr(), out.data_ptr(),
        out_off.data_ptr(), out_len.data_ptr(), cells.data_ptr() if cells is not None else None,
        native.FLAG_DOS_EMPTY if dos_empty else 0, _stream_handle(stream)))
    return AlignResult(cost, out, out_off, out_len, cap, cells)


def autotune(batch: PairBatch, cm: CostMatrix, align: bool = True, deltaw=None,
             dos_empty: bool = False, reps: int = 2, stream=None) -> dict:
    """Times the launch variants of the batched linear DP on this batch
    (``poyd_autotune_batch``) and keeps the fastest for every later batch
    of its shape class; all variants give identical results (checked).
    `align` tunes ``align_2``, else ``cost_2`` with `deltaw` ("dos" or
    None).  Returns the variant kept and the time of each tried."""
    dev = batch.seq.device
    cost = torch.empty(batch.n, dtype=torch.int32, device=dev)
    out = out_off = out_len = None
    if align:
        out_off, total, _ = batch.out_layout()
        out = torch.empty(max(total, 16), dtype=torch.uint8, device=dev)
        out_len = torch.empty(2 * batch.n, dtype=torch.int32, device=dev)
    pol = native.DELTAW_DOS_DISTANCE if deltaw == "dos" else native.DELTAW_DEFAULT
    res = native.PoydTuneResult()
    ptr = lambda t: t.data_ptr() if t is not None else None
    check(lib().poyd_autotune_batch(
        cm.ref, int(bool(align)), batch.n, batch.seq.data_ptr(), batch.a_off.data_ptr(),
        batch.a_len.data_ptr(), batch.b_off.data_ptr(), batch.b_len.data_ptr(), pol,
        cost.data_ptr(), ptr(out), ptr(out_off), ptr(out_len),
        native.FLAG_DOS_EMPTY if dos_empty else 0, int(reps), C.byref(res),
        _stream_handle(stream)))
    tried = [{"packed": res.variant[i][0], "blocks_per_sm": res.variant[i][1],
              "solo": res.variant[i][2], "ms": float(res.ms[i])} for i in range(res.n_variants)]
    return {"packed": res.packed, "blocks_per_sm": res.blocks_per_sm, "solo": res.solo,
            "lg_pairs": res.lg_pairs, "lg_width": res.lg_width, "tried": tried}


def host_outputs(parts, pin: bool = True) -> dict:
    """Host result buffers for :func:`align_2_host` on a batch whose host
    arrays are `parts` (``PairBatch.pack_host``); reusable across calls."""
    a_len = torch.as_tensor(parts[2]).to(torch.int64)
    b_len = torch.as_tensor(parts[4]).to(torch.int64)
    n = int(a_len.numel())
    cap = (a_len + b_len + 2 + 3) // 4 * 4
    mk = lambda shape, dt: torch.empty(shape, dtype=dt, pin_memory=pin)
    return {"cost": mk(n, torch.int32), "out_len": mk(2 * n, torch.int32),
            "out": mk(max(int(4 * cap.sum()), 16), torch.uint8),
            "out_off": mk(max(n, 1), torch.int64), "cap": cap}


def align_2_host(parts, cm: CostMatrix, dos_empty: bool = False,
                 out: dict | None = None) -> AlignResult:
    """Batched ``align_2`` from and to host memory (``poyd_align_2_host``):
    `parts` are the host arrays of ``PairBatch.pack_host`` (page-locked for
    speed).  The result slots (``align_2``'s layout, at offsets the library
    chooses) are downloaded while the DP runs; everything is returned in
    host memory."""
    parts = [torch.as_tensor(x) for x in parts]
    seq, a_off, a_len, b_off, b_len = parts
    assert seq.dtype == torch.uint8 and a_off.dtype == torch.int64 and a_len.dtype == torch.int32
    n = int(a_len.numel())
    out = out if out is not None else host_outputs(parts, pin=seq.is_pinned())
    check(lib().poyd_align_2_host(
        cm.ref, n, seq.data_ptr(), a_off.data_ptr(), a_len.data_ptr(), b_off.data_ptr(),
        b_len.data_ptr(), out["cost"].data_ptr(), out["out"].data_ptr(), int(out["out"].numel()),
        out["out_off"].data_ptr(), out["out_len"].data_ptr(),
        native.FLAG_DOS_EMPTY if dos_empty else 0))
    return AlignResult(out["cost"][:n], out["out"], out["out_off"][:n], out["out_len"][:2 * n],
                       out["cap"], None)


def closest(batch: PairBatch, cm: CostMatrix, dos_empty: bool = True,
            stream=None) -> AlignResult:
    """Batched ``Sequence.Align.closest`` (sequence.ml:967-1033): pair i =
    (parent single sequence a_i, node median b_i) gives the node's single
    sequence in the ``median`` place of the result (``DOS.to_single``'s
    empty rules with `dos_empty`, seqCS.ml:730-745); ``cost`` is the
    alignment cost of the pair."""
    dev = batch.seq.device
    out_off, total, cap = batch.out_layout()
    out = torch.empty(max(total, 16), dtype=torch.uint8, device=dev)
    cost = torch.empty(batch.n, dtype=torch.int32, device=dev)
    out_len = torch.empty(2 * batch.n, dtype=torch.int32, device=dev)
    check(lib().poyd_closest_batch(
        cm.ref, batch.n, batch.seq.data_ptr(), batch.a_off.data_ptr(), batch.a_len.data_ptr(),
        batch.b_off.data_ptr(), batch.b_len.data_ptr(), cost.data_ptr(), out.data_ptr(),
        out_off.data_ptr(), out_len.data_ptr(), native.FLAG_DOS_EMPTY if dos_empty else 0,
        _stream_handle(stream)))
    return AlignResult(cost, out, out_off, out_len, cap, None)


# ---- single-pair forms with the reference's signatures --------------------

def cost_2_pair(s1, s2, cm: CostMatrix, deltaw: int | None = None) -> int:
    b = PairBatch.from_host([np.asarray(s1, np.uint8)], [np.asarray(s2, np.uint8)])
    d = None if deltaw is None else torch.tensor([deltaw], dtype=torch.int32, device=b.seq.device)
    c, _ = cost_2(b, cm, d)
    return int(c.item())


def align_2_pair(s1, s2, cm: CostMatrix):
    """``Sequence.Align.align_2 s1 s2 c m`` -> (s1', s2', cost)."""
    b = PairBatch.from_host([np.asarray(s1, np.uint8)], [np.asarray(s2, np.uint8)])
    r = align_2(b, cm).to_host()[0]
    return r["a"], r["b"], r["cost"]


# ---- column operations on aligned pairs (no DP) ------------------------------

_COLUMN_SEQ = {"median_2_with_gaps": "poyd_median_2_with_gaps_batch",
               "median_2_no_gaps": "poyd_median_2_no_gaps_batch",
               "ancestor_2": "poyd_ancestor_2_batch"}
_COLUMN_VAL = {"worst_2": "poyd_worst_2_batch", "verify_2": "poyd_verify_2_batch"}


def columns(op: str, a_list, b_list, cm: CostMatrix, device="cuda", stream=None):
    """Batched column operation `op` on aligned pairs (a_i, b_i of equal
    length): ``median_2_with_gaps``, ``median_2_no_gaps``, ``ancestor_2``
    (lists of uint8 arrays) or ``worst_2``, ``verify_2`` (int costs)."""
    assert all(len(x) == len(y) for x, y in zip(a_list, b_list)), "pairs must be aligned"
    b = PairBatch.from_host(a_list, b_list, device)
    ln = b.a_len
    if op in _COLUMN_VAL:
        val = torch.empty(b.n, dtype=torch.int32, device=device)
        check(getattr(lib(), _COLUMN_VAL[op])(
            cm.ref, b.n, b.seq.data_ptr(), b.a_off.data_ptr(), b.b_off.data_ptr(), ln.data_ptr(),
            val.data_ptr(), _stream_handle(stream)))
        return [int(x) for x in val.cpu().numpy()]
    cap = ln.to(torch.int64) + 1
    off = torch.cumsum(cap, 0) - cap
    out = torch.empty(max(int(cap.sum()), 16), dtype=torch.uint8, device=device)
    out_len = torch.empty(b.n, dtype=torch.int32, device=device)
    check(getattr(lib(), _COLUMN_SEQ[op])(
        cm.ref, b.n, b.seq.data_ptr(), b.a_off.data_ptr(), b.b_off.data_ptr(), ln.data_ptr(),
        out.data_ptr(), off.data_ptr(), out_len.data_ptr(), _stream_handle(stream)))
    o, n, e = out.cpu().numpy(), out_len.cpu().numpy(), (off + cap).cpu().numpy()
    return [o[int(e[i]) - int(n[i]):int(e[i])].copy() for i in range(b.n)]


def column_pair(op: str, a, b, cm: CostMatrix):
    """Single-pair form with the reference's signature (host buffers)."""
    a = np.ascontiguousarray(a, np.uint8)
    b = np.ascontiguousarray(b, np.uint8)
    assert len(a) == len(b), "pairs must be aligned"
    p = lambda x: x.ctypes.data_as(C.c_void_p)
    if op in _COLUMN_VAL:
        v = C.c_int32()
        check(getattr(lib(), "poyd_algn_" + op)(p(a), p(b), len(a), cm.ref, C.byref(v)))
        return int(v.value)
    out = np.zeros(len(a) + 1, np.uint8)
    n = C.c_int32()
    check(getattr(lib(), "poyd_algn_" + op)(p(a), p(b), len(a), cm.ref, p(out), C.byref(n)))
    return out[:n.value].copy()
