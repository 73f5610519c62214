"""Three-sequence alignment of the Iterative (ThreeD) cost mode.

Python mirror of ``Sequence.Align.align_3_powell`` / ``readjust_3d``
(sequence.ml:1075-1140) over the library's batched kernels
(``csrc/three.cu``).  Sequences are uint8 arrays with POY's leading gap at
position 0.  The cost equals ``powell_3D_align``'s (ukkCommon.c:111-143);
among equally cheap alignments the kernel keeps its own choice (see
``include/poyd_gb300.h``)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from .align import CostMatrix, _stream_handle
from .native import check, lib


class TripleBatch:
    """k sequences per item (3 for align_3_powell: a, b, c; 4 for
    readjust_3d: s1, s2, m, p) packed in one device byte buffer."""

    def __init__(self, seq, offs, lens):
        self.seq, self.offs, self.lens = seq, offs, lens

    @property
    def n(self) -> int:
        return int(self.lens[0].numel())

    @staticmethod
    def pack_host(items):
        k = len(items[0]) if items else 3
        n = len(items)
        lens = np.array([[len(x) for x in it] for it in items], dtype=np.int64).reshape(n, k)
        flat = lens.reshape(-1)
        offs = np.zeros(flat.size + 1, dtype=np.int64)
        np.cumsum(flat, out=offs[1:])
        seq = np.zeros(int(offs[-1]) + 64, dtype=np.uint8)
        q = 0
        for it in items:
            for x in it:
                seq[offs[q]:offs[q + 1]] = np.asarray(x, dtype=np.uint8)
                q += 1
        o = offs[:-1].reshape(n, k)
        return seq, [o[:, j].copy() for j in range(k)], [lens[:, j].astype(np.int32) for j in range(k)]

    @classmethod
    def from_host(cls, items, device="cuda") -> "TripleBatch":
        seq, offs, lens = cls.pack_host(items)
        return cls(torch.from_numpy(seq).to(device),
                   [torch.from_numpy(x).to(device) for x in offs],
                   [torch.from_numpy(x).to(device) for x in lens])

    def out_layout(self):
        """Slots of 4 sequences of cap = a + b + c (first three lengths)
        rounded up to a multiple of 4."""
        tot = self.lens[0].to(torch.int64) + self.lens[1].to(torch.int64)
        tot = tot + (self.lens[3] if len(self.lens) == 4 else self.lens[2]).to(torch.int64)
        cap = (tot + 3) // 4 * 4
        sizes = 4 * cap
        off = torch.zeros_like(sizes)
        if self.n:
            off[1:] = torch.cumsum(sizes, 0)[:-1]
        return off, int((off[-1] + sizes[-1]).item()) if self.n else 0, cap


class ThreeResult:
    def __init__(self, cost, out, out_off, out_len, cap, changed=None):
        self.cost, self.out, self.out_off, self.out_len, self.cap = cost, out, out_off, out_len, cap
        self.changed = changed

    def to_host(self):
        """List of dicts: cost, aligned a, b, c, median (and changed)."""
        out = self.out.cpu().numpy()
        off = self.out_off.cpu().numpy()
        ln = self.out_len.view(-1, 2).cpu().numpy()
        cap = self.cap.cpu().numpy()
        cost = self.cost.cpu().numpy()
        ch = self.changed.cpu().numpy() if self.changed is not None else None
        res = []
        for i in range(len(cost)):
            c, o = int(cap[i]), int(off[i])
            n, nm = int(ln[i, 0]), int(ln[i, 1])
            d = {"cost": int(cost[i]),
                 "a": out[o + c - n:o + c].copy() if n > 0 else np.zeros(0, np.uint8),
                 "b": out[o + 2 * c - n:o + 2 * c].copy() if n > 0 else np.zeros(0, np.uint8),
                 "c": out[o + 3 * c - n:o + 3 * c].copy() if n > 0 else np.zeros(0, np.uint8),
                 "median": out[o + 4 * c - nm:o + 4 * c].copy() if nm > 0 else np.zeros(0, np.uint8)}
            if ch is not None:
                d["changed"] = bool(ch[i])
            res.append(d)
        return res


def median3_table(cm: CostMatrix) -> np.ndarray:
    """``Cost_matrix.Three_D.of_two_dim`` medians (cost_matrix.ml:803-851),
    32,768 bytes indexed (i << 10) | (j << 5) | k."""
    tab = np.zeros(32768, dtype=np.uint8)
    check(lib().poyd_cm_median3(cm.ref, tab.ctypes.data))
    return tab


def powell_params(cm: CostMatrix):
    """(mm, go, ge) of align_3_powell_inter (sequence.ml:1091-1102)."""
    return cm.cost(1, 2), (cm.gap_opening if cm.affine else 0), cm.cost(1, 16)


def align_3_powell(batch: TripleBatch, mm: int, go: int, ge: int, cm: CostMatrix | None = None,
                   stream=None) -> ThreeResult:
    """Batched ``align_3_powell`` (sequence.ml:1078-1087); with `cm`, also
    the median ``align_3_powell_inter`` builds (sequence.ml:1103-1115)."""
    dev = batch.seq.device
    out_off, total, cap = batch.out_layout()
    out = torch.empty(max(total, 16), dtype=torch.uint8, device=dev)
    cost = torch.empty(batch.n, dtype=torch.int32, device=dev)
    out_len = torch.empty(2 * batch.n, dtype=torch.int32, device=dev)
    tab = median3_table(cm) if cm is not None else None
    o, l = batch.offs, batch.lens
    check(lib().poyd_powell_3d_batch(
        batch.n, batch.seq.data_ptr(), o[0].data_ptr(), l[0].data_ptr(), o[1].data_ptr(),
        l[1].data_ptr(), o[2].data_ptr(), l[2].data_ptr(), mm, go, ge,
        tab.ctypes.data if tab is not None else None, cost.data_ptr(), out.data_ptr(),
        out_off.data_ptr(), out_len.data_ptr(), _stream_handle(stream)))
    return ThreeResult(cost, out, out_off, out_len, cap)


def readjust_3d(batch: TripleBatch, cm: CostMatrix, stream=None) -> ThreeResult:
    """Batched ``Sequence.Align.readjust_3d s1 s2 m cm cm3 p``
    (sequence.ml:1117-1140); items are (s1, s2, m, p)."""
    if len(batch.lens) != 4:
        raise ValueError("readjust_3d items are (s1, s2, m, p)")
    dev = batch.seq.device
    out_off, total, cap = batch.out_layout()  # slots sized by s1 + s2 + p
    out = torch.empty(max(total, 16), dtype=torch.uint8, device=dev)
    cost = torch.empty(batch.n, dtype=torch.int32, device=dev)
    out_len = torch.empty(2 * batch.n, dtype=torch.int32, device=dev)
    changed = torch.empty(batch.n, dtype=torch.int32, device=dev)
    o, l = batch.offs, batch.lens
    check(lib().poyd_readjust_3d_batch(
        cm.ref, batch.n, batch.seq.data_ptr(), o[0].data_ptr(), l[0].data_ptr(), o[1].data_ptr(),
        l[1].data_ptr(), o[2].data_ptr(), l[2].data_ptr(), o[3].data_ptr(), l[3].data_ptr(),
        cost.data_ptr(), out.data_ptr(), out_off.data_ptr(), out_len.data_ptr(), changed.data_ptr(),
        _stream_handle(stream)))
    return ThreeResult(cost, out, out_off, out_len, cap, changed)


def powell_3D_align(sa, sb, sc, mm: int, go: int, ge: int):
    """The OCaml external ``powell_3d`` (sequence.ml:1075-1076) on host
    sequences: (aligned a, aligned b, aligned c, cost)."""
    sa, sb, sc = (np.ascontiguousarray(x, dtype=np.uint8) for x in (sa, sb, sc))
    cap = len(sa) + len(sb) + len(sc)
    ra, rb, rc = (np.zeros(cap, dtype=np.uint8) for _ in range(3))
    n, cost = C.c_int32(), C.c_int32()
    check(lib().poyd_powell_3D_align(sa.ctypes.data, len(sa), sb.ctypes.data, len(sb),
                                     sc.ctypes.data, len(sc), ra.ctypes.data, rb.ctypes.data,
                                     rc.ctypes.data, cap, C.byref(n), mm, go, ge, C.byref(cost)))
    k = n.value
    return ra[cap - k:].copy(), rb[cap - k:].copy(), rc[cap - k:].copy(), cost.value
