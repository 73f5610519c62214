"""The candidate-pass backend interface of poyd_gb300.search implemented on
the CPU oracle (test infrastructure): DOS.median / DOS.distance, NonaddCS8
and SankCS from oracle/, one pair at a time as the reference does."""
import numpy as np

from oracle import oracle as O
from poyd_gb300.simulate import SANK_INF


class OracleBackend:
    def __init__(self, data, om):
        self.om = om
        self.n = data.n_taxa
        self.seq = {v: np.asarray(s, np.uint8) for v, s in enumerate(data.seqs)}
        self.fitch = {v: data.fitch[v].copy() for v in range(self.n)}
        big = O.SANK_INF
        self.sank = {}
        for v in range(self.n):
            s = data.sank[v].astype(np.int64)
            s[s >= SANK_INF] = big
            self.sank[v] = s
        self.tcm = data.sank_tcm.astype(np.int64)
        self.nf = data.fitch.shape[1]
        self.ns = data.sank.shape[1]

    def median_levels(self, levels):
        return [self.medians(a, b, out) for a, b, out in levels]

    def medians(self, a, b, out):
        do, fi = [], []
        for x, y, v in zip(a, b, out):
            c, med, _, _, _ = O.dos_median(self.seq[int(x)], self.seq[int(y)], self.om)
            self.seq[int(v)] = med
            do.append(c)
            if self.nf:
                fc, fm = O.nonadd_median(self.fitch[int(x)], self.fitch[int(y)])
            else:
                fc, fm = 0, np.zeros(0, np.uint8)
            self.fitch[int(v)] = fm
            fi.append(fc)
            rows = []
            for ch in range(self.ns):
                c_, _, _ = O.sank_elt_median(self.tcm, self.sank[int(x)][ch], self.sank[int(y)][ch])
                rows.append(c_)
            self.sank[int(v)] = np.array(rows, np.int64).reshape(self.ns, -1) if self.ns else \
                np.zeros((0, self.tcm.shape[0]), np.int64)
        return np.array(do, np.int64), np.array(fi, np.int64)

    def distances(self, a, b):
        out = []
        for x, y in zip(a, b):
            s1, s2 = self.seq[int(x)], self.seq[int(y)]
            if np.all(s1 == 16) or np.all(s2 == 16):
                d = 0  # the join cost's missing distance
            else:
                d = O.cost_2(s1, s2, self.om, max(abs(len(s1) - len(s2)), 8))
            if self.nf:
                d += O.nonadd_distance(self.fitch[int(x)], self.fitch[int(y)])
            tot = 0.0
            for ch in range(self.ns):
                tot += O.sank_elt_distance(self.tcm, self.sank[int(x)][ch], self.sank[int(y)][ch])
            out.append(d + int(tot))
        return np.array(out, np.int64)

    def singles(self, parent, node, out):
        for p, v, o in zip(parent, node, out):
            self.seq[int(o)] = O.closest(self.seq[int(p)], self.seq[int(v)], self.om)

    def do_distances(self, a, b):
        out = []
        for x, y in zip(a, b):
            s1, s2 = self.seq[int(x)], self.seq[int(y)]
            if np.all(s1 == 16) or np.all(s2 == 16):
                out.append(0)   # missing distance
            else:
                out.append(O.cost_2(s1, s2, self.om, max(abs(len(s1) - len(s2)), 8)))
        return np.array(out, np.int64)

    def readjust(self, ch1, ch2, par, mine, out, mode="three"):
        ch, cs = [], []
        tab = O.median3_table(self.om) if mode == "three" else None
        for a, b, c, m_, o in zip(ch1, ch2, par, mine, out):
            changed, res, cost = O.dos_readjust(mode, self.seq[int(a)], self.seq[int(b)],
                                                self.seq[int(c)], self.seq[int(m_)], self.om, tab)
            self.seq[int(o)] = res
            ch.append(changed)
            cs.append(cost)
        return np.array(ch, bool), np.array(cs, np.int64)

    def sank_costs(self, vs):
        return np.array([self.sank_cost(v) for v in vs], np.int64)

    def sank_cost(self, v):
        if not self.ns:
            return 0
        return int(sum(int(min(r)) for r in self.sank[int(v)]))

    def node_seq(self, v):
        return self.seq[int(v)]

    def node_fitch(self, v):
        return self.fitch[int(v)]

    def node_sank(self, v):
        s = self.sank[int(v)].copy()
        s[s >= O.SANK_INF] = SANK_INF
        return s.astype(np.int32)

    def ensure_nodes(self, n_nodes):
        pass

    def rebind_nodes(self, dst, src):
        for v, t in zip(dst, src):
            self.seq[int(v)] = self.seq[int(t)]
            self.fitch[int(v)] = self.fitch[int(t)]
            self.sank[int(v)] = self.sank[int(t)]

    def release_nodes(self, first):
        for d in (self.seq, self.fitch, self.sank):
            for v in [v for v in d if v >= first]:
                del d[v]

    # final states of the non-DO characters (the search module's uppass)
    def final_slots(self, n_slots, fitch_base):
        self.fin = {}

    def final_root(self, node, slot):
        f = self.fitch[int(node)].copy() if self.nf else np.zeros(0, np.uint8)
        rows, bits = [], []
        for s in self.sank[int(node)]:
            mn = int(min(s))
            rows.append([O.SANK_INF if x >= O.SANK_INF else x - mn for x in s])
            bits.append(sum(1 << i for i, x in enumerate(s) if x == mn))
        self.fin[int(slot)] = (f, np.array(rows, np.int64).reshape(self.ns, -1),
                               np.array(bits, np.int64))

    def final_states(self, anc, node, left, right, out):
        for a, v, l, r, o in zip(anc, node, left, right, out):
            fa, ea, ba = self.fin[int(a)]
            f = O.nonadd_median_3(fa, self.fitch[int(v)], self.fitch[int(l)],
                                  self.fitch[int(r)]) if self.nf else np.zeros(0, np.uint8)
            rows, bits = [], []
            for ch in range(self.ns):
                e, bb = O.sank_elt_median_3(self.tcm, np.zeros(len(ea[ch]), np.int64), ea[ch],
                                            int(ba[ch]), self.sank[int(v)][ch],
                                            self.sank[int(l)][ch], self.sank[int(r)][ch])
                rows.append(e)
                bits.append(bb)
            self.fin[int(o)] = (f, np.array(rows, np.int64).reshape(self.ns, -1),
                                np.array(bits, np.int64))

    def node_final(self, slot):
        """(Fitch row, Sankoff e rows with infinity as simulate.SANK_INF,
        best-state bits) of a final slot, in the GPU backend's layout."""
        f, e, b = self.fin[int(slot)]
        e = e.copy()
        e[e >= O.SANK_INF] = SANK_INF
        return f, e.astype(np.int32), b.astype(np.int32)
