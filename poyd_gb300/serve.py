"""Continuous-batching request loop for align / median jobs.

Stands in for poyd's master/servant task stream (PoydMasterImpl.run_task,
poyd/PoydMasterImpl.ml:48-173; PoydParallel.do_parallel,
poyd/PoydParallel.ml:167-308), with the coarse per-search task farming
replaced by fine-grained pair jobs from many concurrent searches.  Sequences
of every client dataset stay resident in one device pool.  Jobs that arrive
while batches are running are admitted as soon as a stream slot is free and
the HBM budget (an estimate of each job's direction-matrix and output bytes)
allows; up to ``n_streams`` batches overlap on the device, each on its own
CUDA stream with its own workspace.  A job's result does not depend on the
batch it lands in: every pair is computed independently by the same kernels.
"""
from __future__ import annotations

import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np
import torch

from . import align


@dataclass
class Job:
    jid: int
    kind: str          # "cost" (cost_2, DOS.distance deltaw) or "median" (DOS.median)
    a: int             # sequence ids in the device pool
    b: int
    arrival: float = 0.0
    done: float = 0.0
    cost: int = 0
    median: np.ndarray = field(default=None)


def dm_bytes_estimate(la: int, lb: int) -> int:
    """Upper estimate of the linear DP's direction matrix for a pair: rows x
    (band + pipeline) / 2 bytes (4 bits per cell)."""
    l1, l2 = max(la, lb), min(la, lb)
    band = (l1 - l2) + 2 * (50 + int(0.05 * l1) + 8) + 100
    band = min(band, l1 + l2)
    return ((l1 + 63) // 64) * 64 * (band + 128) // 2 + 4 * (la + lb + 5)


class SequencePool:
    """Client sequences resident in HBM (one byte buffer + offsets)."""

    def __init__(self, seqs, device="cuda"):
        lens = np.array([len(s) for s in seqs], np.int64)
        self.off = np.zeros(len(seqs), np.int64)
        self.off[1:] = np.cumsum(lens)[:-1]
        self.len = lens.astype(np.int32)
        buf = np.concatenate([np.asarray(s, np.uint8) for s in seqs] + [np.zeros(64, np.uint8)])
        self.buf = torch.from_numpy(buf).to(device)

    def batch(self, a_ids, b_ids, device) -> align.PairBatch:
        t = lambda x, dt: torch.from_numpy(np.ascontiguousarray(x, dt)).to(device, non_blocking=True)
        return align.PairBatch(self.buf, t(self.off[a_ids], np.int64), t(self.len[a_ids], np.int32),
                               t(self.off[b_ids], np.int64), t(self.len[b_ids], np.int32))


class Server:
    def __init__(self, pool: SequencePool, cm: align.CostMatrix, budget_bytes: int = 120 << 30,
                 n_streams: int = 3, max_batch: int = 8192, device="cuda"):
        self.pool, self.cm, self.budget = pool, cm, budget_bytes
        self.dev = torch.device(device)
        self.streams = [torch.cuda.Stream(device=self.dev) for _ in range(n_streams)]
        self.busy = [None] * n_streams  # (jobs, event, result handles, bytes)
        self.pending: deque = deque()
        self.in_use = 0
        self.max_batch = max_batch
        self.completed = []
        self.batches = 0

    def submit(self, job: Job):
        self.pending.append(job)

    def _retire(self):
        for k, slot in enumerate(self.busy):
            if slot is None or not slot["event"].query():
                continue
            now = time.perf_counter()
            for kind, jobs, res in slot["parts"]:
                if kind == "cost":
                    cost = res.cpu().numpy()
                    for j, c in zip(jobs, cost):
                        j.cost, j.done = int(c), now
                else:
                    out = res.to_host()
                    for j, r in zip(jobs, out):
                        j.cost, j.median, j.done = r["cost"], r["median"], now
                self.completed.extend(jobs)
            self.in_use -= slot["bytes"]
            self.busy[k] = None

    def _admit(self):
        for k in range(len(self.busy)):
            if self.busy[k] is not None or not self.pending:
                continue
            take, nbytes = [], 0
            while self.pending and len(take) < self.max_batch:
                j = self.pending[0]
                need = dm_bytes_estimate(int(self.pool.len[j.a]), int(self.pool.len[j.b]))
                if self.in_use + nbytes + need > self.budget and take:
                    break
                take.append(self.pending.popleft())
                nbytes += need
            if not take:
                return
            st = self.streams[k]
            parts = []
            with torch.cuda.stream(st):
                for kind in ("cost", "median"):
                    jobs = [j for j in take if j.kind == kind]
                    if not jobs:
                        continue
                    b = self.pool.batch([j.a for j in jobs], [j.b for j in jobs], self.dev)
                    if kind == "cost":
                        res, _ = align.cost_2(b, self.cm, deltaw="dos", stream=st)
                    else:
                        res = align.align_2(b, self.cm, dos_empty=True, stream=st)
                    parts.append((kind, jobs, res))
                ev = torch.cuda.Event()
                ev.record(st)
            self.busy[k] = {"parts": parts, "event": ev, "bytes": nbytes}
            self.in_use += nbytes
            self.batches += 1

    def step(self):
        self._retire()
        self._admit()

    def idle(self) -> bool:
        return not self.pending and all(s is None for s in self.busy)

    def run(self, jobs, t0: float | None = None):
        """Replays jobs at their arrival offsets (seconds from start) in real
        time; returns the completed jobs."""
        jobs = sorted(jobs, key=lambda j: j.arrival)
        t0 = time.perf_counter() if t0 is None else t0
        i = 0
        while i < len(jobs) or not self.idle():
            now = time.perf_counter() - t0
            while i < len(jobs) and jobs[i].arrival <= now:
                jobs[i].arrival_abs = t0 + jobs[i].arrival
                self.submit(jobs[i])
                i += 1
            self.step()
            if self.idle() and i < len(jobs):
                time.sleep(max(0.0, min(0.001, jobs[i].arrival - (time.perf_counter() - t0))))
        return self.completed


def make_workload(seed: int, n_clients: int = 16, rate: float = 2000.0, seconds: float = 5.0,
                  taxa=(50, 500), lens=(200, 5000), median_frac: float = 0.3):
    """16 simulated searches: each a dataset of 50-500 related sequences with
    log-uniform lengths; a Poisson stream (mean `rate` req/s overall) of cost
    and median jobs over pairs of one client's sequences."""
    from . import synth
    rng = np.random.default_rng(seed)
    seqs, owner = [], []
    for c in range(n_clients):
        n = int(rng.integers(taxa[0], taxa[1] + 1))
        L = int(np.exp(rng.uniform(np.log(lens[0]), np.log(lens[1]))))
        root = synth.random_dna(rng, L)
        for _ in range(n):
            s = synth.mutate(rng, root, float(rng.uniform(0.02, 0.15)), float(rng.uniform(0.005, 0.03)))
            seqs.append(synth.with_gap(s))
            owner.append(c)
    owner = np.array(owner)
    by_client = [np.nonzero(owner == c)[0] for c in range(n_clients)]
    n_jobs = rng.poisson(rate * seconds)
    arrivals = np.sort(rng.uniform(0, seconds, size=n_jobs))
    jobs = []
    for i, t in enumerate(arrivals):
        c = int(rng.integers(n_clients))
        a, b = rng.choice(by_client[c], size=2, replace=False)
        kind = "median" if rng.random() < median_frac else "cost"
        jobs.append(Job(i, kind, int(a), int(b), float(t)))
    return seqs, jobs


def latency_stats(jobs):
    lat = np.array([j.done - j.arrival_abs for j in jobs]) * 1e3
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "n": int(len(lat))}
