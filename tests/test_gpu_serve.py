"""Serving loop: jobs arriving while batches run are admitted continuously
(several batches in flight on separate streams), every job completes, and
each job's result is identical to running it alone."""
import numpy as np
import pytest
import torch

from poyd_gb300 import align, serve

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("budget", [120 << 30, 2 << 20])
def test_results_identical_alone_and_in_mix(budget):
    seqs, jobs = serve.make_workload(3, n_clients=4, rate=600, seconds=1.0, taxa=(10, 30),
                                     lens=(200, 1500), median_frac=0.4)
    pool = serve.SequencePool(seqs)
    cm = align.CostMatrix.default()
    srv = serve.Server(pool, cm, budget_bytes=budget, n_streams=3, max_batch=64)
    done = srv.run(jobs)
    assert len(done) == len(jobs) and srv.idle()
    if budget >= (1 << 30):
        assert srv.batches < len(jobs)  # continuous batching merged arrivals
    st = serve.latency_stats(done)
    assert st["p99_ms"] >= st["p50_ms"] > 0
    dev = torch.device("cuda")
    for j in jobs:
        b = pool.batch([j.a], [j.b], dev)
        if j.kind == "cost":
            c, _ = align.cost_2(b, cm, deltaw="dos")
            assert int(c.item()) == j.cost, j.jid
        else:
            r = align.align_2(b, cm, dos_empty=True).to_host()[0]
            assert r["cost"] == j.cost and np.array_equal(r["median"], j.median), j.jid
