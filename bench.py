"""Benchmark: batched direct-optimization align_2 (DOS.median pieces) GCUPS.

Workload (one "step"): 65,536 independent DNA pairs, L1 ~ U[100, 5000], each
partner carrying 10-30 % substitutions and 2-5 % indels (geometric length,
mean 2), 5 % of positions IUPAC ambiguity masks; TCM substitution 1 / indel 2
(Cost_matrix.Two_D.default).  Per pair the step runs cost_2 (default deltaw,
the ``align_2`` path), backtrack_2d, ancestor_2 and median_2_with_gaps on the
device.  The unit is a DP cell the reference's band evaluates (counted per
pair by the plan kernel, mirroring algn.c:872-968); GCUPS = cells / s.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

``value`` is device throughput with inputs resident in HBM; ``e2e`` is the
same metric through the public API with pinned host buffers, the input
upload and the download of every result (packed: aligned pairs, medians
with gaps, medians, costs, lengths) inside the timed region.  N > 1 runs one
replica per GPU (the pairs are independent; no collective).  ``--impl
reference`` times the CPU restatement of the reference (oracle/) on all host
cores over a bounded sample of the same workload.

The default single-GPU run adds, on a bounded budget, the other
configurations as keys of the same line: ``affine`` (the same pairs under
gap opening 3: value, e2e, roofline, CPU baseline, parity),
``spr_joins_per_s`` (one SPR pass's candidate joins scored per second, 200
taxa x 1,500 bp + Fitch + Sankoff), ``learned_speedup`` (time to the plain
search's exact tree cost, plain / learned, 500 taxa x 1,000 bp) and
``serving`` (req_s, p50_ms, p99_ms of the Poisson request loop).
``--no-extras`` prints the headline alone; ``--workload`` runs one of them
on its own line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "align_2 GCUPS (bit-exact)"
UNIT = "GCUPS"
# Algorithmic integer ops per band cell: linear 3 adds + 2 mins + 3 direction
# compares; affine 24 for its four-state recurrence (algn.c:1740-1977).
OPS_PER_CELL = {"linear": 8, "affine": 24}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--pairs", type=int, default=65536)
    p.add_argument("--model", default="linear", choices=["linear", "affine"])
    p.add_argument("--seed", type=int, default=2026)
    p.add_argument("--cpu-sample-s", type=float, default=12.0)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-autotune", action="store_true",
                   help="launch the default variant instead of the autotuner's choice")
    p.add_argument("--no-extras", action="store_true",
                   help="headline only: skip the affine, SPR, learned, config0, readjust_3d and serving keys")
    p.add_argument("--workload", default="align",
                   choices=["align", "spr", "tbr", "learned", "serving", "kernels", "three",
                            "adjust", "config0"],
                   help="align (default, the headline line) or one of the other configs")
    p.add_argument("--train-trees", type=int, default=2)
    p.add_argument("--max-passes", type=int, default=8)
    p.add_argument("--serve-s", type=float, default=10.0)
    p.add_argument("--triples", type=int, default=1216,
                   help="three: node triples per step (readjust_3d)")
    p.add_argument("--tri-len", type=int, nargs=2, default=[100, 300],
                   help="three: ancestor length range of the triples")
    return p.parse_args()


def workload_config(args):
    return {
        "workload": "batched DNA align_2 + ancestor_2 + median_2_with_gaps (DOS.median)",
        "pairs": args.pairs, "len_range": [100, 5000], "sub": [0.10, 0.30],
        "indel": [0.02, 0.05], "ambiguity": 0.05,
        "tcm": "sub 1 / indel 2" + (" / gap_opening 3" if args.model == "affine" else ""),
        "model": args.model, "seed": args.seed,
        "l2_policy": "inputs larger than L2 (sequences ~330 MB, direction matrix tens of GB); no flush",
        "parallelism": "replicas" if args.gpus > 1 else "single",
    }


def cm_for(args, align_mod):
    if args.model == "affine":
        return align_mod.CostMatrix.dna(1, 2, 3)
    return align_mod.CostMatrix.default()


def oracle_cm(args, O):
    return O.cm_dna(1, 2, 3 if args.model == "affine" else -1)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def result_set(res):
    """Host copies of a batched align_2 result for the oracle's check (the
    arrays are kept alive by the returned tuple)."""
    import ctypes as C
    from oracle import oracle as O
    arrs = [np.ascontiguousarray(x.cpu().numpy() if hasattr(x, "cpu") else x)
            for x in (res.cost, res.out, res.out_off, res.out_len)]
    s = O.OrResultSet(*[a.ctypes.data for a in arrs])
    return s, arrs


def cpu_time_sample(host, idx, cm_o, threads, sets=()):
    """Runs the oracle's DOS.median on pairs idx over `threads` host threads;
    returns (seconds, band cells, per-set mismatch counts).  With `sets`
    (result_set tuples) every output of those batched results on the
    sampled pairs is compared with the oracle's in the same pass (a
    memcmp per pair, negligible beside the DP)."""
    import ctypes as C
    from oracle import oracle as O
    L = O.lib()
    seq, ao, al, bo, bl = host
    chunks = np.array_split(np.asarray(idx, np.int32), threads)
    cells = [0] * threads
    bads = [None] * threads
    arr = (O.OrResultSet * max(len(sets), 1))(*[s for s, _ in sets])

    def work(t):
        ch = np.ascontiguousarray(chunks[t])
        cost = np.zeros(len(ch), np.int32)
        if sets:
            bad = np.zeros(len(ch), np.int32)
            cells[t] = L.or_dos_median_check_many(
                seq.ctypes.data, ao.ctypes.data, al.ctypes.data, bo.ctypes.data,
                bl.ctypes.data, ch.ctypes.data, len(ch), cm_o, cost.ctypes.data, len(sets),
                C.cast(arr, C.c_void_p), bad.ctypes.data)
            bads[t] = bad
        else:
            cells[t] = L.or_dos_median_many(seq.ctypes.data, ao.ctypes.data, al.ctypes.data,
                                            bo.ctypes.data, bl.ctypes.data, ch.ctypes.data,
                                            len(ch), cm_o, cost.ctypes.data)

    ths = [threading.Thread(target=work, args=(t,)) for t in range(threads)]
    t0 = time.perf_counter()
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    dt = time.perf_counter() - t0
    if not sets:
        return dt, int(sum(cells))
    bad = np.concatenate(bads)
    return dt, int(sum(cells)), [int(((bad >> k) & 1).sum()) for k in range(len(sets))]


def cpu_sample_indices(host, budget_s, threads, cm_o, seed):
    """Picks a random sample of pairs whose CPU time is about budget_s."""
    rng = np.random.default_rng(seed)
    n = len(host[2])
    perm = rng.permutation(n).astype(np.int32)
    probe = perm[:max(threads * 2, 32)]
    dt, cells = cpu_time_sample(host, probe, cm_o, threads)
    per_pair = dt / len(probe)
    k = int(min(n, max(len(probe), budget_s / max(per_pair, 1e-9))))
    return perm[:k]


def run_reference(args):
    """CPU arm: the oracle's restatement of the reference on all host cores."""
    import ctypes as C
    from oracle import oracle as O
    from poyd_gb300 import synth
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    O.build()
    host = synth.pair_batch_fast(args.seed, args.pairs)
    cm_o = oracle_cm(args, O)
    threads = os.cpu_count() or 1
    per_step = max(1.0, args.cpu_sample_s / 2)
    idx = cpu_sample_indices(host, per_step, threads, C.byref(cm_o), args.seed)
    for _ in range(args.warmup):
        cpu_time_sample(host, idx[:max(threads, len(idx) // 8)], C.byref(cm_o), threads)
    tot_t, tot_c = 0.0, 0
    for s in range(args.steps):
        dt, cells = cpu_time_sample(host, idx, C.byref(cm_o), threads)
        tot_t += dt
        tot_c += cells
    v = tot_c / tot_t / 1e9
    sample = "%d of %d pairs per step (random, seeded), DOS.median pieces" % (len(idx), args.pairs)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": tot_t / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded)",
        "config": workload_config(args),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def aggregate(cells: int, seconds: float, dev, world: int):
    """Replica aggregation: (sum of band cells over ranks, max step time over
    ranks).  Each rank runs its own independent pairs; no data-path
    collective, only these two reductions of the timing."""
    import torch
    import torch.distributed as dist
    c = torch.tensor([float(cells)], dtype=torch.float64, device=dev)
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=dev)
    if world > 1:
        dist.all_reduce(c, op=dist.ReduceOp.SUM)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(c.item()), float(t.item())


def run_ours(args):
    import torch
    import torch.distributed as dist
    from poyd_gb300 import align, synth

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    host = synth.pair_batch_fast(args.seed + rank, args.pairs)
    pinned = [torch.from_numpy(x).pin_memory() for x in host]
    batch = align.PairBatch.from_packed(pinned, device=dev)
    env = {"world": world, "rank": rank, "local": local, "dev": dev, "host": host,
           "pinned": pinned, "batch": batch}
    line = measure_align(args, env)
    failed = bool(line and line.get("parity", {}).get("mismatches"))
    if rank == 0 and world == 1 and args.workload == "align" and not args.no_extras:
        # The other configurations, on a bounded budget, as keys of the same
        # line: the affine variant of the same pairs, one SPR pass's
        # candidate scoring, the learned vs plain search, the Iterative
        # (ThreeD) node readjustments and the serving loop.
        extras = argparse.Namespace(**vars(args))
        extras.cpu_sample_s = min(args.cpu_sample_s, 6.0)
        extras.serve_s = min(args.serve_s, 8.0)
        if args.model == "linear":
            extras.model = "affine"
            aff = _guard(lambda: measure_align(extras, env))
            keep = ("value", "unit", "ms_per_step", "e2e", "roofline", "cpu_baseline", "parity",
                    "gpu_launches", "clocks", "kernel_ms_per_step", "autotune")
            line["affine"] = {k: aff[k] for k in keep if k in aff} if "error" not in aff else aff
            line["affine"]["config"] = {"tcm": "sub 1 / indel 2 / gap_opening 3",
                                        "pairs": args.pairs, "same_pairs_as_headline": True}
            failed |= bool(line["affine"].get("parity", {}).get("mismatches"))
            extras.model = "linear"
        spr = _guard(lambda: run_spr(extras))
        line["spr_joins_per_s"] = spr.get("value")
        line["spr"] = spr
        failed |= spr.get("cpu_baseline", {}).get("bit_exact_on_sample") is False
        lrn = _guard(lambda: run_learned(extras))
        # a speedup counts only where the learned search reached the plain
        # search's exact cost
        line["learned_speedup"] = lrn.get("speedup") if lrn.get("reached_same_cost") else None
        line["learned"] = lrn
        c0 = _guard(lambda: run_config0(extras))
        line["config0_s"] = c0.get("value")
        line["config0"] = c0
        failed |= c0.get("parity", {}).get("identical_tree_costs_and_medians") is False
        tri = argparse.Namespace(**vars(extras))
        tri.steps, tri.warmup = min(args.steps, 5), 1
        line["readjust_3d"] = _guard(lambda: run_three(tri))
        failed |= bool(line["readjust_3d"].get("parity", {}).get("mismatches"))
        srv = _guard(lambda: run_serving(extras))
        line["serving"] = {"req_s": srv.get("value"), "p50_ms": srv.get("p50_ms"),
                           "p99_ms": srv.get("p99_ms"), **srv}
        failed |= srv.get("sample_identical_alone") is False
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    if failed:
        sys.stderr.write("bench: a result differs from the oracle or the one-at-a-time run\n")
        sys.exit(1)


def _guard(fn):
    """Runs one extra workload; an exception is reported in its key rather
    than losing the headline line."""
    try:
        return fn()
    except Exception as ex:  # noqa: BLE001 -- reported, not hidden
        return {"error": "%s: %s" % (type(ex).__name__, str(ex)[:300])}


def measure_align(args, env):
    """The batched align_2 measurement (``args.model``) on the pairs of
    `env`: device-resident value, the host-buffer e2e run, the roofline,
    the oracle's CPU time on a sample and the parity of both runs' results
    on that sample.  Returns the line (rank 0) or None."""
    import torch
    import torch.distributed as dist
    from poyd_gb300 import align, native
    world, rank, local, dev = env["world"], env["rank"], env["local"], env["dev"]
    host, pinned, batch = env["host"], env["pinned"], env["batch"]
    cm = cm_for(args, align)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    # autotuner (untimed): the launch variant for this batch's shape class,
    # every variant checked to give the same results
    tuned = None
    if args.model == "linear" and not args.no_autotune:
        tuned = align.autotune(batch, cm, align=True, reps=1)
    # warm-up (also sizes the workspace)
    res = None
    for _ in range(args.warmup):
        res = align.align_2(batch, cm, band_cells=True)
    torch.cuda.synchronize()
    cells = int(res.band_cells.sum().item())
    full_cells = int((batch.a_len.to(torch.int64) * batch.b_len.to(torch.int64)).sum().item())

    # ---- device-resident timed region ----
    native.lib().poyd_profile_enable(1)
    native.profile_read(clear=True)
    launches0 = native.lib().poyd_launch_count()
    barrier()
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(st)
        for _ in range(args.steps):
            res = align.align_2(batch, cm)
        e1.record(st)
        barrier()
    ms = e0.elapsed_time(e1) / args.steps
    launches = native.lib().poyd_launch_count() - launches0
    kname = "lin_dp_dm" if args.model == "linear" else "aff_dp_dm"
    dp_ms, dp_n = native.profile_read(kname, clear=False)
    all_ms, all_n = native.profile_read(None, clear=True)
    native.lib().poyd_profile_enable(0)
    total_cells, ms_max = aggregate(cells, ms, dev, world)
    value = total_cells / (ms_max * 1e-3) / 1e9

    # ---- end-to-end through the public API with host buffers ----
    e2e = None
    res_e2e = None
    if not args.no_e2e:
        # sequences plus, per pair, offsets and lengths (a, b) and the slot
        # offset
        h2d = int(pinned[0].numel()) + 32 * int(pinned[2].numel())

        # one public call per step: poyd_align_2_host uploads the pinned
        # host arrays, runs the batch and downloads every result slot (laid
        # out in the DP's finishing order, so the download runs while the
        # DP does) plus the costs and lengths
        out_host = align.host_outputs(pinned)  # untimed: pinned result buffers

        def e2e_step():
            r = align.align_2_host(pinned, cm, out=out_host)
            e2e_step.d2h = r.cost.numel() * 4 + int(4 * r.cap.sum()) + r.out_len.numel() * 4
            return r

        e2e_step()
        barrier()
        t0 = time.perf_counter()
        n_e2e = max(1, args.steps // 2)
        for _ in range(n_e2e):
            res_e2e = e2e_step()
        dt = (time.perf_counter() - t0) / n_e2e
        d2h = int(e2e_step.d2h)
        _, dt_max = aggregate(cells, dt, dev, world)
        e2e = {"value": total_cells / dt_max / 1e9, "unit": UNIT,
               "api": "poyd_align_2_host (download overlapping the DP)",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}

    if rank != 0:
        return None
    peak_gops = native.int32_peak()
    dp_launch_ms = dp_ms / max(dp_n, 1)
    achieved = cells / (dp_launch_ms * 1e-3) * OPS_PER_CELL[args.model] / 1e9
    traffic = None
    prof = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(prof):
        try:
            traffic = json.load(open(prof)).get(kname)
        except Exception:
            traffic = None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "int32", "data": "synthetic (seeded generator, poyd_gb300/synth.py)",
        "config": dict(workload_config(args), band_cells_per_step=cells,
                       full_matrix_cells_per_step=full_cells),
        "gpu_launches": int(launches),
        "kernel_ms_per_step": {"dp": dp_ms / args.steps, "all": all_ms / args.steps},
        "roofline": {"bound": "int32", "achieved": achieved, "peak": peak_gops,
                     "unit": "Gop/s", "frac": achieved / peak_gops if peak_gops else None,
                     "traffic": traffic, "kernel": kname,
                     "ops_per_cell": OPS_PER_CELL[args.model],
                     "peak_source": "measured (poyd_int32_peak: fused add-min on the ALU "
                                    "pipe interleaved with multiply-add adds on the FMA pipe)",
                     "peak_alu_pipe_only": native.int_pipe_rate(0)},
        "clocks": clk.summary(),
        "e2e": e2e,
    }
    if tuned is not None:
        line["autotune"] = tuned
    # CPU baseline: the oracle port on a bounded sample, all host threads
    try:
        import ctypes as C
        from oracle import oracle as O
        O.build()
        cm_o = oracle_cm(args, O)
        threads = os.cpu_count() or 1
        idx = cpu_sample_indices(host, args.cpu_sample_s, threads, C.byref(cm_o), args.seed)
        # the last timed step's results (device-resident run and, when
        # measured, the host-buffer run) are checked against the oracle on
        # every sampled pair while the oracle is timed
        names = ["value"] + (["e2e"] if res_e2e is not None else [])
        sets = [result_set(res)] + ([result_set(res_e2e)] if res_e2e is not None else [])
        dt, c, bad = cpu_time_sample(host, idx, C.byref(cm_o), threads, sets)
        line["cpu_baseline"] = {
            "value": c / dt / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d of %d pairs (random, seeded), %.1f s" % (len(idx), args.pairs, dt)}
        fields = (["cost", "aligned a", "aligned b", "median_2_with_gaps", "ancestor_2 median"]
                  if args.model == "linear" else
                  ["cost", "aligned a", "aligned b", "median with gaps", "median"])
        line["parity"] = {
            "checked": int(len(idx)), "mismatches": int(sum(bad)),
            "by_run": dict(zip(names, bad)), "fields": fields,
            "against": "oracle (C restatement of algn.c / sequence.ml, pinned against "
                       "the compiled reference)"}
    except Exception as ex:  # the baseline must not hide the GPU line
        line["cpu_baseline"] = {"value": None, "error": str(ex)[:200]}
    if line.get("parity", {}).get("mismatches"):
        sys.stderr.write("bench: %d of %d sampled %s pairs differ from the oracle\n"
                         % (line["parity"]["mismatches"], line["parity"]["checked"], args.model))
    return line


def _emit(line):
    print(json.dumps(line))


def _snapshot(be):
    """Host copies of a GpuBackend's node data, in the oracle's layout."""
    from oracle import oracle as O
    seqs = [be.node_seq(v) for v in range(len(be.len))]
    lens = np.array([len(s) for s in seqs], np.int32)
    off = np.zeros(len(seqs), np.int64)
    off[1:] = np.cumsum(lens.astype(np.int64))[:-1]
    buf = np.concatenate(seqs + [np.zeros(64, np.uint8)])
    fitch = np.ascontiguousarray(be.fitch[:, :be.nf].cpu().numpy()) if be.nf else np.zeros(1, np.uint8)
    sank = be.sank[:, :be.ns].cpu().numpy().astype(np.int64)
    sank[sank >= (1 << 30)] = O.SANK_INF
    return buf, off, lens, fitch, np.ascontiguousarray(sank)


def cpu_candidate_rate(be, S, E, budget_s, threads):
    """Candidates/s of the oracle's C scoring on all host threads (sample)."""
    import ctypes as C
    from oracle import oracle as O
    L = O.lib()
    buf, off, lens, fitch, sank = _snapshot(be)
    tcm = np.ascontiguousarray(be.tcm.cpu().numpy().astype(np.int64))
    om = O.cm_dna(1, 2, -1)
    rng = np.random.default_rng(0)

    def run(idx):
        chunks = np.array_split(idx, threads)
        outs = [np.zeros(len(c), np.int64) for c in chunks]

        def work(i):
            a = np.ascontiguousarray(S[chunks[i]], np.int32)
            b = np.ascontiguousarray(E[chunks[i]], np.int32)
            L.or_candidate_scores(buf.ctypes.data, off.ctypes.data, lens.ctypes.data, fitch.ctypes.data,
                                  be.nf, sank.ctypes.data, be.ns, be.k, tcm.ctypes.data, a.ctypes.data,
                                  b.ctypes.data, len(a), C.byref(om), outs[i].ctypes.data)
        ths = [threading.Thread(target=work, args=(i,)) for i in range(threads)]
        t0 = time.perf_counter()
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        return time.perf_counter() - t0, np.concatenate(outs)

    probe = rng.choice(len(S), size=min(len(S), threads * 4), replace=False)
    dt, _ = run(probe)
    k = int(min(len(S), max(len(probe), budget_s / max(dt / len(probe), 1e-9))))
    idx = rng.choice(len(S), size=k, replace=False)
    dt, out = run(idx)
    return k / dt, k, idx, out


def run_spr(args):
    """Config 2: one SPR pass, 200 taxa x ~1,500 bp + 2,000 Fitch (2-8 states)
    + 200 Sankoff (4 states); every candidate join scored in one batch."""
    import torch
    from poyd_gb300 import align, learned, native, search, simulate
    data = simulate.simulate(args.seed, 200, 1500, n_fitch=2000, n_sank=200)
    be = search.GpuBackend(data, align.CostMatrix.default())
    # a random start, not the generating tree (which the same seed would draw)
    t = learned.random_tree(data.n_taxa, args.seed + 7)
    search.downpass(t, be)
    S, E = search.spr_candidates(t)
    for _ in range(2):  # warm-up
        be.distances(S[:4096], E[:4096])
    native.lib().poyd_profile_enable(1)
    native.profile_read(clear=True)
    be.stats["do_cells"] = 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    score = be.distances(S, E)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    k = {}
    for name in ("lin_dp_cost", "lin_plan", "fitch_distance", "sank_distance"):
        k[name] = native.profile_read(name, clear=False)[0]
    native.profile_read(clear=True)
    native.lib().poyd_profile_enable(0)
    threads = os.cpu_count() or 1
    rate, k_cpu, idx, out = cpu_candidate_rate(be, S, E, args.cpu_sample_s, threads)
    st = search.spr_pass(t, be, max_moves=16)
    n = len(S)
    fitch_bytes = 2.0 * n * be.nf
    sank_bytes = 2.0 * n * be.ns * be.k * 4
    peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))).get("hbm_gbs") \
        if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else 6774.9
    line = {
        "workload": "config 2: SPR pass, 200 taxa x 1500 bp + 2000 Fitch + 200 Sankoff",
        "metric": "candidate joins scored per second", "value": n / dt, "unit": "joins/s",
        "candidates": n, "seconds_scoring": dt,
        "kernel_ms": k,
        "do_gcups_cost_only": be.stats["do_cells"] / 1e9 / (k["lin_dp_cost"] * 1e-3)
        if k["lin_dp_cost"] else None,
        "fitch_gbs": fitch_bytes / (k["fitch_distance"] * 1e-3) / 1e9 if k["fitch_distance"] else None,
        "sank_gbs": sank_bytes / (k["sank_distance"] * 1e-3) / 1e9 if k["sank_distance"] else None,
        "hbm_peak_gbs": peak,
        "pass": {"moves_tried": st.moves_tried, "moves_accepted": st.moves_accepted,
                 "cost_before": st.cost_before, "cost_after": st.cost_after,
                 "seconds": st.seconds_total},
    }
    line["cpu_baseline"] = {"value": rate, "unit": "joins/s", "cores": threads, "kind": "port",
                            "sample": "%d of %d candidates" % (k_cpu, n),
                            "bit_exact_on_sample": bool(np.array_equal(out, score[idx]))}
    return line


def run_tbr(args):
    """TBR pass on the config-2 data (200 taxa x ~1,500 bp + 2,000 Fitch +
    200 Sankoff): every (clade, re-rooting, join edge) candidate scored in
    one batch, the re-rootings' medians included."""
    import torch
    from poyd_gb300 import align, learned, search, simulate
    data = simulate.simulate(args.seed, 200, 1500, n_fitch=2000, n_sank=200)
    be = search.GpuBackend(data, align.CostMatrix.default())
    # a random start, not the generating tree (which the same seed would draw)
    t = learned.random_tree(data.n_taxa, args.seed + 7)
    diag = search.downpass(t, be)
    search.tbr_candidates(t, be, diag)  # warm-up (buffer growth)
    be.stats["median_pairs"] = be.stats["distance_pairs"] = 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    S, U, E, score, _ = search.tbr_candidates(t, be, diag)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    medians = be.stats["median_pairs"]
    st = search.tbr_pass(t, be, max_moves=16, diag=diag)
    return ({
        "workload": "TBR pass, 200 taxa x 1500 bp + 2000 Fitch + 200 Sankoff",
        "metric": "TBR candidate joins scored per second", "value": len(S) / dt,
        "unit": "joins/s", "candidates": int(len(S)),
        "rerooted": int((U >= 0).sum()), "clades": int(len(np.unique(S))),
        "reroot_medians": int(medians), "seconds_scoring": dt,
        "pass": {"moves_tried": st.moves_tried, "moves_accepted": st.moves_accepted,
                 "cost_before": st.cost_before, "cost_after": st.cost_after,
                 "seconds": st.seconds_total},
    })


def run_learned(args):
    """Config 3: learned proposal vs plain exhaustive SPR, time to the same
    exact tree cost (500 taxa x ~1,000 bp)."""
    import torch
    from poyd_gb300 import align, learned, search, simulate
    data = simulate.simulate(args.seed, 500, 1000, n_fitch=400, n_sank=40)
    be = search.GpuBackend(data, align.CostMatrix.default())
    Xs, ys = [], []
    t0 = time.perf_counter()
    for s in range(args.train_trees):
        t = learned.random_tree(data.n_taxa, 1000 + s)
        search.downpass(t, be)
        X, y = learned.log_pass(t, be)
        Xs.append(X)
        ys.append(y)
    X, y = torch.cat(Xs), torch.cat(ys)
    t_log = time.perf_counter() - t0
    prop = learned.Proposal(seed=0)
    t0 = time.perf_counter()
    prop.fit(X, y, epochs=4, batch=4096, lr=1e-3)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    tp = learned.random_tree(data.n_taxa, args.seed + 7)
    times_p = []
    hist_p, sec_all_p = learned.run_search(tp, be, None, max_passes=args.max_passes,
                                           times=times_p)
    target = hist_p[-1]
    # time to first reach the final cost (the converged search's last pass,
    # which finds no move, only confirms it)
    sec_p = times_p[hist_p.index(target)]
    tl = learned.random_tree(data.n_taxa, args.seed + 7)
    stats = {}
    sc = learned.learned_scorer(prop, be, frac=0.03, stats=stats)
    t0 = time.perf_counter()
    hist_l = []
    diag = None
    for _ in range(3 * args.max_passes):
        st = search.spr_pass(tl, be, max_moves=16, scorer=sc, diag=diag)
        diag = st.diag
        hist_l.append(st.cost_after)
        if st.cost_after <= target:
            break
        if st.moves_accepted == 0:
            st = search.spr_pass(tl, be, max_moves=16, diag=diag)  # exhaustive fallback
            diag = st.diag
            hist_l.append(st.cost_after)
            if st.moves_accepted == 0 or st.cost_after <= target:
                break
    torch.cuda.synchronize()
    sec_l = time.perf_counter() - t0
    return ({
        "workload": "config 3: learned join proposal vs plain exhaustive SPR, 500 taxa x 1000 bp",
        "metric": "SPR time to equal tree cost, learned vs plain GPU",
        "plain_seconds": sec_p, "plain_seconds_with_confirming_pass": sec_all_p,
        "plain_cost": target, "plain_passes": len(hist_p),
        "learned_seconds": sec_l, "learned_cost": hist_l[-1], "learned_passes": len(hist_l),
        "speedup": sec_p / sec_l if sec_l else None,
        "reached_same_cost": hist_l[-1] <= target,
        "training_pairs": int(X.shape[0]), "log_seconds": t_log, "train_seconds": t_train,
        "exact_evaluated_fraction": stats.get("exact", 0) / max(stats.get("candidates", 1), 1),
    })


def run_serving(args):
    """Config 4: Poisson stream (2,000 req/s) from 16 simulated searches."""
    import torch
    from poyd_gb300 import align, serve
    seqs, jobs = serve.make_workload(args.seed, n_clients=16, rate=2000.0, seconds=args.serve_s)
    pool = serve.SequencePool(seqs)
    cm = align.CostMatrix.default()
    warm = serve.Server(pool, cm, n_streams=3)
    warm.run([serve.Job(-1 - i, j.kind, j.a, j.b, 0.0) for i, j in enumerate(jobs[:256])])
    srv = serve.Server(pool, cm, budget_bytes=120 << 30, n_streams=3)
    t0 = time.perf_counter()
    done = srv.run(jobs)
    wall = time.perf_counter() - t0
    st = serve.latency_stats(done)
    rng = np.random.default_rng(1)
    ok = True
    for j in rng.choice(done, size=min(64, len(done)), replace=False):
        b = pool.batch([j.a], [j.b], torch.device("cuda"))
        if j.kind == "cost":
            ok &= int(align.cost_2(b, cm, deltaw="dos")[0].item()) == j.cost
        else:
            r = align.align_2(b, cm, dos_empty=True).to_host()[0]
            ok &= r["cost"] == j.cost and np.array_equal(r["median"], j.median)
    return ({"workload": "config 4: serving loop, 16 searches, Poisson 2000 req/s, 120 GB budget",
           "metric": "served requests/s", "value": len(done) / wall, "unit": "req/s",
           "offered_rate": 2000.0, "seconds": wall, "batches": srv.batches,
           "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "mean_ms": st["mean_ms"],
           "jobs": st["n"], "sample_identical_alone": bool(ok)})


def run_three(args):
    """Iterative (ThreeD) mode: ``Sequence.Align.readjust_3d`` for a batch of
    node triples (two children, the current median, the parent) descended
    from seeded ancestors of --tri-len bp with 5-20 % substitutions and
    1-4 % indels per sequence, DNA sub 1 / indel 2 (Powell's mm 1, go 0,
    ge 2).  A step is one batched readjust of every triple.  Device-resident
    value (triples/s, cube cells/s), the end-to-end run from pinned host
    buffers (uploads, the call, the download of every result), parity with
    the oracle on the smallest triples and the oracle's CPU rate on a
    sample."""
    import torch
    from oracle import oracle as O
    from poyd_gb300 import align, native, synth, three
    torch.cuda.set_device(0)
    # the choice cubes want free memory: drop what earlier workloads cached
    torch.cuda.empty_cache()
    native.check(native.lib().poyd_workspace_release())
    T = synth.triple_batch(args.seed, args.triples, args.tri_len[0], args.tri_len[1])
    items = [(a, b, a.copy(), p) for a, b, p in T]  # current median: the first child
    cm = align.CostMatrix.dna(1, 2)
    seq, offs, lens = three.TripleBatch.pack_host(items)
    host = [torch.from_numpy(x).pin_memory() for x in [seq] + offs + lens]
    batch = three.TripleBatch(host[0].cuda(), [x.cuda() for x in host[1:5]],
                              [x.cuda() for x in host[5:9]])
    cells = float(sum(len(a) * len(b) * len(p) for a, b, _, p in items))
    native.lib().poyd_profile_enable(1)
    native.profile_read(clear=True)
    for _ in range(max(args.warmup, 1)):
        r = three.readjust_3d(batch, cm)
    torch.cuda.synchronize()
    native.profile_read(clear=True)
    launches0 = native.lib().poyd_launch_count()
    steps = max(args.steps, 1)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        r = three.readjust_3d(batch, cm)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    kern_ms = native.profile_read("p3", clear=True)[0] / steps
    launches = (native.lib().poyd_launch_count() - launches0) / steps
    # end to end: pinned host inputs -> device, readjust, every result back
    e2e_ms, h2d, d2h = [], 0, 0
    for _ in range(steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dev = [x.to("cuda", non_blocking=True) for x in host]
        b2 = three.TripleBatch(dev[0], dev[1:5], dev[5:9])
        r2 = three.readjust_3d(b2, cm)
        outs = [r2.out.to("cpu"), r2.out_len.to("cpu"), r2.cost.to("cpu"), r2.changed.to("cpu")]
        torch.cuda.synchronize()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
        h2d = sum(x.numel() * x.element_size() for x in host)
        d2h = sum(x.numel() * x.element_size() for x in outs)
    e2e = float(np.median(e2e_ms))
    # parity: the smallest triples against the oracle (cost, median, changed)
    res = r.to_host()
    order = np.argsort([len(a) * len(b) * len(p) for a, b, _, p in items])[:6]
    m = O.cm_dna(1, 2, -1)
    tab = O.median3_table(m)
    bad = 0
    for i in order:
        c, med, ch = O.readjust_3d(*items[i], m, tab)
        bad += (c, ch) != (res[i]["cost"], res[i]["changed"]) or not np.array_equal(med, res[i]["median"])
    # the oracle's rate on a sample of median-sized triples, all host threads
    threads = os.cpu_count() or 1
    mid = np.argsort([len(a) * len(b) * len(p) for a, b, _, p in items])
    pick = mid[len(mid) // 2 - threads // 2:len(mid) // 2 - threads // 2 + threads]

    def work(i):
        O.readjust_3d(*items[i], m, tab)
    ths = [threading.Thread(target=work, args=(int(i),)) for i in pick]
    t0 = time.perf_counter()
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    cdt = time.perf_counter() - t0
    ccells = float(sum(len(items[i][0]) * len(items[i][1]) * len(items[i][3]) for i in pick))
    pairs_per_cell = 256  # (previous, next) state pairs: one fused add-min each
    peak = native.int32_peak()
    del r, r2, outs, batch
    native.check(native.lib().poyd_workspace_release())  # the choice cubes: tens of GB
    return {
        "workload": "Iterative (ThreeD) readjust_3d: %d node triples, ancestors %d-%d bp, "
                    "DNA sub 1 / indel 2" % (args.triples, args.tri_len[0], args.tri_len[1]),
        "metric": "node readjustments per second", "value": args.triples / (ms * 1e-3),
        "unit": "triples/s", "ms_per_step": ms, "steps": steps, "warmup": args.warmup,
        "cube_cells_per_step": cells, "gcells_s": cells / (ms * 1e-3) / 1e9,
        "kernel_ms_per_step": kern_ms, "gpu_launches": launches, "dtype": "int32",
        "data": "synthetic (seeded)",
        "roofline": {"bound": "int32", "achieved": cells * pairs_per_cell * 2 / (kern_ms * 1e-3) / 1e12
                     if kern_ms else None, "peak": peak / 1e3, "unit": "Tops/s",
                     "frac": cells * pairs_per_cell * 2 / (kern_ms * 1e-3) / 1e9 / peak
                     if kern_ms else None,
                     "ops_per_cell": "256 add-min (2 ops each) of 16 x 16 state pairs"},
        "e2e": {"value": args.triples / (e2e * 1e-3), "unit": "triples/s", "ms_per_step": e2e,
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "parity": {"checked": len(order), "mismatches": int(bad), "against": "oracle (or_readjust_3d)"},
        "cpu_baseline": {"value": len(pick) / cdt, "unit": "triples/s", "cores": len(pick),
                         "kind": "port", "gcells_s": ccells / cdt / 1e9,
                         "sample": "%d median-sized triples of the batch, one per thread" % len(pick)},
    }


def run_config0(args):
    """Config 0: a Wagner build plus one SPR pass on 20 taxa x ~300 bp
    (seeded Yule tree, JC 0.05 per site per branch, indels 0.01 per site;
    DNA sub 1 / indel 2), wall time of the whole search on the GPU backend
    and on the oracle backend (the CPU restatement, one core), and parity:
    the same tree, the same costs and every per-node median."""
    import torch
    from oracle import oracle as O
    from poyd_gb300 import align, search, simulate
    from tests.oracle_backend import OracleBackend  # the CPU leg only
    torch.cuda.set_device(0)
    data = simulate.simulate(args.seed, 20, 300)

    def run(be):
        t0 = time.perf_counter()
        t, d = search.wagner(data.n_taxa, be)
        st = search.spr_pass(t, be, max_moves=16)
        if hasattr(be, "pool"):
            torch.cuda.synchronize()
        return time.perf_counter() - t0, t, d, st

    run(search.GpuBackend(data, align.CostMatrix.default()))  # warm-up
    g = search.GpuBackend(data, align.CostMatrix.default())
    gdt, tg, dg, sg = run(g)
    o = OracleBackend(data, O.cm_dna(1, 2, -1))
    odt, to, do, so = run(o)
    same = tg.newick() == to.newick() and (dg.total, sg.cost_after) == (do.total, so.cost_after) \
        and all(np.array_equal(g.node_seq(v), o.node_seq(v)) for v in tg.nodes())
    return {"workload": "config 0: Wagner build + one SPR pass, 20 taxa x ~300 bp",
            "metric": "seconds per search", "value": gdt, "unit": "s", "higher_is_better": False,
            "data": "synthetic (seeded)", "wagner_cost": int(dg.total),
            "spr": {"cost_before": sg.cost_before, "cost_after": sg.cost_after,
                    "moves_accepted": sg.moves_accepted},
            "parity": {"identical_tree_costs_and_medians": bool(same)},
            "cpu_baseline": {"value": odt, "unit": "s", "cores": 1, "kind": "port",
                             "sample": "the same search on the oracle backend"}}


def run_adjust(args):
    """Iterative cost modes end to end: ``AllDirChar.adjust_tree`` after the
    default diagnosis of a seeded random tree (100 taxa x 500 bp, JC 0.1 per
    site per branch, indels 0.02; DNA sub 1 / indel 2), ThreeD and ApproxD,
    on the GPU backend; the same driver over the CPU oracle on a 20-taxon x
    120 bp tree gives the CPU time and the parity check."""
    import torch
    from oracle import oracle as O
    from poyd_gb300 import align, learned, search, simulate
    from tests.oracle_backend import OracleBackend  # the CPU leg only
    torch.cuda.set_device(0)
    out = {"workload": "Iterative modes: adjust_tree, 100 taxa x 500 bp (GPU), 20 x 120 (parity)",
           "metric": "seconds per adjustment", "unit": "s", "higher_is_better": False,
           "data": "synthetic (seeded)", "modes": {}}
    big = simulate.simulate(3, 100, 500, 0, 0, sub_per_branch=0.1, indel_rate=0.02)
    small = simulate.simulate(4, 20, 120, 0, 0, sub_per_branch=0.1, indel_rate=0.02)
    tb, ts = learned.random_tree(100, 9), learned.random_tree(20, 9)
    for mode in ("three", "approx"):
        be = search.GpuBackend(big, align.CostMatrix.default())
        search.adjust_tree(tb, be, mode, max_count=1)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = search.adjust_tree(tb, be, mode)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        t1 = time.perf_counter()
        g = search.adjust_tree(ts, search.GpuBackend(small, align.CostMatrix.default()), mode)
        torch.cuda.synchronize()
        gdt = time.perf_counter() - t1
        t1 = time.perf_counter()
        o = search.adjust_tree(ts, OracleBackend(small, O.cm_dna(1, 2, -1)), mode)
        cdt = time.perf_counter() - t1
        same = (g.cost, g.passes, g.changes) == (o.cost, o.passes, o.changes) and \
            all(np.array_equal(g.seqs[v], o.seqs[v]) for v in o.seqs)
        out["modes"][mode] = {
            "seconds": dt, "cost_before": r.initial_cost, "cost_after": r.cost,
            "passes": r.passes, "changes": r.changes, "batched_calls": r.calls,
            "parity_20_taxa": {"identical": bool(same), "cost": g.cost, "gpu_seconds": gdt},
            "cpu_baseline_20_taxa": {"seconds": cdt, "cores": 1, "kind": "port"}}
    out["value"] = out["modes"]["three"]["seconds"]
    return out


def run_kernels(args):
    """The other kernels on their own: Fitch and Sankoff distance / median
    over node arrays larger than L2 (HBM-bound: achieved GB/s of the bytes
    each launch must move, against the measured copy bandwidth), closest
    on config-1 pairs, and the MLP's BF16 GEMMs (against the measured
    cuBLAS bf16 rate).  Inputs are seeded random state sets and costs; CUDA
    events, 3 warm-up launches, the mean of `--steps` launches."""
    import ctypes as C
    import torch
    from poyd_gb300 import align, learned, native, synth
    dev = torch.device("cuda")
    L = native.lib()
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    P = lambda t: C.c_void_p(t.data_ptr())
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) \
        if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    hbm = peaks.get("hbm_gbs", 6800.0)
    bf16 = peaks.get("bf16_tflops", 1900.0)
    g = torch.Generator(device="cpu").manual_seed(args.seed)
    steps = max(args.steps, 1)

    def timed(fn):
        for _ in range(3):
            native.check(fn())
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            native.check(fn())
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    def hbm_line(ms, nbytes, **kw):
        gbs = nbytes / (ms * 1e-3) / 1e9
        return dict(kw, ms=ms, bytes_per_launch=int(nbytes), gb_s=gbs, peak_gb_s=hbm,
                    frac=gbs / hbm)

    out = {}
    # Fitch: 262,144 nodes x 2,048 characters (512 MiB of rows)
    NN, NF, n = 1 << 18, 2048, 1 << 20
    fitch = torch.randint(1, 256, (NN, NF), dtype=torch.uint8, generator=g).to(dev)
    ia = torch.randint(0, NN, (n,), dtype=torch.int32, generator=g).to(dev)
    ib = torch.randint(0, NN, (n,), dtype=torch.int32, generator=g).to(dev)
    dist = torch.empty(n, dtype=torch.int64, device=dev)
    ms = timed(lambda: L.poyd_nonadd8_distance_batch(P(fitch), C.c_int64(NF), NF, n, P(ia),
                                                     P(ib), P(dist), st))
    out["fitch_distance"] = hbm_line(ms, n * (2 * NF + 8), kernel="k_fitch_distance", pairs=n,
                                     row_bytes=NF, node_array_mib=NN * NF >> 20)
    nm = 1 << 18
    res = torch.empty((nm, NF), dtype=torch.uint8, device=dev)
    added = torch.empty(nm, dtype=torch.int64, device=dev)
    ms = timed(lambda: L.poyd_nonadd8_median_batch(P(fitch), C.c_int64(NF), NF, nm, P(ia),
                                                   P(ib), P(res), P(added), st))
    out["fitch_median"] = hbm_line(ms, nm * (3 * NF + 8), kernel="k_fitch_median", pairs=nm,
                                   row_bytes=NF)
    del res
    # Sankoff: 131,072 nodes x 256 characters x 4 states, int32 (512 MiB)
    NS, NC, K = 1 << 17, 256, 4
    sank = torch.randint(0, 20, (NS, NC, K), dtype=torch.int32, generator=g).to(dev)
    tcm = torch.tensor([[0 if i == j else 1 + (i + j) % 5 for j in range(K)] for i in range(K)],
                       dtype=torch.int32, device=dev)
    sa, sb = ia % NS, ib % NS
    row = NC * K * 4
    ms = timed(lambda: L.poyd_sank_distance_batch(P(sank), NC, K, P(tcm), n, P(sa), P(sb),
                                                  P(dist), st))
    out["sank_distance"] = hbm_line(ms, n * (2 * row + 8), kernel="k_sank_distance", pairs=n,
                                    row_bytes=row, node_array_mib=NS * row >> 20)
    ns_ = 1 << 17
    out_s = torch.empty((ns_, NC, K), dtype=torch.int32, device=dev)
    ms = timed(lambda: L.poyd_sank_median_batch(P(sank), NC, K, P(tcm), ns_, P(sa), P(sb),
                                                P(out_s), None, None, st))
    out["sank_median"] = hbm_line(ms, ns_ * 3 * row, kernel="k_sank_median", pairs=ns_,
                                  row_bytes=row)
    del out_s, sank, fitch
    torch.cuda.synchronize()
    # closest: (parent single, node median) = config-1 pairs
    host = synth.pair_batch_fast(args.seed, 8192)
    batch = align.PairBatch.from_packed([torch.from_numpy(x) for x in host], device=dev)
    cm = align.CostMatrix.default()
    for _ in range(3):
        align.closest(batch, cm)
    torch.cuda.synchronize()
    native.lib().poyd_profile_enable(1)
    native.profile_read(clear=True)
    t0 = time.perf_counter()
    for _ in range(steps):
        align.closest(batch, cm)
    torch.cuda.synchronize()
    wall = (time.perf_counter() - t0) / steps
    cms, _ = native.profile_read("closest", clear=False)
    dps, _ = native.profile_read("lin_dp_dm", clear=False)
    native.profile_read(clear=True)
    native.lib().poyd_profile_enable(0)
    out["closest"] = {"kernel": "k_closest (after the batched align_2 of each pair)", "pairs": 8192,
                      "pairs_per_s": 8192 / wall, "column_pass_ms": cms / steps,
                      "align_dp_ms": dps / steps}
    # the MLP (32-256-256-128-1): forward + backward + Adam at batch 65,536
    prop = learned.Proposal(seed=0)
    X = torch.randn((1 << 16, learned.NFEAT), generator=g).to(dev)
    y = torch.randn(1 << 16, generator=g).to(dev)
    prop.fit(X, y, epochs=1, batch=4096)
    torch.cuda.synchronize()
    native.lib().poyd_profile_enable(1)
    native.profile_read(clear=True)
    t0 = time.perf_counter()
    prop.fit(X, y, epochs=steps, batch=4096)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    gms, gn = native.profile_read("mlp_gemm", clear=False)
    native.profile_read(clear=True)
    native.lib().poyd_profile_enable(0)
    dims = (learned.NFEAT, 256, 256, 128)
    fwd = sum(2 * dims[i] * dims[i + 1] for i in range(3))  # per sample, GEMM layers
    flops = steps * (1 << 16) * (3 * fwd - 2 * dims[0] * dims[1])  # fwd, dW, dH (no dX)
    tf = flops / (gms * 1e-3) / 1e12 if gms else None
    out["mlp_gemm"] = {"kernel": "k_gemm_bf16 (mma.sync m16n8k16)", "samples_per_s":
                       steps * (1 << 16) / wall, "gemm_ms": gms, "gemm_launches": gn,
                       "tflop_s": tf, "peak_tflop_s": bf16, "frac": tf / bf16 if tf else None}
    return {"workload": "kernels: Fitch / Sankoff rows larger than L2, closest, MLP GEMMs",
            "steps": steps, "results": out}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "spr":
        _emit(run_spr(args))
    elif args.workload == "tbr":
        _emit(run_tbr(args))
    elif args.workload == "learned":
        _emit(run_learned(args))
    elif args.workload == "serving":
        _emit(run_serving(args))
    elif args.workload == "kernels":
        _emit(run_kernels(args))
    elif args.workload == "three":
        _emit(run_three(args))
    elif args.workload == "adjust":
        _emit(run_adjust(args))
    elif args.workload == "config0":
        _emit(run_config0(args))
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
