"""Benchmark of the GB300 clustering hot path.

Workload (one "step" = one full ParallelModularityClusterer::Cluster on the
graph): RMAT scale 22, edge factor 16, a/b/c/d = 0.57/0.19/0.19/0.05,
symmetrised, deduplicated, self-loops removed (~60M undirected edges), unit
weights; modularity resolution 1.0, refine, NBHR_MOVE, synchronous moves.
Synthetic data from a seeded generator (no dataset download).

Metric: best-move edge visits per second -- an edge visit is one adjacency
entry scanned by a best-move evaluation; the count is summed over every
round, level and refinement pass, identically to the oracle.

  value   edge visits / device time of Cluster() with the graph resident in
          HBM (CUDA events on the library's stream, summed over the steps)
  e2e     the same metric through pcc_cluster_host_csr on pinned host
          buffers: upload + cluster + label download every step
  cpu_baseline   the oracle (the CPU restatement of the reference
          clusterer) on all host cores: one clustering of the same graph
          with the same config; its labels pin the GPU's (quality.oracle)
  --impl reference   the same oracle timed per step on the same graph and
          config; it generates the graph itself and loads no library of the
          GPU package

Three more workloads ride on the same JSON line (rank 0, one GPU each):
  lfr       LFR-like graph, 8M vertices, real weights (FP64 mode), in the
            same edge-visits/s metric, with the oracle on a 1M-vertex sample
  batched   4096 SBM graphs through the batch call (disjoint unions), in
            graphs/s end to end, beside one call per graph on a sample
  serving   the continuous-batching server under Poisson arrivals: closed-
            loop capacity and p50/p99 latency at 0.25x-1.1x of it

Multi-GPU: the path does not shard (a Louvain round needs the whole graph's
cluster state), so N GPUs run N independent replicas ("replicas only").
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

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "parallel-correlation-clustering_gb300")
sys.path.insert(0, PKG)
# The oracle (CPU restatement) is imported only by the CPU-baseline leg and
# --impl reference.
ORACLE_DIR = os.path.join(ROOT, "oracle")

METRIC = "best-move edge-visits/s"
UNIT = "edge-visits/s"

# DRAM bytes (read + write) per evaluated entry of each best-move kernel
# family, from ncu captures of RMAT scale 20, level 0, first round (the whole
# frontier; cold L2); the summary and command are in profiles/.  Traffic
# scales with the entries evaluated, so the per-launch figure at the bench's
# size is this times the entries of a launch.
TRAFFIC_BYTES_PER_ENTRY = {"groups": 51.9, "warps": 8.82, "small_hubs": 6.22, "big_hubs": 9.92}


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scale", type=int, default=22)
    ap.add_argument("--async", dest="async_", action="store_true")
    ap.add_argument("--cpu-scale", type=int, default=20,
                    help="RMAT scale of the async-quality comparison with the oracle (5 seeds each)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch-graphs", type=int, default=4096,
                    help="graphs of the batched SBM leg (0 = skip the leg)")
    ap.add_argument("--batch-sample", type=int, default=256,
                    help="graphs clustered one call each for the per-graph baseline")
    ap.add_argument("--serve-requests", type=int, default=240,
                    help="requests of the serving leg (0 = skip the leg)")
    ap.add_argument("--serve-slots", type=int, default=8)
    ap.add_argument("--lfr-n", type=int, default=8_000_000,
                    help="vertices of the LFR-like real-weight leg (0 = skip the leg)")
    ap.add_argument("--detailed-timing", action="store_true",
                    help="host-driven rounds throughout (for per-launch profilers, which do not list the "
                         "kernels of the device-side round loop's graph body)")
    return ap.parse_args()


def config_dict(args, n, m):
    return {
        "workload": f"rmat{args.scale}_ef16_modularity_refine_nbhr_{'async' if args.async_ else 'sync'}",
        "graph": f"RMAT scale {args.scale}, edge factor 16, a/b/c/d=0.57/0.19/0.19/0.05, symmetrised, "
                 "deduplicated, self-loops removed, unit weights",
        "n": n, "m_entries": m, "undirected_edges": m // 2,
        "clusterer": "ParallelModularityClusterer", "resolution": 1.0, "refine": True,
        "move_method": "NBHR_MOVE", "async": bool(args.async_),
        "louvain_num_iterations": 10, "louvain_num_inner_iterations": 10,
        "l2": "inputs larger than L2 (CSR > 129 MB), no flush",
        "parallelism": "replicas",
    }


def make_cfg(P, args):
    return P.make_config(resolution=1.0, refine=True, move_method=P.NBHR_MOVE, async_=args.async_,
                         random_seed=1)


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.idx = device_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def phases(st, bpe):
    """Per-phase device time of one clustering run with detailed timing, with
    the algorithmic GB/s of best moves, compression and the frontier push."""
    peak, _ = measured_peak()

    def rate(byts, ms):
        if not byts or not ms:
            return None, None
        gbs = byts / (ms / 1000.0) / 1e9
        return gbs, gbs / peak

    out = {"note": "one clustering with detailed timing (host-driven rounds, CUDA events per phase)",
           "total": st["ms_total"]}
    for name, key, byts in (("best_moves", "ms_best_moves", st["algo_bytes_best_moves"]),
                            ("compress", "ms_compress", st["algo_bytes_compress"]),
                            ("apply", "ms_apply", None),
                            ("frontier", "ms_frontier", st["algo_bytes_frontier"])):
        gbs, frac = rate(byts, st[key])
        out[name] = {"ms": st[key], "algo_bytes": byts, "achieved_gbs": gbs, "frac": frac}
    out["bytes_rule"] = {"best_moves": f"{bpe} B per entry + 40 B per vertex evaluated",
                         "compress": "(12 or 8) m + 8 m' + 20 n + 16 n' per contraction",
                         "frontier": "4 B per entry of each expanded row + 4 B per expanded row"}
    return out


def families(P, st, bpe, peak):
    """Best-move kernel families of one detailed-timing run: device time,
    launches and algorithmic GB/s ({bpe} B per entry + 40 B per vertex)."""
    out = {}
    for f, name in enumerate(P.PccStats.FAMILIES):
        ms, nl = st["family_ms"][f], st["family_launches"][f]
        if ms <= 0 or nl == 0:
            continue
        byts = bpe * st["family_entries"][f] + 40 * st["family_vertices"][f]
        gbs = byts / (ms / 1000.0) / 1e9
        out[name] = {"ms_per_step": ms, "launches_per_step": nl, "entries_per_step": st["family_entries"][f],
                     "achieved_gbs": gbs, "frac": gbs / peak}
    return out


def cpu_baseline(args, P, g, gpu_labels, gpu_stats):
    """The oracle on all host cores: one full clustering of the bench's own
    graph with the same config (about 15-20 s of CPU work on 16 cores).  Its
    labels and modularity also pin the GPU result of the timed steps: sync
    moves on a unit-weight graph must give identical labels."""
    import numpy as np
    sys.path.insert(0, ORACLE_DIR)
    import oracle as O
    O.set_threads(0)
    threads = O.get_threads()
    og = O.OracleGraph(g)
    cfg = make_cfg(P, args)
    t = time.perf_counter()
    labels, st = O.modularity_cluster(og, cfg)
    dt = time.perf_counter() - t
    cpu = {
        "value": st["edge_visits"] / dt, "unit": UNIT, "cores": threads, "kind": "port",
        "sample": f"one full clustering of the bench graph (RMAT scale {args.scale}, n={g.n}, m={g.m}) with the "
                  f"same config; {st['edge_visits']} edge visits in {dt:.2f} s",
    }
    same = bool(np.array_equal(labels, gpu_labels))
    parity = {
        "oracle_modularity": st["modularity"], "gpu_modularity": gpu_stats["modularity"],
        "labels_identical": same,
        "differing_labels": int((labels != gpu_labels).sum()),
        "edge_visits_equal": st["edge_visits"] == gpu_stats["edge_visits"],
        "rounds_equal": st["rounds"] == gpu_stats["rounds"],
        "levels_equal": st["levels"] == gpu_stats["levels"],
    }
    return cpu, parity


def async_quality(args, P, G, ctx, seeds: int = 5):
    """Async mode is nondeterministic (in the reference too): the GPU's mean
    modularity over seeds beside the oracle's, on RMAT scale --cpu-scale with
    the headline config in async mode.  The oracle runs on one worker (the
    reference's async result also moves with its worker count; one worker
    is deterministic per seed).  Each GPU modularity is recomputed by the
    oracle from the GPU's labels."""
    import numpy as np
    sys.path.insert(0, ORACLE_DIR)
    import oracle as O
    O.set_threads(1)
    g = G.rmat(args.cpu_scale, 16, seed=1)
    og = O.OracleGraph(g)
    dg = ctx.upload(g)
    gpu, cpu = [], []
    for seed in range(1, seeds + 1):
        cfg = P.make_config(resolution=1.0, refine=True, move_method=P.NBHR_MOVE, async_=True, random_seed=seed)
        lab, _ = P.modularity_cluster(dg, cfg)
        gpu.append(O.modularity(og, 1.0, lab))
        _, so = O.modularity_cluster(og, cfg)
        cpu.append(so["modularity"])
    dg.free()
    O.set_threads(0)
    mg, mc = float(np.mean(gpu)), float(np.mean(cpu))
    return {"graph": f"RMAT scale {args.cpu_scale} (n={g.n}, m={g.m})", "seeds": seeds, "oracle_workers": 1,
            "gpu_mean_modularity": mg, "oracle_mean_modularity": mc,
            "relative_difference": (mg - mc) / abs(mc) if mc else None,
            "gpu": gpu, "oracle": cpu}


def batched_leg(args, P, G, ctx):
    """Batched SBM workload: graphs with n log-uniform in [200, 50000],
    blocks U[2, 200], mean degree U[8, 32], p_out/p_in = 0.02, unit weights;
    correlation, resolution 0.05, refine.  Timed end to end through the
    public batch call (host CSR in, host labels out: upload, clustering and
    download inside the timed region).  The per-graph baseline is one
    pcc_cluster_host_csr call per graph on a sample of the same graphs; the
    batch's labels and objectives must equal those calls'."""
    import numpy as np
    graphs = G.batch_sbm_graphs(args.batch_graphs, seed=7)
    cfg = P.make_config(resolution=0.05, refine=True)
    sample = graphs[:min(args.batch_sample, len(graphs))]
    P.cluster_batch(graphs[:64], cfg)
    for g in sample[:4]:
        P.cluster_host_csr(ctx, g, cfg)
    t = time.perf_counter()
    ref = [P.cluster_host_csr(ctx, g, cfg) for g in sample]
    plain_s = time.perf_counter() - t
    t = time.perf_counter()
    labels, stats, wall_ms = P.cluster_batch(graphs, cfg)
    batch_s = time.perf_counter() - t
    identical = all(np.array_equal(lab, r[0]) and st["objective"] == r[1]["objective"]
                    for lab, st, r in zip(labels, stats, ref))
    value = len(graphs) / batch_s
    plain = len(sample) / plain_s
    # Breakdown: the same graphs as disjoint unions on one context with
    # detailed timing (CUDA events per phase); wall minus device time is the
    # host side (upload, union build, per-round flag reads, download).
    detailed = ctx.detailed_timing
    ctx.set_detailed_timing(True)
    t = time.perf_counter()
    _, ustats, tot = P.cluster_union(ctx, graphs, cfg)
    union_wall_ms = (time.perf_counter() - t) * 1000.0
    ctx.set_detailed_timing(detailed)
    dev_ms = tot["ms_total"]
    breakdown = {
        "note": "one more run of the same graphs as unions on one context with detailed timing",
        "wall_ms": union_wall_ms, "device_ms": dev_ms,
        "best_moves_ms": tot["ms_best_moves"], "compress_ms": tot["ms_compress"],
        "apply_ms": tot["ms_apply"], "frontier_ms": tot["ms_frontier"],
        "other_device_ms": dev_ms - tot["ms_best_moves"] - tot["ms_compress"] - tot["ms_apply"] - tot["ms_frontier"],
        "host_side_ms": union_wall_ms - dev_ms,
        "union_rounds": tot["rounds"], "kernel_launches": tot["kernel_launches"],
        "edge_visits": tot["edge_visits"],
        "best_move_edge_visits_per_s": tot["edge_visits"] / (tot["ms_best_moves"] / 1000.0)
        if tot["ms_best_moves"] > 0 else None,
    }
    return {
        "workload": "batched_sbm_correlation_refine",
        "graphs": len(graphs), "n_total": int(sum(g.n for g in graphs)), "m_total": int(sum(g.m for g in graphs)),
        "value": value, "unit": "graphs/s", "ms_per_batch": 1000.0 * batch_s,
        "per_graph_calls": {"value": plain, "unit": "graphs/s", "sample_graphs": len(sample)},
        "speedup_vs_per_graph_calls": value / plain,
        "identical_to_per_graph_calls": bool(identical),
        "path": "pcc_cluster_batch -> disjoint unions (pcc_cluster_union), host buffers in and out",
        "breakdown": breakdown,
    }


def lfr_leg(args, P, G, ctx, dist_steps: int = 2):
    """LFR-like planted partition with real weights (FP64 mode): degrees
    power-law(2.2, mean 20, max 2000), community sizes power-law(2.5,
    5..5000), mixing 0.3, weights U[0.5, 1.5] stored as float32;
    correlation, resolution 0.1, refine, NBHR_CLUSTER_MOVE, permute, sync.
    Graph resident in HBM; the oracle runs the same config on a 1M-vertex
    graph of the same distribution (bounded CPU sample)."""
    import numpy as np
    g, planted = G.lfr(args.lfr_n, mean_degree=20, dmax=2000, seed=6)
    cfg = P.make_config(resolution=0.1, refine=True, move_method=P.NBHR_CLUSTER_MOVE, permute=True, random_seed=1)
    dg = ctx.upload(g)
    P.correlation_cluster(dg, cfg)
    ev, ms = 0, 0.0
    st = labels = None
    for _ in range(dist_steps):
        labels, st = P.correlation_cluster(dg, cfg)
        ev += st["edge_visits"]
        ms += st["ms_total"]
    # One more clustering with detailed timing: the phase and family split.
    detailed = ctx.detailed_timing
    ctx.set_detailed_timing(True)
    _, sd = P.correlation_cluster(dg, cfg)
    ctx.set_detailed_timing(detailed)
    dg.free()
    # Ground-truth scoring (CompareCommunities) of the clustering against the
    # planted communities, on the device; host arrays in, report out.
    order = np.argsort(planted, kind="stable").astype(np.uint32)
    comm_off = np.zeros(int(planted.max()) + 2, np.uint64)
    comm_off[1:] = np.cumsum(np.bincount(planted), dtype=np.uint64)
    P.compare_communities(ctx, labels, offsets=comm_off, members=order)
    t = time.perf_counter()
    score, _, _ = P.compare_communities(ctx, labels, offsets=comm_off, members=order)
    score_ms = (time.perf_counter() - t) * 1000.0
    out = {
        "workload": "lfr_like_real_weights_correlation_refine_nbhr_cluster_sync",
        "n": g.n, "m_entries": g.m, "dtype": "f64 (real weights: FP64 best moves)",
        "value": ev / (ms / 1000.0), "unit": UNIT, "ms_per_step": ms / dist_steps,
        "objective": st["objective"], "num_clusters": st["num_clusters"], "levels": st["levels"],
        "rounds": st["rounds"], "mean_degree": g.m / g.n,
        "phases_ms_per_step": phases(sd, bpe=12),
        "kernel_families": families(P, sd, 12, measured_peak()[0]),
        "scoring": {"what": "CompareCommunities on the device against the planted communities "
                            "(pcc_compare_communities, host arrays in and out)",
                    "communities": int(comm_off.size - 1), "ms": score_ms,
                    "avg_precision": score["avg_precision"], "avg_recall": score["avg_recall"]},
    }
    if not args.no_cpu_baseline:
        sys.path.insert(0, ORACLE_DIR)
        import oracle as O
        O.set_threads(0)
        gs, _ = G.lfr(1_000_000, mean_degree=20, dmax=2000, seed=6)
        og = O.OracleGraph(gs)
        t = time.perf_counter()
        _, so = O.correlation_cluster(og, cfg)
        dt = time.perf_counter() - t
        out["cpu_baseline"] = {"value": so["edge_visits"] / dt, "unit": UNIT, "cores": O.get_threads(),
                               "kind": "port",
                               "sample": f"one clustering of a 1M-vertex graph of the same distribution "
                                         f"(m={gs.m}) in {dt:.2f} s"}
    return out


def serving_leg(args, P, G, ctx):
    """Serving workload: 95% graphs of the batched SBM distribution, 5% RMAT
    scale 20 (edge factor 16; two distinct graphs reused), resolution from
    {0.01, 0.1, 0.5}, modularity or correlation with equal probability,
    120 GB HBM budget, `--serve-slots` concurrent slots.  Capacity is the
    closed-loop rate (every request queued at once); then Poisson arrivals at
    0.25x, 0.5x, 0.75x, 0.9x and 1.1x that rate give latency percentiles
    (submit to completion).
    Sampled responses must equal standalone calls."""
    import numpy as np
    reqs = G.serving_requests(args.serve_requests, seed=11, rmat_scale=20, distinct_rmat=2)
    cfgs = [P.make_config(resolution=r["resolution"], refine=True) for r in reqs]
    srv = P.Server(slots=args.serve_slots, hbm_budget=120 << 30)
    try:
        for r, c in list(zip(reqs, cfgs))[:8]:
            srv.wait(srv.submit(r["graph"], c, r["objective"]))

        def closed_loop(idx):
            t0 = time.perf_counter()
            ts = [srv.submit(reqs[i]["graph"], cfgs[i], reqs[i]["objective"]) for i in idx]
            res = [srv.wait(t) for t in ts]
            return res, len(idx) / (time.perf_counter() - t0)

        closed, capacity = closed_loop(list(range(len(reqs))))
        sbm_idx = [i for i, r in enumerate(reqs) if r["kind"] == "sbm"]
        rmat_idx = [i for i, r in enumerate(reqs) if r["kind"] != "sbm"]
        _, cap_sbm = closed_loop(sbm_idx)
        _, cap_rmat = closed_loop(rmat_idx) if rmat_idx else (None, None)
        loads = []
        for frac in (0.25, 0.5, 0.75, 0.9, 1.1):
            lam = frac * capacity
            arrivals = np.cumsum(np.random.default_rng(13).exponential(1.0 / lam, len(reqs)))
            start = time.perf_counter()
            tickets = []
            for i, (r, c) in enumerate(zip(reqs, cfgs)):
                d = start + arrivals[i] - time.perf_counter()
                if d > 0:
                    time.sleep(d)
                tickets.append(srv.submit(r["graph"], c, r["objective"]))
            res = [srv.wait(t) for t in tickets]
            total = time.perf_counter() - start
            lat = np.array([x[2] for x in res])
            q = np.array([x[3] for x in res])
            loads.append({"offered_fraction_of_capacity": frac, "offered_graphs_per_s": lam,
                          "achieved_graphs_per_s": len(reqs) / total,
                          "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                          "mean_queue_ms": float(q.mean())})
    finally:
        srv.close()
    pick = [i for i, r in enumerate(reqs) if r["kind"] != "sbm"][:2] + list(range(0, len(reqs), max(len(reqs) // 12, 1)))
    identical = True
    for i in pick:
        ref, _ = P.cluster_host_csr(ctx, reqs[i]["graph"], cfgs[i], objective=reqs[i]["objective"])
        identical &= bool(np.array_equal(closed[i][0], ref))
    # Plain per-graph launches: the same requests one call after another
    # (a prefix of the mix, and a prefix of its SBM requests).
    def plain_rate(idx):
        t = time.perf_counter()
        for i in idx:
            P.cluster_host_csr(ctx, reqs[i]["graph"], cfgs[i], objective=reqs[i]["objective"])
        return len(idx) / (time.perf_counter() - t)

    plain_n = min(len(reqs), 120)
    plain = plain_rate(list(range(plain_n)))
    plain_sbm = plain_rate(sbm_idx[:60])
    return {
        "workload": "serving_sbm95_rmat20_5pct_mixed_objectives",
        "requests": len(reqs), "slots": args.serve_slots, "hbm_budget_gb": 120,
        "value": capacity, "unit": "graphs/s", "note": "value = closed-loop capacity",
        "per_graph_calls": {"value": plain, "unit": "graphs/s", "sample_requests": plain_n},
        "speedup_vs_per_graph_calls": capacity / plain,
        "by_kind": {
            "sbm": {"requests": len(sbm_idx), "capacity": cap_sbm, "per_graph_calls": plain_sbm,
                    "speedup_vs_per_graph_calls": cap_sbm / plain_sbm},
            "rmat20": {"requests": len(rmat_idx), "capacity": cap_rmat,
                       "note": "RMAT scale 20 requests take 30-220 ms each alone (NBHR_CLUSTER_MOVE); "
                               "they bound the mix's closed-loop capacity"},
        },
        "loads": loads,
        "identical_to_standalone_on_sample": identical, "sample_requests": len(pick),
    }


def reduce_over_ranks(dist, to_max, to_sum, device):
    """Replicas: the slowest rank's times and the sum of every rank's counts
    (one process per GPU; any backend)."""
    import torch
    t = torch.tensor([float(x) for x in to_max], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    s = torch.tensor([float(x) for x in to_sum], dtype=torch.float64, device=device)
    dist.all_reduce(s, op=dist.ReduceOp.SUM)
    return [float(x) for x in t.tolist()], [float(x) for x in s.tolist()]


def run_reference(args):
    """--impl reference: the oracle (the CPU restatement of the reference
    clusterer) on all host threads, rank 0 only.  Each step is one full
    clustering of the GPU arm's graph (RMAT scale --scale) with the GPU arm's
    config.  The graph comes from the oracle's own generator, so this process
    loads no library of the GPU package (the package's Python module is
    imported for its ctypes struct definitions only)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    sys.path.insert(0, ORACLE_DIR)
    import oracle as O
    import pcc_gb300 as P
    O.build()
    O.set_threads(0)
    threads = O.get_threads()
    t = time.perf_counter()
    og = O.rmat(args.scale, 16, seed=1)
    gen_s = time.perf_counter() - t
    n, m = og.info()
    cfg = make_cfg(P, args)
    for _ in range(args.warmup):
        O.modularity_cluster(og, cfg)
    total_ev = 0
    total_t = 0.0
    mod = None
    for _ in range(args.steps):
        t = time.perf_counter()
        _, st = O.modularity_cluster(og, cfg)
        total_t += time.perf_counter() - t
        total_ev += st["edge_visits"]
        mod = st["modularity"]
    value = total_ev / total_t
    sample = (f"each step one full clustering of RMAT scale {args.scale} (n={n}, m={m}), the GPU arm's graph "
              f"and config, generated by the oracle in {gen_s:.1f} s (not timed)")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total_t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded RMAT generator)", "config": config_dict(args, n, m),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "quality": {"modularity": mod, "edge_visits_per_step": total_ev // max(args.steps, 1)},
        "parity": "unpinned-vs-binary (the reference cannot be built here); this arm is the oracle restatement",
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    import numpy as np
    import torch
    import pcc_gb300 as P
    import pcc_graphs as G
    import build_native

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    build_native.build_all()

    g = G.rmat(args.scale, 16, seed=1)
    ctx = P.Context(local)
    ctx.set_detailed_timing(args.detailed_timing)
    dg = ctx.upload(g)
    cfg = make_cfg(P, args)

    def barrier():
        torch.cuda.synchronize(local)
        if dist is not None:
            dist.barrier()

    for _ in range(max(args.warmup, 0)):
        P.modularity_cluster(dg, cfg)
    bpe = 12 if g.weights is not None else 8   # algorithmic bytes per entry evaluated

    # Timed region: K full clusterings on the resident graph.
    sampler = ClockSampler(local)
    barrier()
    sampler.start()
    wall0 = time.perf_counter()
    ev = 0
    vv = 0
    dev_ms = 0.0
    bm_ms = 0.0
    algo_bytes = 0
    labels = last_stats = None
    launches = 0
    fam_ms = [0.0] * 4
    fam_launch = [0] * 4
    fam_e = [0] * 4
    fam_v = [0] * 4
    quality = {}
    for _ in range(args.steps):
        labels, st = P.modularity_cluster(dg, cfg)
        last_stats = st
        ev += st["edge_visits"]
        vv += st["vertex_visits"]
        dev_ms += st["ms_total"]
        launches += st["kernel_launches"]
        quality = {"modularity": st["modularity"], "objective": st["objective"],
                   "num_clusters": st["num_clusters"], "levels": st["levels"], "rounds": st["rounds"]}
    barrier()
    wall = time.perf_counter() - wall0
    clocks = sampler.stop()

    # The timed steps run the rounds as a device-side graph loop; one more
    # clustering with detailed timing (host-driven rounds, CUDA events around
    # every phase and best-move kernel family) gives the breakdown and the
    # per-launch figures of the roofline.
    ctx.set_detailed_timing(True)
    _, st_detail = P.modularity_cluster(dg, cfg)
    ctx.set_detailed_timing(args.detailed_timing)
    st = st_detail
    bm_ms = st["ms_best_moves"]
    algo_bytes = st["algo_bytes_best_moves"]
    for f in range(4):
        fam_ms[f] = st["family_ms"][f]
        fam_launch[f] = st["family_launches"][f]
        fam_e[f] = st["family_entries"][f]
        fam_v[f] = st["family_vertices"][f]

    # End to end through the public C ABI from pinned host memory.
    off_h = torch.from_numpy(g.offsets.view(np.int64)).pin_memory()
    nbr_h = torch.from_numpy(g.neighbors.view(np.int32)).pin_memory()
    g_pinned = P.CsrGraph(off_h.numpy().view(np.uint64), nbr_h.numpy().view(np.uint32), None)
    P.cluster_host_csr(ctx, g_pinned, cfg, objective=1)
    barrier()
    e2e_t = 0.0
    e2e_ev = 0
    for _ in range(args.steps):
        t = time.perf_counter()
        lab, st = P.cluster_host_csr(ctx, g_pinned, cfg, objective=1)
        e2e_t += time.perf_counter() - t
        e2e_ev += st["edge_visits"]
    barrier()

    # The same configuration in async mode (reported beside the sync line).
    acfg = P.make_config(resolution=1.0, refine=True, move_method=P.NBHR_MOVE, async_=True, random_seed=1)
    P.modularity_cluster(dg, acfg)
    a_ev, a_ms, a_mod = 0, 0.0, []
    for _ in range(args.steps):
        _, st = P.modularity_cluster(dg, acfg)
        a_ev += st["edge_visits"]
        a_ms += st["ms_total"]
        a_mod.append(st["modularity"])
    barrier()

    # Whole-cluster moves (DEFAULT_CLUSTER_MOVES): one level of up to 20
    # rounds, each with vertex moves then whole-cluster moves.
    ccfg = P.make_config(resolution=1.0, move_method=P.NBHR_MOVE, clustering_moves_method=P.DEFAULT_CLUSTER_MOVES)
    P.modularity_cluster(dg, ccfg)
    c_ev, c_ms, c_mod, c_steps = 0, 0.0, None, min(args.steps, 3)
    for _ in range(c_steps):
        _, st = P.modularity_cluster(dg, ccfg)
        c_ev += st["edge_visits"]
        c_ms += st["ms_total"]
        c_mod = st["modularity"]
    barrier()

    # Async quality against the oracle (rank 0; RMAT scale --cpu-scale).
    async_check = None
    if rank == 0 and not args.no_cpu_baseline:
        async_check = async_quality(args, P, G, ctx)

    # Batched and serving workloads (rank 0; one GPU each).
    batched = serving = lfr = None
    if rank == 0 and args.lfr_n > 0:
        lfr = lfr_leg(args, P, G, ctx)
    if rank == 0 and args.batch_graphs > 0:
        batched = batched_leg(args, P, G, ctx)
    if rank == 0 and args.serve_requests > 0:
        serving = serving_leg(args, P, G, ctx)
    barrier()

    # Max time over ranks; edge visits summed over ranks.
    dev_s = dev_ms / 1000.0
    if dist is not None:
        (dev_s, e2e_t), (ev_all, e2e_ev_all) = reduce_over_ranks(dist, [dev_s, e2e_t], [ev, e2e_ev],
                                                                 f"cuda:{local}")
    else:
        ev_all, e2e_ev_all = float(ev), float(e2e_ev)

    if rank == 0:
        peak, peak_kind = measured_peak()
        names = P.PccStats.FAMILIES
        families = {}
        for f in range(4):
            if fam_ms[f] <= 0 or fam_launch[f] == 0:
                continue
            byts = bpe * fam_e[f] + 40 * fam_v[f]
            gbs = byts / (fam_ms[f] / 1000.0) / 1e9
            families[names[f]] = {
                "ms_per_step": fam_ms[f], "launches_per_step": fam_launch[f],
                "entries_per_step": fam_e[f], "achieved_gbs": gbs, "frac": gbs / peak}
        top = max(range(4), key=lambda f: fam_ms[f])
        top_bytes_per_launch = (bpe * fam_e[top] + 40 * fam_v[top]) / max(fam_launch[top], 1)
        top_ms_per_launch = fam_ms[top] / max(fam_launch[top], 1)
        achieved = top_bytes_per_launch / (top_ms_per_launch / 1000.0) / 1e9 if top_ms_per_launch > 0 else None
        # DRAM bytes per evaluated entry of the family's kernels, from the ncu
        # capture summarised in profiles/ (RMAT scale 20, level 0, round 1).
        traffic_per_entry = TRAFFIC_BYTES_PER_ENTRY.get(names[top])
        traffic = (traffic_per_entry * fam_e[top] / max(fam_launch[top], 1)) if traffic_per_entry else None
        cpu = None
        pinning = None
        if not args.no_cpu_baseline:
            try:
                cpu, pinning = cpu_baseline(args, P, g, labels, last_stats)
            except Exception as e:  # the baseline is reported, never required
                cpu = {"value": None, "unit": UNIT, "cores": None, "kind": "port", "sample": f"failed: {e}"}

        line = {
            "metric": METRIC, "value": ev_all / dev_s, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * dev_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded RMAT generator)",
            "config": config_dict(args, g.n, g.m),
            "e2e": {"value": e2e_ev_all / e2e_t, "unit": UNIT,
                    "h2d_bytes_per_step": int(g.offsets.nbytes + g.neighbors.nbytes),
                    "d2h_bytes_per_step": int(4 * g.n)},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                         "kernel": f"best-move family '{names[top]}' (largest device time): "
                                   f"{bpe} B per entry + 40 B per vertex evaluated, per launch",
                         "peak_kind": f"{peak_kind} hbm_gbs",
                         "best_move_phase_gbs": (algo_bytes / (bm_ms / 1000.0)) / 1e9 if bm_ms > 0 else None},
            "kernel_families": families,
            "cpu_baseline": cpu,
            "clocks": clocks,
            "gpu_launches": launches,
            "phases_ms_per_step": phases(st_detail, bpe),
            "wall_s": wall,
            "quality": dict(quality, **({"oracle": pinning} if pinning else {})),
            "parity": "unpinned-vs-binary (the reference cannot be built here), "
                      + ("bit-exact-vs-oracle on this graph" if pinning and pinning["labels_identical"]
                         else "checked against the oracle on this graph: see quality.oracle"
                         if pinning else "not checked in this run"),
            "modes": {"async": {"value": a_ev / (a_ms / 1000.0) if a_ms > 0 else None, "unit": UNIT,
                                "ms_per_step": a_ms / args.steps, "modularity_mean": sum(a_mod) / len(a_mod),
                                "note": "same graph and config with async=true, 16 waves per round"},
                      "async_quality": async_check,
                      "cluster_moves": {"value": c_ev / (c_ms / 1000.0) if c_ms > 0 else None, "unit": UNIT,
                                        "ms_per_step": c_ms / c_steps if c_steps else None, "modularity": c_mod,
                                        "note": "same graph, clustering_moves_method DEFAULT_CLUSTER_MOVES "
                                                "(one level, 20 rounds, whole-cluster moves after each "
                                                "round's vertex moves), no refine"}},
            "lfr": lfr,
            "batched": batched,
            "serving": serving,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
