"""Launch-shape autotuner for the best-move kernels (one GPU).

For each level-graph size class it times whole clusterings of a
representative seeded graph under every launch shape
(group_max_degree {8, 16, 32} x cta_min_degree {1000, 512, 256} x
grid_waves {0.5, 1, 2}, set through pcc_set_launch_tuning) and keeps the fastest by median device time
(stats.ms_total).  The winners are written as csrc/tuning_table.cuh (or
--out), which the library compiles in; the full timing table is printed as
markdown and JSON.  Every shape must give the same labels: the tuner checks
that too, so a table it writes never changes a result.

Classes (by vertices of the level graph, the key the library looks up):
  n <= 65,536       RMAT scale 15 (modularity, headline config) and an SBM
                    of 50,000 vertices (correlation, resolution 0.05)
  n <= 1,048,576    RMAT scale 20 (modularity) and LFR 200,000 vertices
                    (correlation, real weights)
  n <= 16,777,216   RMAT scale 22 (modularity, the headline workload)
  larger            not timed: the 16M row's shape is copied

Run: python tune_launch.py [--reps 5] [--out path] [--quick]
"""

from __future__ import annotations

import argparse
import itertools
import json
import os
import statistics
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, _HERE)

import pcc_gb300 as P  # noqa: E402
import pcc_graphs as G  # noqa: E402

GROUP_MAX = (8, 16, 32)
CTA_MIN = (1000, 512, 256)
WAVES = (0.5, 1.0, 2.0)
DEFAULT = "32/1000/1.0"
CLASSES = [65536, 1048576, 16777216]


def _workloads(cls: int, quick: bool):
    headline = P.make_config(resolution=1.0, refine=True, move_method=P.NBHR_MOVE, random_seed=1)
    if cls == 65536:
        yield "rmat15_modularity", G.rmat(15, 16, seed=1), headline, 1
        g, _ = G.sbm(50_000, 250, 0.01, 0.0005, 3)
        yield "sbm50k_correlation", g, P.make_config(resolution=0.05, refine=True), 0
    elif cls == 1048576:
        yield "rmat20_modularity", G.rmat(18 if quick else 20, 16, seed=1), headline, 1
        g, _ = G.lfr(200_000, mean_degree=20, dmax=2000, seed=6)
        yield "lfr200k_correlation", g, P.make_config(resolution=0.1, refine=True, move_method=P.NBHR_CLUSTER_MOVE,
                                                      permute=True, random_seed=1), 0
    else:
        yield "rmat22_modularity", G.rmat(20 if quick else 22, 16, seed=1), headline, 1


def _run(dg, cfg, objective):
    if objective == 1:
        return P.modularity_cluster(dg, cfg)
    return P.correlation_cluster(dg, cfg)


def pick_best(per_workload):
    """The class's launch shape: the smallest sum over its workloads of
    time / default-shape time (so that the workloads weigh equally); ties
    keep the default.  per_workload: {workload: {"g/c/w": median ms}}.
    Returns (best key, {key: score})."""
    score = {}
    for gmax, cta, waves in itertools.product(GROUP_MAX, CTA_MIN, WAVES):
        key = f"{gmax}/{cta}/{waves}"
        score[key] = sum(r[key] / r[DEFAULT] for r in per_workload.values())
    best = min(score, key=lambda k: (score[k], k != DEFAULT))
    return best, score


def tune(reps: int, quick: bool):
    ctx = P.Context()
    results = {}
    table = []
    for cls in CLASSES:
        per_workload = {}
        for name, g, cfg, objective in _workloads(cls, quick):
            dg = ctx.upload(g)
            ctx.set_launch_tuning(0, 0, 0.0)
            want, _ = _run(dg, cfg, objective)
            _run(dg, cfg, objective)  # warm
            rows = {}
            for gmax, cta, waves in itertools.product(GROUP_MAX, CTA_MIN, WAVES):
                ctx.set_launch_tuning(gmax, cta, waves)
                _run(dg, cfg, objective)  # warm this shape
                ms = []
                for _ in range(reps):
                    labels, st = _run(dg, cfg, objective)
                    if not np.array_equal(labels, want):
                        raise RuntimeError(f"{name}: labels differ under {gmax}/{cta}/{waves}")
                    ms.append(st["ms_total"])
                med = statistics.median(ms)
                rows[f"{gmax}/{cta}/{waves}"] = med
            per_workload[name] = rows
            ctx.set_launch_tuning(0, 0, 0.0)
            dg.free()
        best, score = pick_best(per_workload)
        gmax, cta, waves = best.split("/")
        table.append((cls, int(gmax), int(cta), float(waves)))
        results[str(cls)] = {"workloads": per_workload, "score": score, "best": best}
    table.append((0xFFFFFFFF,) + tuple(table[-1][1:]))
    return table, results


def write_table(path: str, table) -> None:
    lines = [
        "// Best-move launch shapes by level-graph size, written by tune_launch.py",
        "// (the fastest launch shape per size class, timed on GB300).",
        "// Columns: max_vertices, group_max_degree, cta_min_degree, grid_waves.",
        "#pragma once",
        "",
        "namespace pcc {",
        "",
        "constexpr TuningRow kTuningTable[] = {",
    ]
    for n, gmax, cta, waves in table:
        lines.append(f"    {{{n}u, {gmax}u, {cta}u, {waves:.1f}f}},")
    lines += ["};", "", "}  // namespace pcc", ""]
    with open(path, "w") as f:
        f.write("\n".join(lines))


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--out", default=os.path.join(_HERE, "csrc", "tuning_table.cuh"))
    ap.add_argument("--quick", action="store_true", help="smaller graphs (a smoke run of the tuner)")
    args = ap.parse_args(argv)
    table, results = tune(args.reps, args.quick)
    write_table(args.out, table)
    for cls, r in results.items():
        print(f"\n### level graphs with n <= {cls}: best {r['best']} (group_max/cta_min/waves)\n")
        names = list(r["workloads"])
        print("| shape | " + " | ".join(f"{n} ms" for n in names) + " | score |")
        print("|---|" + "---:|" * (len(names) + 1))
        for key in r["score"]:
            cells = " | ".join(f"{r['workloads'][n][key]:.2f}" for n in names)
            print(f"| {key} | {cells} | {r['score'][key]:.3f} |")
    print(json.dumps({"table": table, "results": results}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
