"""GPU test of the C++ host mirror end to end: the CLI reads a GBBS file,
clusters on the GPU and writes the clustering; it must equal the clustering
the C ABI returns for the same graph and config, and the oracle's."""

import os
import subprocess

import numpy as np
import pytest

import oracle as O
import pcc_gb300 as P
import pcc_graphs as G

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "parallel-correlation-clustering_gb300", "_build", "cluster-in-memory_main")


def _read_clustering(path):
    out = []
    with open(path) as f:
        for line in f:
            out.append([int(x) for x in line.rstrip("\n").split("\t") if x])
    return out


@pytest.mark.parametrize("device_io", [True, False])
@pytest.mark.parametrize("case", ["sbm_corr", "sbm_mod", "lfr_weighted"])
def test_cli_matches_c_abi(ctx, tmp_path, case, device_io):
    """--device_io (the default) parses the graph and formats the clustering
    on the GPU; --nodevice_io uses the host reader and writer."""
    if case == "lfr_weighted":
        g, truth = G.lfr(5000, mean_degree=15, dmax=300, seed=3)
        name, objective = "ParallelCorrelationClusterer", 0
        text = "correlation_clusterer_config { resolution: 0.1 refine: true move_method: NBHR_CLUSTER_MOVE }"
        kw = dict(resolution=0.1, refine=True)
    else:
        g, truth = G.sbm(3000, 30, 0.05, 0.0005, 21)
        if case == "sbm_corr":
            name, objective = "ParallelCorrelationClusterer", 0
            text = ("correlation_clusterer_config { resolution: 0.01 refine: true move_method: ALL_MOVE "
                    "louvain_config { num_iterations: 10 num_inner_iterations: 10 } }")
            kw = dict(resolution=0.01, refine=True, move_method=P.ALL_MOVE, louvain_num_iterations=10,
                      louvain_num_inner_iterations=10)
        else:
            name, objective = "ParallelModularityClusterer", 1
            text = "correlation_clusterer_config { resolution: 1.0 refine: true move_method: NBHR_MOVE }"
            kw = dict(resolution=1.0, refine=True, move_method=P.NBHR_MOVE)
    gpath = str(tmp_path / "g.adj")
    G.write_gbbs(gpath, g)
    cpath = tmp_path / "truth.txt"
    comms = [np.flatnonzero(truth == c) for c in np.unique(truth)]
    cpath.write_text("".join("".join(f"{v}\t" for v in c) + "\n" for c in comms))
    out = str(tmp_path / "clustering.txt")
    args = [CLI, f"--clusterer_name={name}", f"--clusterer_config={text}", f"--input_graph={gpath}",
            f"--output_clustering={out}", f"--input_communities={cpath}"]
    if g.weights is not None:
        args.append("--float_weighted")
    if not device_io:
        args.append("--nodevice_io")
    r = subprocess.run(args, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "Avg precision:" in r.stdout and "Avg recall:" in r.stdout
    got = _read_clustering(out)
    with open(out) as f:
        text_out = f.read()
    assert text_out == "".join("".join(f"{v}\t" for v in c) + "\n" for c in got)

    cfg = P.make_config(**kw)
    dg = ctx.upload(g)
    if objective == 1:
        labels, _ = P.modularity_cluster(dg, cfg)
    else:
        labels, _ = P.correlation_cluster(dg, cfg)
    dg.free()
    assert got == P.labels_to_clustering(labels)
    og = O.OracleGraph(g)
    o_labels, _ = (O.modularity_cluster if objective == 1 else O.correlation_cluster)(og, cfg)
    if g.weights is None:
        np.testing.assert_array_equal(labels, o_labels)
    # The CLI's scores equal the host library's CompareCommunities.
    scores = G.compare_communities(str(cpath), labels)
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("Avg precision:")][0]
    assert abs(float(line.split(":")[1]) - scores["avg_precision"]) < 1e-12
