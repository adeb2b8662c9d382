"""GPU parity on the measured workloads' own configurations, at the largest
sizes the oracle finishes in seconds:

  * the RMAT headline config (ParallelModularityClusterer, resolution 1.0,
    refine, NBHR_MOVE, synchronous, 10 x 10 iterations) on RMAT scale 18 and
    20 with the bench's generator parameters: labels, edge visits, rounds,
    levels and modularity bit-exact against the oracle;
  * the LFR-like real-weight config (correlation, resolution 0.1, refine,
    NBHR_CLUSTER_MOVE, permute) at 200k vertices: FP64 mode, objective within
    1e-9 relative;
  * a graph of the batched SBM distribution with 20k-50k vertices
    (correlation, resolution 0.05, refine), through the batch call and a
    single call: labels bit-exact against the oracle.
"""

import numpy as np
import pytest

import oracle as O
import pcc_gb300 as P
import pcc_graphs as G

pytestmark = pytest.mark.gpu

REL_TOL = 1e-9


@pytest.mark.parametrize("scale", [18, 20])
def test_rmat_headline_config_bit_exact(ctx, built, scale):
    g = G.rmat(scale, 16, 0.57, 0.19, 0.19, seed=1)
    cfg = P.make_config(resolution=1.0, refine=True, move_method=P.NBHR_MOVE, async_=False,
                        louvain_num_iterations=10, louvain_num_inner_iterations=10, random_seed=1)
    dg = ctx.upload(g)
    lab_g, st_g = P.modularity_cluster(dg, cfg)
    dg.free()
    lab_o, st_o = O.modularity_cluster(O.OracleGraph(g), cfg)
    np.testing.assert_array_equal(lab_g, lab_o)
    for key in ("edge_visits", "vertex_visits", "rounds", "levels", "refine_passes", "num_clusters"):
        assert st_g[key] == st_o[key], (key, st_g[key], st_o[key])
    assert st_g["modularity"] == pytest.approx(st_o["modularity"], rel=REL_TOL, abs=1e-12)
    assert st_g["modularity"] == pytest.approx(O.modularity(O.OracleGraph(g), 1.0, lab_g), rel=REL_TOL, abs=1e-12)


def test_lfr_200k_real_weights_objective(ctx, built):
    g, _ = G.lfr(200_000, mean_degree=20, dmax=2000, seed=6)
    assert g.weights is not None
    cfg = P.make_config(resolution=0.1, refine=True, move_method=P.NBHR_CLUSTER_MOVE, permute=True, random_seed=1)
    dg = ctx.upload(g)
    lab_g, st_g = P.correlation_cluster(dg, cfg)
    dg.free()
    og = O.OracleGraph(g)
    _, st_o = O.correlation_cluster(og, cfg)
    # The GPU's own objective, recomputed by the oracle from its labels.
    assert st_g["objective"] == pytest.approx(O.objective(og, cfg, lab_g), rel=REL_TOL)
    assert st_g["objective"] == pytest.approx(st_o["objective"], rel=REL_TOL)


def test_batched_distribution_graph_bit_exact(ctx, built):
    graphs = G.batch_sbm_graphs(64, seed=7)
    big = [g for g in graphs if 20_000 <= g.n <= 50_000]
    assert big, "no graph of 20k-50k vertices in the sample"
    g = big[0]
    cfg = P.make_config(resolution=0.05, refine=True)
    lab_o, st_o = O.correlation_cluster(O.OracleGraph(g), cfg)
    lab_s, st_s = P.cluster_host_csr(ctx, g, cfg)
    np.testing.assert_array_equal(lab_s, lab_o)
    assert st_s["edge_visits"] == st_o["edge_visits"]
    assert st_s["objective"] == pytest.approx(st_o["objective"], rel=REL_TOL)
    # Inside a batch beside other graphs of the distribution.
    labels, stats, _ = P.cluster_batch([graphs[0], g, graphs[1]], cfg)
    np.testing.assert_array_equal(labels[1], lab_o)
    assert stats[1]["objective"] == st_s["objective"]
