"""GPU parity tests: the CUDA path (through the C ABI) against the oracle.

Bar (from the clustering path's contract):
  * integer-weight graphs: best-move decisions, contraction and full sync
    clusterings are bit-exact;
  * real weights: objective within 1e-9 relative and >= 99.9% of single-round
    decisions identical (in practice all, since the <= 1000-degree sums run
    in the reference's order);
"""

import numpy as np
import pytest

import oracle as O
import pcc_gb300 as P
import pcc_graphs as G
from conftest import rand_state

pytestmark = pytest.mark.gpu

REL_TOL = 1e-9
ASYNC_SEEDS = 20      # seeds per side of the async quality comparison
ASYNC_WINDOW = 0.005  # |GPU mean - oracle mean| / |oracle mean|


def _graphs():
    """Named test graphs covering every degree bin and both arithmetic modes."""
    out = {}
    g, _ = G.sbm(2000, 20, 0.05, 0.001, 7)
    out["sbm2k"] = g
    out["rmat14"] = G.rmat(14, 16, seed=3)          # hubs > 1000 (CTA bin)
    out["rmat16"] = G.rmat(16, 16, seed=5)          # hubs > 4096 (global-hash bin)
    lg, _ = G.lfr(20000, mean_degree=20, dmax=1500, seed=9)
    out["lfr20k_real"] = lg                         # real weights -> FP64 mode
    rng = np.random.default_rng(11)
    gi, _ = G.sbm(3000, 10, 0.03, 0.002, 13)
    src = np.repeat(np.arange(gi.n), np.diff(gi.offsets).astype(np.int64))
    keep = src < gi.neighbors
    s, d = src[keep], gi.neighbors[keep].astype(np.int64)
    w = rng.integers(1, 6, size=s.size).astype(np.float32)
    out["sbm3k_int"] = P.CsrGraph.from_edges(gi.n, s, d, w)   # integer weights -> INT mode
    # Two hubs of degree 100k and 60k on an SBM: 9 and 5 partitions, the
    # global path (rows spread over many CTAs, per-hub HBM tables).
    hb, _ = G.sbm(120000, 100, 0.004, 0.00002, 17)
    src = np.repeat(np.arange(hb.n), np.diff(hb.offsets).astype(np.int64))
    keep = src < hb.neighbors
    s = np.concatenate([src[keep], np.zeros(100000, np.int64), np.ones(60000, np.int64)])
    d = np.concatenate([hb.neighbors[keep].astype(np.int64), np.arange(1, 100001), np.arange(50000, 110000)])
    out["hubs100k"] = P.CsrGraph.from_edges(hb.n, s, d)
    wr = rng.uniform(0.5, 1.5, size=s.size).astype(np.float32)
    out["hubs100k_real"] = P.CsrGraph.from_edges(hb.n, s, d, wr)
    return out


@pytest.fixture(scope="module")
def graphs(built):
    return _graphs()


def _both(ctx, g):
    return ctx.upload(g), O.OracleGraph(g)


@pytest.mark.parametrize("name", ["sbm2k", "rmat14", "rmat16", "sbm3k_int", "lfr20k_real", "hubs100k"])
@pytest.mark.parametrize("nclusters_div", [1, 7, 300])
def test_best_moves_replay(ctx, graphs, name, nclusters_div):
    """One sync best-move pass from a random state: GPU == oracle."""
    g = graphs[name]
    dg, og = _both(ctx, g)
    C, s, k, K = rand_state(g.n, g.n // nclusters_div, seed=nclusters_div)
    for res, off in ((0.01, 0.0), (0.3, 0.0), (0.05, 1.0)):
        cfg = P.make_config(resolution=res, edge_weight_offset=off)
        t_g, v_g, m_g = P.best_moves(dg, cfg, C, s, k, K)
        t_o, v_o, m_o = O.best_moves(og, cfg, C, s, k, K)
        deg = g.degrees()
        if g.weights is None or np.all(g.weights == np.round(g.weights)):
            np.testing.assert_array_equal(t_g, t_o)
            np.testing.assert_array_equal(v_g.view(np.uint64), v_o.view(np.uint64))
            np.testing.assert_array_equal(m_g, m_o)
        else:
            low = deg <= 1000   # the reference's sequential path: same order, bit-exact
            np.testing.assert_array_equal(t_g[low], t_o[low])
            np.testing.assert_array_equal(v_g[low].view(np.uint64), v_o[low].view(np.uint64))
            agree = np.mean(m_g == m_o)
            assert agree >= 0.999, agree
            np.testing.assert_allclose(v_g, v_o, rtol=REL_TOL, atol=1e-12)


@pytest.mark.parametrize("name", ["sbm2k", "rmat14", "sbm3k_int", "lfr20k_real"])
def test_compress_bit_exact(ctx, graphs, name):
    """CompressGraph: same CSR (ids, order, FP32 sums) and node weights."""
    g = graphs[name]
    dg, og = _both(ctx, g)
    for nclusters_div in (3, 50):
        C, s, k, K = rand_state(g.n, max(1, g.n // nclusters_div), seed=nclusters_div)
        k = np.arange(g.n, dtype=np.float64) % 5 + 1
        gc = P.compress(dg, C, k)
        got = gc.download()
        got_k = gc.node_weights()
        want, want_k = O.compress(og, C, k)
        np.testing.assert_array_equal(got.offsets, want.offsets)
        np.testing.assert_array_equal(got.neighbors, want.neighbors)
        np.testing.assert_array_equal(got.weights.view(np.uint32), want.weights.view(np.uint32))
        np.testing.assert_array_equal(got_k, want_k)
        gc.free()


CONFIGS = [
    dict(resolution=0.01, refine=True, move_method=P.ALL_MOVE),
    dict(resolution=0.05, refine=True, move_method=P.NBHR_MOVE),
    dict(resolution=0.1, refine=False, move_method=P.NBHR_CLUSTER_MOVE),
    dict(resolution=0.2, refine=True, move_method=P.NBHR_CLUSTER_MOVE,
         louvain_num_iterations=3, louvain_num_inner_iterations=4),
    dict(resolution=0.02, edge_weight_offset=0.0, refine=False, move_method=P.ALL_MOVE,
         louvain_num_iterations=1),
]


@pytest.mark.parametrize("name", ["sbm2k", "rmat14", "sbm3k_int", "hubs100k"])
@pytest.mark.parametrize("ci", range(len(CONFIGS)))
def test_correlation_cluster_bit_exact(ctx, graphs, name, ci):
    g = graphs[name]
    dg, og = _both(ctx, g)
    cfg = P.make_config(**CONFIGS[ci])
    lab_g, st_g = P.correlation_cluster(dg, cfg)
    lab_o, st_o = O.correlation_cluster(og, cfg)
    np.testing.assert_array_equal(lab_g, lab_o)
    assert st_g["num_clusters"] == st_o["num_clusters"]
    assert st_g["edge_visits"] == st_o["edge_visits"]
    assert st_g["rounds"] == st_o["rounds"]
    assert st_g["levels"] == st_o["levels"]
    assert st_g["objective"] == pytest.approx(st_o["objective"], rel=REL_TOL, abs=1e-9)


@pytest.mark.parametrize("name", ["sbm2k", "rmat14", "rmat16", "hubs100k"])
@pytest.mark.parametrize("move", [P.NBHR_MOVE, P.ALL_MOVE])
def test_modularity_cluster_bit_exact(ctx, graphs, name, move):
    g = graphs[name]
    dg, og = _both(ctx, g)
    cfg = P.make_config(resolution=1.0, refine=True, move_method=move)
    lab_g, st_g = P.modularity_cluster(dg, cfg)
    lab_o, st_o = O.modularity_cluster(og, cfg)
    np.testing.assert_array_equal(lab_g, lab_o)
    assert st_g["edge_visits"] == st_o["edge_visits"]
    assert st_g["modularity"] == pytest.approx(st_o["modularity"], rel=REL_TOL, abs=1e-12)
    assert st_g["objective"] == pytest.approx(st_o["objective"], rel=REL_TOL, abs=1e-12)


@pytest.mark.parametrize("name", ["lfr20k_real", "hubs100k_real"])
def test_real_weights_full_run(ctx, graphs, name):
    """FP64 mode end to end: objective within 1e-9 relative of the oracle."""
    g = graphs[name]
    dg, og = _both(ctx, g)
    cfg = P.make_config(resolution=0.1, refine=True, move_method=P.NBHR_CLUSTER_MOVE)
    lab_g, st_g = P.correlation_cluster(dg, cfg)
    lab_o, st_o = O.correlation_cluster(og, cfg)
    assert st_g["objective"] == pytest.approx(st_o["objective"], rel=REL_TOL)
    assert np.mean(lab_g == lab_o) >= 0.999


def test_objective_and_modularity_api(ctx, graphs):
    g = graphs["sbm2k"]
    dg, og = _both(ctx, g)
    rng = np.random.default_rng(0)
    lab = rng.integers(0, 40, size=g.n).astype(np.uint32)
    for res, off in ((0.01, 0.0), (0.5, 0.25)):
        cfg = P.make_config(resolution=res, edge_weight_offset=off)
        assert P.objective(dg, cfg, lab) == pytest.approx(O.objective(og, cfg, lab), rel=REL_TOL)
    assert P.modularity(dg, 1.0, lab) == pytest.approx(O.modularity(og, 1.0, lab), rel=REL_TOL)


def test_initial_clustering_and_node_weights(ctx, graphs):
    """RefineClusters(config, &clustering) with node weights (integral)."""
    g = graphs["sbm3k_int"]
    dg, og = _both(ctx, g)
    rng = np.random.default_rng(5)
    init = rng.integers(0, 200, size=g.n).astype(np.uint32)
    k = rng.integers(1, 4, size=g.n).astype(np.float64)
    cfg = P.make_config(resolution=0.05, refine=True, move_method=P.NBHR_MOVE)
    lab_g, st_g = P.correlation_cluster(dg, cfg, node_weights=k, initial_labels=init)
    lab_o, st_o = O.correlation_cluster(og, cfg, node_weights=k, initial_labels=init)
    np.testing.assert_array_equal(lab_g, lab_o)


def test_edge_cases(ctx):
    # isolated vertices, a self-loop, a duplicate entry, a star hub > 4096
    n = 6000
    src = [0] * 5000 + [5001, 5002, 5003, 5003]
    dst = list(range(1, 5001)) + [5002, 5001, 5003, 5004]
    g = P.CsrGraph.from_edges(n, src, dst, dedupe=False)
    dg, og = _both(ctx, g)
    for cfg in (P.make_config(resolution=0.01, refine=True, move_method=P.NBHR_MOVE),
                P.make_config(resolution=0.5, refine=False, move_method=P.ALL_MOVE)):
        lab_g, _ = P.correlation_cluster(dg, cfg)
        lab_o, _ = O.correlation_cluster(og, cfg)
        np.testing.assert_array_equal(lab_g, lab_o)
    # a single vertex, no edges
    g1 = P.CsrGraph(np.zeros(2, np.uint64), np.zeros(0, np.uint32))
    d1 = ctx.upload(g1)
    lab, st = P.correlation_cluster(d1, P.make_config(resolution=0.1))
    assert lab.tolist() == [0] and st["num_clusters"] == 1


def test_c1_sbm10k_config_bit_exact(ctx):
    """The CPU-runnable config exactly: SBM n = 10,000, 50 blocks of
    uniform-multinomial sizes, p_in 0.05, p_out 0.0005, unit weights (mean
    degree 14.9); correlation, resolution 0.01, refine, sync, ALL_MOVE, 10 x 10
    iterations.  Labels, counters and objective equal the oracle's."""
    g, _ = G.sbm(10000, 50, 0.05, 0.0005, 1)
    dg, og = _both(ctx, g)
    cfg = P.make_config(resolution=0.01, refine=True, move_method=P.ALL_MOVE, louvain_num_iterations=10,
                        louvain_num_inner_iterations=10)
    lab_g, st_g = P.correlation_cluster(dg, cfg)
    lab_o, st_o = O.correlation_cluster(og, cfg)
    np.testing.assert_array_equal(lab_g, lab_o)
    assert st_g["edge_visits"] == st_o["edge_visits"]
    assert st_g["rounds"] == st_o["rounds"]
    assert st_g["levels"] == st_o["levels"]
    assert st_g["objective"] == pytest.approx(st_o["objective"], rel=REL_TOL, abs=1e-9)


# Whole-cluster moves (DEFAULT_CLUSTER_MOVES): one level of num_iterations
# rounds, each with vertex moves then whole-cluster moves.  With refine the
# reference's level loop returns the identity clustering (a single level has
# nothing to refine into).
CM_CONFIGS = [
    dict(resolution=0.05, move_method=P.ALL_MOVE, num_iterations=8),
    dict(resolution=0.1, move_method=P.NBHR_CLUSTER_MOVE),
    dict(resolution=0.02, edge_weight_offset=0.5, move_method=P.NBHR_MOVE, num_iterations=12),
    dict(resolution=0.01, move_method=P.NBHR_CLUSTER_MOVE, refine=True),
]


@pytest.mark.parametrize("name", ["sbm2k", "rmat14", "sbm3k_int", "hubs100k"])
@pytest.mark.parametrize("ci", range(len(CM_CONFIGS)))
def test_cluster_moves_bit_exact(ctx, graphs, name, ci):
    g = graphs[name]
    dg, og = _both(ctx, g)
    cfg = P.make_config(clustering_moves_method=P.DEFAULT_CLUSTER_MOVES, **CM_CONFIGS[ci])
    lab_g, st_g = P.correlation_cluster(dg, cfg)
    lab_o, st_o = O.correlation_cluster(og, cfg)
    np.testing.assert_array_equal(lab_g, lab_o)
    assert st_g["edge_visits"] == st_o["edge_visits"]
    assert st_g["rounds"] == st_o["rounds"]
    assert st_g["levels"] == st_o["levels"]
    assert st_g["objective"] == pytest.approx(st_o["objective"], rel=REL_TOL, abs=1e-9)


@pytest.mark.parametrize("name", ["sbm2k", "rmat16"])
@pytest.mark.parametrize("move", [P.NBHR_MOVE, P.NBHR_CLUSTER_MOVE])
def test_modularity_cluster_moves_bit_exact(ctx, graphs, name, move):
    g = graphs[name]
    dg, og = _both(ctx, g)
    cfg = P.make_config(resolution=1.0, move_method=move, clustering_moves_method=P.DEFAULT_CLUSTER_MOVES)
    lab_g, st_g = P.modularity_cluster(dg, cfg)
    lab_o, st_o = O.modularity_cluster(og, cfg)
    np.testing.assert_array_equal(lab_g, lab_o)
    assert st_g["rounds"] == st_o["rounds"]
    assert st_g["modularity"] == pytest.approx(st_o["modularity"], rel=REL_TOL, abs=1e-12)


def test_cluster_moves_real_weights(ctx, graphs):
    """FP64 mode with whole-cluster moves: objective within 1e-9 relative."""
    g = graphs["lfr20k_real"]
    dg, og = _both(ctx, g)
    cfg = P.make_config(resolution=0.1, move_method=P.NBHR_CLUSTER_MOVE,
                        clustering_moves_method=P.DEFAULT_CLUSTER_MOVES)
    _, st_g = P.correlation_cluster(dg, cfg)
    _, st_o = O.correlation_cluster(og, cfg)
    assert st_g["objective"] == pytest.approx(st_o["objective"], rel=REL_TOL)


def _same(a, b):
    return a == b or (isinstance(a, float) and isinstance(b, float) and np.isnan(a) and np.isnan(b))


@pytest.mark.parametrize("ci", range(3))
def test_compare_communities_device(ctx, ci):
    """Device CompareCommunities equals the oracle bit for bit: repeats, ids
    outside the graph, empty communities, sparse labels, > 1024 communities."""
    from test_oracle import community_cases
    labels, comms = community_cases()[ci]
    got, gp, gr = P.compare_communities(ctx, labels, comms)
    want, wp, wr = O.compare_communities(labels, comms)
    np.testing.assert_array_equal(gp, wp)
    np.testing.assert_array_equal(gr, wr)
    for key, val in want.items():
        assert _same(float(got[key]), float(val)), key


def test_compare_communities_planted(ctx, graphs):
    """A GPU clustering of an SBM scored against its planted blocks."""
    g, blocks = G.sbm(3000, 30, 0.05, 0.001, 21)
    dg = ctx.upload(g)
    labels, _ = P.correlation_cluster(dg, P.make_config(resolution=0.02, refine=True))
    comms = [np.flatnonzero(blocks == b).tolist() for b in range(int(blocks.max()) + 1)]
    got, gp, gr = P.compare_communities(ctx, labels, comms)
    want, wp, wr = O.compare_communities(labels, comms)
    np.testing.assert_array_equal(gp, wp)
    np.testing.assert_array_equal(gr, wr)
    for key, val in want.items():
        assert _same(float(got[key]), float(val)), key
    assert got["avg_precision"] > 0.5 and got["avg_recall"] > 0.5
    # No graph: every member is outside it; sizes report the reference's
    # start values.
    got0, gp0, _ = P.compare_communities(ctx, np.zeros(0, np.uint32), [[0, 1], []])
    want0, wp0, _ = O.compare_communities(np.zeros(0, np.uint32), [[0, 1], []])
    np.testing.assert_array_equal(gp0, wp0)
    for key, val in want0.items():
        assert _same(float(got0[key]), float(val)), key
    with pytest.raises(P.PccError) as e:  # labels must be below n
        P.compare_communities(ctx, np.array([0, 5], np.uint32), [[0]])
    assert e.value.code == 3


def test_errors_are_status_codes(ctx, graphs):
    g = graphs["sbm2k"]
    dg = ctx.upload(g)
    with pytest.raises(P.PccError) as e:
        P.correlation_cluster(dg, P.make_config(clustering_moves_method=7))
    assert e.value.code == 12  # UNIMPLEMENTED, as the reference
    with pytest.raises(P.PccError) as e:  # subcluster moves inside cluster-move rounds are not built
        P.correlation_cluster(dg, P.make_config(subclustering_method=1,
                                                clustering_moves_method=P.DEFAULT_CLUSTER_MOVES))
    assert e.value.code == 12
    with pytest.raises(P.PccError) as e:
        P.correlation_cluster(dg, P.make_config(subclustering_method=9))
    assert e.value.code == 12
    bad = np.full(g.n, g.n + 5, np.uint32)
    with pytest.raises(P.PccError) as e:
        P.correlation_cluster(dg, P.make_config(), initial_labels=bad)
    assert e.value.code == 3  # INVALID_ARGUMENT
    with pytest.raises(P.PccError) as e:
        ctx.upload(P.CsrGraph(np.array([0, 1], np.uint64), np.array([7], np.uint32)))
    assert e.value.code == 3


def test_hbm_budget_admission(built):
    c = P.Context(0, hbm_budget_bytes=1 << 20)
    g = G.rmat(14, 16, seed=3)
    with pytest.raises(P.PccError) as e:
        c.upload(g)
    assert e.value.code == 8  # RESOURCE_EXHAUSTED
    c.close()


def test_host_csr_end_to_end(ctx, graphs):
    g = graphs["sbm2k"]
    og = O.OracleGraph(g)
    cfg = P.make_config(resolution=1.0, refine=True, move_method=P.NBHR_MOVE)
    lab_g, _ = P.cluster_host_csr(ctx, g, cfg, objective=1)
    lab_o, _ = O.modularity_cluster(og, cfg)
    np.testing.assert_array_equal(lab_g, lab_o)


def test_clusterer_class_dropin(ctx, graphs):
    g = graphs["sbm2k"]
    og = O.OracleGraph(g)
    cl = P.ParallelModularityClustererGB300(ctx)
    cl.set_graph(g)
    cfg = P.make_config(resolution=1.0, refine=True, move_method=P.NBHR_MOVE)
    clustering = cl.cluster(cfg)
    lab_o, _ = O.modularity_cluster(og, cfg)
    assert clustering == P.labels_to_clustering(lab_o)
    # RefineClusters from that clustering
    refined = cl.refine_clusters(cfg, clustering)
    init = np.empty(g.n, np.uint32)
    for i, grp in enumerate(clustering):
        init[grp] = i
    lab_o2, _ = O.modularity_cluster(og, cfg, initial_labels=init)
    assert refined == P.labels_to_clustering(lab_o2)


@pytest.mark.parametrize("name", ["sbm2k", "rmat14", "sbm3k_int"])
@pytest.mark.parametrize("weights", ["int", "real", "huge"])
def test_best_moves_certified_paths(ctx, graphs, name, weights):
    """INT-mode replays over node weights and resolutions that push the FP32
    certification to both outcomes.  Replay runs the exact FP64 path and
    raises an error if a certified decision disagrees with it; the result
    must equal the oracle bit for bit."""
    g = graphs[name]
    dg, og = _both(ctx, g)
    rng = np.random.default_rng(17)
    if weights == "int":
        k = rng.integers(1, 6, size=g.n).astype(np.float64)
    elif weights == "real":
        k = rng.uniform(0.25, 3.0, size=g.n)
    else:
        k = rng.integers(1, 4, size=g.n).astype(np.float64) * 2.0**26   # K beyond 2^24
    for div in (1, 5, 200):
        C, s, _, K = rand_state(g.n, max(1, g.n // div), seed=div, node_weights=k)
        for res in (0.0, 1e-12, 1e-3, 0.37, 5.0):
            cfg = P.make_config(resolution=res * (2.0**-52 if weights == "huge" else 1.0))
            t_g, v_g, m_g = P.best_moves(dg, cfg, C, s, k, K)
            t_o, v_o, m_o = O.best_moves(og, cfg, C, s, k, K)
            np.testing.assert_array_equal(t_g, t_o)
            np.testing.assert_array_equal(v_g.view(np.uint64), v_o.view(np.uint64))
            np.testing.assert_array_equal(m_g, m_o)


@pytest.mark.parametrize("name,kind,res,move,permute", [
    ("sbm2k", "corr", 0.01, P.NBHR_CLUSTER_MOVE, True),
    ("rmat16", "mod", 1.0, P.NBHR_MOVE, True),
    ("lfr20k_real", "corr", 0.1, P.NBHR_CLUSTER_MOVE, True),
    ("sbm2k", "corr", 0.01, P.NBHR_CLUSTER_MOVE, False),
    ("rmat16", "mod", 1.0, P.NBHR_MOVE, False),
])
def test_async_mean_objective_matches_oracle(ctx, graphs, name, kind, res, move, permute):
    """Async mode is nondeterministic in the reference too (AsyncMove,
    parallel-correlation-clusterer-internal.cc:371-403), so quality is
    compared as a mean over seeds.  The reference's async quality also moves
    with its worker count (the oracle's RMAT-16 mean: 0.09806 on one worker,
    0.0975-0.0978 on 8-16), so the oracle runs on one worker: the reference's
    algorithm without scheduler noise, deterministic per seed.  Permuted
    rounds (vertexMapPermute, parallel-correlation-clusterer.cc:69-109): the
    GPU's mean objective over 20 seeds must lie within 0.5% of the oracle's,
    either way.  Unpermuted rounds: the GPU's hashed waves are not the
    reference's id order, so the GPU mean must not be more than 0.5% worse.
    Every GPU objective is first recomputed by the oracle from the GPU's
    labels."""
    g = graphs[name]
    dg, og = _both(ctx, g)
    gpu, cpu = [], []
    O.set_threads(1)
    for seed in range(ASYNC_SEEDS):
        cfg = P.make_config(resolution=res, refine=True, async_=True, move_method=move, permute=permute,
                            random_seed=seed + 1)
        if kind == "mod":
            lab, sg = P.modularity_cluster(dg, cfg)
            _, so = O.modularity_cluster(og, cfg)
            q = O.modularity(og, res, lab)
            assert q == pytest.approx(sg["modularity"], rel=1e-9, abs=1e-12)
            gpu.append(q)
            cpu.append(so["modularity"])
        else:
            lab, sg = P.correlation_cluster(dg, cfg)
            _, so = O.correlation_cluster(og, cfg)
            q = O.objective(og, cfg, lab)
            assert q == pytest.approx(sg["objective"], rel=1e-9, abs=1e-9)
            gpu.append(q)
            cpu.append(so["objective"])
    O.set_threads(0)
    mg, mc = float(np.mean(gpu)), float(np.mean(cpu))
    info = (name, permute, mg, mc, (mg - mc) / abs(mc), gpu, cpu)
    if permute:
        assert abs(mg - mc) <= ASYNC_WINDOW * abs(mc), info
    else:
        assert mg >= mc - ASYNC_WINDOW * abs(mc), info


@pytest.mark.parametrize("move", [P.NBHR_CLUSTER_MOVE, P.NBHR_MOVE, P.ALL_MOVE])
@pytest.mark.parametrize("refine", [True, False])
def test_device_round_loop_matches_host_loop(graphs, move, refine):
    """Synchronous rounds run as a device-side graph loop by default; with
    detailed timing the host drives every round.  Labels, objective and the
    control-flow counters must be identical (RMAT-16 has hubs above both hub
    thresholds; the real-weight LFR graph takes the FP64 kernels)."""
    c = P.Context(0)
    try:
        for name, kind, res in [("rmat16", "mod", 1.0), ("sbm3k_int", "corr", 0.05), ("lfr20k_real", "corr", 0.1)]:
            dg = c.upload(graphs[name])
            cfg = P.make_config(resolution=res, refine=refine, move_method=move, louvain_num_iterations=6,
                                louvain_num_inner_iterations=5)
            out = []
            for detailed in (False, True):
                c.set_detailed_timing(detailed)
                if kind == "mod":
                    lab, st = P.modularity_cluster(dg, cfg)
                else:
                    lab, st = P.correlation_cluster(dg, cfg)
                out.append((lab, st))
            (l0, s0), (l1, s1) = out
            np.testing.assert_array_equal(l0, l1, err_msg=name)
            for key in ("objective", "modularity", "num_clusters", "levels", "rounds", "refine_passes",
                        "edge_visits", "vertex_visits", "moves", "algo_bytes_best_moves"):
                assert s0[key] == s1[key], (name, key, s0[key], s1[key])
            assert s1["ms_best_moves"] > 0
            dg.free()
    finally:
        c.close()


def test_overlapped_families_match_serial(graphs, monkeypatch):
    """Synchronous rounds launch the best-move families (lane groups, warps,
    small hubs, big hubs) as parallel stream branches; with
    PCC_SERIAL_FAMILIES=1 they run one after another.  Labels and every
    counter must be identical, in the device-side loop and host-driven."""
    c_par = P.Context(0)
    monkeypatch.setenv("PCC_SERIAL_FAMILIES", "1")
    c_ser = P.Context(0)
    monkeypatch.delenv("PCC_SERIAL_FAMILIES")
    try:
        for name, kind, res, move in [("rmat16", "mod", 1.0, P.NBHR_MOVE), ("hubs100k", "corr", 0.05, P.ALL_MOVE),
                                      ("sbm3k_int", "corr", 0.05, P.NBHR_CLUSTER_MOVE),
                                      ("lfr20k_real", "corr", 0.1, P.NBHR_CLUSTER_MOVE)]:
            cfg = P.make_config(resolution=res, refine=True, move_method=move)
            out = []
            for c in (c_par, c_ser):
                dg = c.upload(graphs[name])
                run = P.modularity_cluster if kind == "mod" else P.correlation_cluster
                out.append(run(dg, cfg))
                dg.free()
            (l0, s0), (l1, s1) = out
            np.testing.assert_array_equal(l0, l1, err_msg=name)
            for key in ("objective", "modularity", "num_clusters", "levels", "rounds", "edge_visits", "moves"):
                assert s0[key] == s1[key], (name, key, s0[key], s1[key])
    finally:
        c_par.close()
        c_ser.close()


def test_launch_tuning_keeps_results(ctx, graphs):
    """Every launch shape pcc_set_launch_tuning accepts (lane-group bins
    routed to the warp kernel, certified warp bins on one CTA per vertex,
    0.125-4 waves of CTAs) gives the labels and counters of the compiled-in
    table: INT (certified) and FP64 kernels, synchronous rounds in the device
    loop and host-driven.  Shapes outside the documented range are
    INVALID_ARGUMENT."""
    cases = [("rmat16", "mod", 1.0, P.NBHR_MOVE), ("sbm3k_int", "corr", 0.05, P.NBHR_CLUSTER_MOVE),
             ("lfr20k_real", "corr", 0.1, P.NBHR_CLUSTER_MOVE), ("sbm2k", "corr", 0.05, P.ALL_MOVE),
             ("hubs100k", "corr", 0.05, P.NBHR_MOVE)]
    shapes = [(4, 1000, 1.0), (8, 512, 0.5), (16, 256, 2.0), (32, 128, 0.125), (32, 64, 4.0)]
    keys = ("objective", "modularity", "num_clusters", "levels", "rounds", "edge_visits", "moves")
    try:
        for name, kind, res, move in cases:
            cfg = P.make_config(resolution=res, refine=True, move_method=move, random_seed=3)
            run = P.modularity_cluster if kind == "mod" else P.correlation_cluster
            dg = ctx.upload(graphs[name])
            ctx.set_launch_tuning(0, 0, 0.0)
            l0, s0 = run(dg, cfg)
            for gmax, cta, waves in shapes:
                for detailed in (False, True):
                    ctx.set_launch_tuning(gmax, cta, waves)
                    ctx.set_detailed_timing(detailed)
                    l1, s1 = run(dg, cfg)
                    np.testing.assert_array_equal(l0, l1, err_msg=f"{name} {gmax}/{cta}/{waves}")
                    for key in keys:
                        assert s0[key] == s1[key], (name, gmax, cta, waves, key, s0[key], s1[key])
            dg.free()
        for bad in [(3, 1000, 1.0), (64, 1000, 1.0), (32, 1000, 0.0), (32, 1000, 100.0), (0, 1000, 1.0),
                    (32, 100, 1.0), (32, 0, 1.0)]:
            with pytest.raises(P.PccError) as e:
                ctx.set_launch_tuning(*bad)
            assert e.value.code == 3
    finally:
        ctx.set_launch_tuning(0, 0, 0.0)
        ctx.set_detailed_timing(False)


@pytest.mark.parametrize("name", ["sbm2k", "rmat14", "rmat16", "sbm3k_int", "hubs100k"])
@pytest.mark.parametrize("nclusters_div", [1, 7, 300])
def test_best_moves_replay_cta_kernels(ctx, graphs, name, nclusters_div):
    """The one-CTA-per-vertex certified kernels (every warp bin routed to
    them) against the oracle on one sync pass from a random state: targets,
    values and moves bit-exact.  The replay path also checks each certified
    decision against the exact FP64 one on the device (a mismatch is an
    INTERNAL error)."""
    g = graphs[name]
    dg, og = _both(ctx, g)
    C, s, k, K = rand_state(g.n, g.n // nclusters_div, seed=nclusters_div)
    try:
        ctx.set_launch_tuning(32, 64, 1.0)
        for res, off in ((0.01, 0.0), (0.3, 0.0), (0.05, 1.0)):
            cfg = P.make_config(resolution=res, edge_weight_offset=off)
            t_g, v_g, m_g = P.best_moves(dg, cfg, C, s, k, K)
            t_o, v_o, m_o = O.best_moves(og, cfg, C, s, k, K)
            np.testing.assert_array_equal(t_g, t_o)
            np.testing.assert_array_equal(v_g.view(np.uint64), v_o.view(np.uint64))
            np.testing.assert_array_equal(m_g, m_o)
    finally:
        ctx.set_launch_tuning(0, 0, 0.0)


@pytest.mark.parametrize("name,res,move", [
    ("sbm2k", 0.01, P.NBHR_CLUSTER_MOVE),
    ("lfr20k_real", 0.1, P.NBHR_CLUSTER_MOVE),
])
def test_async_cluster_moves_mean_objective(ctx, graphs, name, res, move):
    """Async whole-cluster moves (DEFAULT_CLUSTER_MOVES with async:
    parallel-correlation-clusterer.cc:255-268, AsyncMove(moving_nodes) at
    parallel-correlation-clusterer-internal.cc:405-446) are nondeterministic
    in the reference; the oracle restates them as every cluster moving in
    turn on live state, with the vertex moves on one worker.  The GPU's mean
    objective over seeds (recomputed by the oracle from the GPU's labels)
    must lie within 0.5% of the oracle's mean, either way."""
    g = graphs[name]
    dg, og = _both(ctx, g)
    gpu, cpu = [], []
    O.set_threads(1)
    for seed in range(ASYNC_SEEDS):
        cfg = P.make_config(resolution=res, async_=True, move_method=move, permute=True, random_seed=seed + 1,
                            clustering_moves_method=P.DEFAULT_CLUSTER_MOVES)
        lab, sg = P.correlation_cluster(dg, cfg)
        q = O.objective(og, cfg, lab)
        assert q == pytest.approx(sg["objective"], rel=1e-9, abs=1e-9)
        _, so = O.correlation_cluster(og, cfg)
        gpu.append(q)
        cpu.append(so["objective"])
    O.set_threads(0)
    mg, mc = float(np.mean(gpu)), float(np.mean(cpu))
    assert abs(mg - mc) <= ASYNC_WINDOW * abs(mc), (name, mg, mc, (mg - mc) / abs(mc), gpu, cpu)


@pytest.mark.parametrize("method", [1, 2, 3])  # TRIANGLE, CONNECTIVITY, SLOW_CONNECTIVITY
@pytest.mark.parametrize("name,kind,res", [("sbm2k", "corr", 0.05), ("rmat14", "mod", 1.0), ("sbm3k_int", "corr", 0.1),
                                           ("lfr20k_real", "corr", 0.1)])
@pytest.mark.parametrize("refine", [True, False])
def test_subclustering_matches_oracle(ctx, graphs, method, name, kind, res, refine):
    """Subclustering before compression (CompressSubclusters,
    parallel-correlation-clusterer.cc:436-474; ComputeSubcluster and its
    methods, parallel-correlation-clusterer-internal.cc:784-1120): labels,
    levels, rounds and edge visits bit-exact against the oracle on integer
    weights; the objective within 1e-9 on real weights (FP64 mode)."""
    g = graphs[name]
    dg, og = _both(ctx, g)
    cfg = P.make_config(resolution=res, refine=refine, subclustering_method=method, move_method=P.NBHR_MOVE,
                        louvain_num_iterations=4)
    run_g = P.modularity_cluster if kind == "mod" else P.correlation_cluster
    run_o = O.modularity_cluster if kind == "mod" else O.correlation_cluster
    lab_g, st_g = run_g(dg, cfg)
    lab_o, st_o = run_o(og, cfg)
    if g.weights is None or name == "sbm3k_int":
        np.testing.assert_array_equal(lab_g, lab_o)
        for key in ("levels", "rounds", "refine_passes", "edge_visits", "num_clusters"):
            assert st_g[key] == st_o[key], (key, st_g[key], st_o[key])
    assert st_g["objective"] == pytest.approx(st_o["objective"], rel=REL_TOL, abs=1e-9)
