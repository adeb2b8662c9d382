"""GPU tests of batched clustering and the serving loop: every result equals
the standalone call on the same graph, under concurrency, queueing and an
HBM budget."""

import numpy as np
import pytest

import oracle as O
import pcc_gb300 as P
import pcc_graphs as G

pytestmark = pytest.mark.gpu


def _single(ctx, g, cfg, objective, k=None):
    return P.cluster_host_csr(ctx, g, cfg, objective=objective, node_weights=k)


@pytest.fixture(scope="module")
def small_graphs(built):
    return G.batch_sbm_graphs(40, seed=3, n_lo=200, n_hi=4000)


UNION_STATS = ("objective", "num_clusters", "levels", "rounds", "refine_passes", "edge_visits")


def test_batch_matches_single_calls(ctx, small_graphs):
    """One shared correlation config: the batch runs as a disjoint union;
    labels, objective and the per-graph control-flow counters equal the
    standalone call's."""
    cfg = P.make_config(resolution=0.05, refine=True)
    labels, stats, wall = P.cluster_batch(small_graphs, cfg, concurrency=8)
    assert wall > 0
    for g, lab, st in zip(small_graphs, labels, stats):
        ref, rst = _single(ctx, g, cfg, 0)
        np.testing.assert_array_equal(lab, ref)
        for key in UNION_STATS:
            assert st[key] == rst[key], key


def test_pool_batch_matches_single_calls(ctx, small_graphs):
    """Per-graph configs run on the worker pool: labels, objective and the
    control-flow counters of the standalone call are reproduced (launch
    counts differ: pool workers drive small graphs' rounds from the host,
    a plain context runs them as a device-side loop)."""
    # Configs that differ in more than the resolution cannot share a union.
    cfgs = [P.make_config(resolution=0.05, refine=True, move_method=P.NBHR_MOVE if i % 2 else P.NBHR_CLUSTER_MOVE)
            for i in range(16)]
    graphs = small_graphs[:16]
    labels, stats, wall = P.cluster_batch(graphs, cfgs, concurrency=8)
    assert wall > 0
    for g, lab, st, cfg in zip(graphs, labels, stats, cfgs):
        ref, rst = _single(ctx, g, cfg, 0)
        np.testing.assert_array_equal(lab, ref)
        assert st["objective"] == rst["objective"]
        for key in ("edge_visits", "vertex_visits", "rounds", "levels", "moves", "num_clusters"):
            assert st[key] == rst[key], key


def _union_mix():
    """SBMs, an RMAT graph with hubs above both hub thresholds, a graph with
    isolated vertices, an edgeless graph, an empty graph and a triangle."""
    out = list(G.batch_sbm_graphs(6, seed=21, n_lo=200, n_hi=3000))
    out.insert(2, G.rmat(13, 16, seed=5))
    rng = np.random.default_rng(4)
    src = rng.integers(0, 300, 900)
    dst = rng.integers(0, 300, 900)
    out.insert(4, P.CsrGraph.from_edges(500, src, dst, drop_self_loops=True))   # ids 300-499 isolated
    out.append(P.CsrGraph(np.zeros(41, np.uint64), np.zeros(0, np.uint32)))      # 40 vertices, no edges
    out.insert(1, P.CsrGraph(np.zeros(1, np.uint64), np.zeros(0, np.uint32)))    # n = 0
    out.append(P.CsrGraph.from_edges(3, [0, 1, 2], [1, 2, 0]))
    return out


@pytest.mark.parametrize("move", [P.NBHR_CLUSTER_MOVE, P.NBHR_MOVE, P.ALL_MOVE])
@pytest.mark.parametrize("refine", [True, False])
def test_union_matches_single_every_control_path(ctx, move, refine):
    """Graphs stop their levels, inner loops and refinement at different
    points; each must follow its own standalone control flow.  Small
    iteration caps make the caps bind; a small entry cap splits the batch
    into several unions."""
    graphs = _union_mix()
    for iters, inner, cap in [(0, 0, 0), (3, 2, 0), (4, 10, 200_000)]:
        cfg = P.make_config(resolution=0.05, refine=refine, move_method=move,
                            louvain_num_iterations=iters, louvain_num_inner_iterations=inner)
        labels, stats, tot = P.cluster_union(ctx, graphs, cfg, max_union_entries=cap)
        assert tot["kernel_launches"] > 0
        for i, g in enumerate(graphs):
            if g.n == 0:
                assert len(labels[i]) == 0 and stats[i]["num_clusters"] == 0
                continue
            ref, rst = _single(ctx, g, cfg, 0)
            np.testing.assert_array_equal(labels[i], ref, err_msg=f"graph {i} iters {iters}")
            for key in UNION_STATS:
                assert stats[i][key] == rst[key], (i, key, iters)


@pytest.mark.parametrize("move", [P.NBHR_CLUSTER_MOVE, P.NBHR_MOVE, P.ALL_MOVE])
def test_union_device_loop_matches_host_loop(ctx, move):
    """Union rounds run as the device-side loop (per-graph rounds, edge
    visits and in-loop flags kept on the device) and, with detailed timing,
    driven from the host: labels and every per-graph counter agree."""
    graphs = _union_mix()
    cfg = P.make_config(resolution=0.05, refine=True, move_method=move,
                        louvain_num_iterations=4, louvain_num_inner_iterations=3)
    lab_d, st_d, tot_d = P.cluster_union(ctx, graphs, cfg)
    ctx.set_detailed_timing(True)
    try:
        lab_h, st_h, tot_h = P.cluster_union(ctx, graphs, cfg)
    finally:
        ctx.set_detailed_timing(False)
    for i in range(len(graphs)):
        np.testing.assert_array_equal(lab_d[i], lab_h[i], err_msg=f"graph {i}")
        for key in UNION_STATS:
            assert st_d[i][key] == st_h[i][key], (i, key)
    for key in ("edge_visits", "vertex_visits", "moves", "rounds", "levels"):
        assert tot_d[key] == tot_h[key], key


@pytest.mark.parametrize("move", [P.NBHR_CLUSTER_MOVE, P.ALL_MOVE])
def test_union_mixed_resolutions_and_objectives(ctx, small_graphs, move):
    """Graphs with their own resolutions and objectives in one union: every
    vertex reads its graph's resolution (modularity: resolution / sum of
    degrees, degree node weights).  Labels and objective are bit-identical to
    standalone calls (integer sums); modularity within 1e-12."""
    rng = np.random.default_rng(12)
    graphs = small_graphs[:14] + [G.rmat(12, 16, seed=3)]
    cfgs = [P.make_config(resolution=float(rng.choice([0.01, 0.1, 0.5])), refine=True, move_method=move)
            for _ in graphs]
    objs = np.array([i % 2 for i in range(len(graphs))], dtype=np.int32)
    labels, stats, _ = P.cluster_union(ctx, graphs, cfgs, objectives=objs)
    for i, g in enumerate(graphs):
        ref, rst = _single(ctx, g, cfgs[i], int(objs[i]))
        np.testing.assert_array_equal(labels[i], ref, err_msg=f"graph {i}")
        assert stats[i]["objective"] == rst["objective"]
        assert stats[i]["rounds"] == rst["rounds"] and stats[i]["levels"] == rst["levels"]
        if objs[i] == 1:
            assert stats[i]["modularity"] == pytest.approx(rst["modularity"], rel=1e-12, abs=1e-15)
    # The batch call routes such a batch to the union as well.
    labels2, stats2, _ = P.cluster_batch(graphs, cfgs, objectives=objs)
    for a, b in zip(labels, labels2):
        np.testing.assert_array_equal(a, b)


def test_union_matches_oracle_on_batch_distribution(ctx, small_graphs):
    """Two graphs of the batched SBM distribution with 20k-50k vertices, in
    one union with small graphs, at resolution 0.05 with refinement: labels
    and statistics bit-identical to the oracle's sequential clustering."""
    big = G.batch_sbm_graphs(2, seed=21, n_lo=20000, n_hi=50000)
    assert all(20000 <= g.n <= 50000 for g in big)
    graphs = [small_graphs[0], big[0], small_graphs[1], big[1]]
    cfg = P.make_config(resolution=0.05, refine=True)
    labels, stats, _ = P.cluster_union(ctx, graphs, cfg)
    for i in (1, 3):
        lab_o, st_o = O.correlation_cluster(O.OracleGraph(graphs[i]), cfg)
        np.testing.assert_array_equal(labels[i], lab_o)
        for key in ("num_clusters", "rounds", "levels", "edge_visits"):
            assert stats[i][key] == st_o[key], key
        assert stats[i]["objective"] == pytest.approx(st_o["objective"], rel=1e-12, abs=1e-9)


def test_union_node_weights_and_real_weights(ctx, small_graphs):
    """Integer node weights keep every sum exact (bit-identical objective);
    real edge weights take the FP64 path (labels identical, objective within
    FP64 summation order)."""
    graphs = small_graphs[:10]
    cfg = P.make_config(resolution=0.05, refine=True)
    kw = [None if i % 2 else (np.arange(g.n) % 4 + 1.0) for i, g in enumerate(graphs)]
    labels, stats, _ = P.cluster_union(ctx, graphs, cfg, node_weights=kw)
    for i, g in enumerate(graphs):
        ref, rst = P.cluster_host_csr(ctx, g, cfg, objective=0, node_weights=kw[i])
        np.testing.assert_array_equal(labels[i], ref)
        assert stats[i]["objective"] == rst["objective"]
    rng = np.random.default_rng(8)
    real = []
    for g in graphs[:6]:
        d = np.repeat(np.arange(g.n), np.diff(g.offsets).astype(np.int64))
        src, dst = d[d < g.neighbors], g.neighbors[d < g.neighbors]
        real.append(P.CsrGraph.from_edges(g.n, src, dst, rng.uniform(0.5, 1.5, len(src))))
    cfg = P.make_config(resolution=0.1, refine=True, move_method=P.NBHR_CLUSTER_MOVE)
    labels, stats, _ = P.cluster_union(ctx, real, cfg)
    for i, g in enumerate(real):
        ref, rst = _single(ctx, g, cfg, 0)
        np.testing.assert_array_equal(labels[i], ref)
        assert stats[i]["objective"] == pytest.approx(rst["objective"], rel=1e-12, abs=1e-9)


def test_union_rejects_bad_input(ctx):
    good = P.CsrGraph.from_edges(3, [0, 1], [1, 2])
    bad = P.CsrGraph(np.array([0, 1, 2], np.uint64), np.array([1, 2], np.uint32))   # neighbour 2 >= n
    with pytest.raises(P.PccError) as e:
        P.cluster_union(ctx, [good, bad], P.make_config(resolution=0.1))
    assert e.value.code == 3
    with pytest.raises(P.PccError) as e:
        P.cluster_union(ctx, [good], P.make_config(resolution=0.1, async_=True))
    assert e.value.code == 3


def test_batch_mixed_configs_and_objectives(ctx, small_graphs):
    rng = np.random.default_rng(5)
    graphs = small_graphs[:24]
    cfgs = [P.make_config(resolution=float(rng.choice([0.01, 0.1, 0.5])), refine=bool(i % 2),
                          move_method=int(rng.integers(0, 3))) for i in range(len(graphs))]
    objs = rng.integers(0, 2, size=len(graphs)).astype(np.int32)
    weights = [None if i % 3 else np.arange(g.n) % 3 + 1.0 for i, g in enumerate(graphs)]
    labels, stats, _ = P.cluster_batch(graphs, cfgs, objectives=objs, node_weights=weights, concurrency=5)
    for i, g in enumerate(graphs):
        ref, rst = _single(ctx, g, cfgs[i], int(objs[i]), None if objs[i] == 1 else weights[i])
        np.testing.assert_array_equal(labels[i], ref)
        assert stats[i]["modularity"] == rst["modularity"] and stats[i]["objective"] == rst["objective"]


def test_server_results_alone_and_in_the_mix(ctx, small_graphs):
    reqs = G.serving_requests(30, seed=9, rmat_scale=13, n_hi=4000)
    est = max(P.request_bytes_estimate(r["graph"].n, r["graph"].m, False) for r in reqs)
    srv = P.Server(slots=6, hbm_budget=int(est * 2.5))   # admission limits concurrency to ~2
    try:
        tickets = []
        for r in reqs:
            cfg = P.make_config(resolution=r["resolution"], refine=True, move_method=P.NBHR_MOVE)
            tickets.append((srv.submit(r["graph"], cfg, r["objective"]), cfg, r))
        queued = 0
        for t, cfg, r in tickets:
            lab, st, lat, qms = srv.wait(t)
            assert lat >= qms >= 0
            queued += qms > 0
            ref, rst = _single(ctx, r["graph"], cfg, r["objective"])
            np.testing.assert_array_equal(lab, ref)
            assert st["objective"] == rst["objective"]
        assert queued > 0      # the budget made requests wait for admission
    finally:
        srv.close()


def test_server_groups_queued_requests_into_unions(ctx, small_graphs):
    """One worker slot and a burst of same-config correlation requests: the
    queued ones are admitted together as a union run (their stats carry no
    launch count), and every result equals the standalone call."""
    cfg = P.make_config(resolution=0.05, refine=True)
    other = P.make_config(resolution=0.1, refine=True)
    srv = P.Server(slots=1, hbm_budget=0)
    try:
        tickets = []
        for i, g in enumerate(small_graphs[:20]):
            c, obj = (other, 1) if i % 5 == 4 else (cfg, 0)
            tickets.append((srv.submit(g, c, obj), g, c, obj))
        grouped = 0
        for t, g, c, obj in tickets:
            lab, st, _, _ = srv.wait(t)
            ref, rst = _single(ctx, g, c, obj)
            np.testing.assert_array_equal(lab, ref)
            assert st["objective"] == rst["objective"]
            grouped += obj == 0 and st["kernel_launches"] == 0 and st["rounds"] == rst["rounds"]
        assert grouped > 1
    finally:
        srv.close()


def test_server_rejects_request_over_budget(built, small_graphs):
    srv = P.Server(slots=2, hbm_budget=1 << 20)
    try:
        with pytest.raises(P.PccError) as e:
            srv.submit(small_graphs[0], P.make_config(resolution=0.1), 0)
        assert e.value.code == 8
    finally:
        srv.close()


@pytest.mark.parametrize("kind", ["sbm", "rmat", "lfr"])
def test_request_estimate_bounds_peak(built, kind):
    if kind == "sbm":
        g, _ = G.sbm(20000, 40, 0.02, 0.0004, 4)
    elif kind == "rmat":
        g = G.rmat(16, 16, seed=2)
    else:
        g, _ = G.lfr(30000, mean_degree=20, dmax=1500, seed=6)
    c = P.Context(0)
    try:
        c.lib.pcc_device_peak_bytes(c.handle, 1)
        cfg = P.make_config(resolution=0.1, refine=True)
        P.cluster_host_csr(c, g, cfg, objective=1 if kind == "rmat" else 0)
        peak = c.lib.pcc_device_peak_bytes(c.handle, 0)
    finally:
        c.close()
    assert 0 < peak <= P.request_bytes_estimate(g.n, g.m, g.weights is not None)
