"""GPU tests of batched clustering and the serving loop: every result equals
the standalone call on the same graph, under concurrency, queueing and an
HBM budget."""

import numpy as np
import pytest

import pcc_gb300 as P
import pcc_graphs as G

pytestmark = pytest.mark.gpu


def _single(ctx, g, cfg, objective, k=None):
    return P.cluster_host_csr(ctx, g, cfg, objective=objective, node_weights=k)


@pytest.fixture(scope="module")
def small_graphs(built):
    return G.batch_sbm_graphs(40, seed=3, n_lo=200, n_hi=4000)


def test_batch_matches_single_calls(ctx, small_graphs):
    cfg = P.make_config(resolution=0.05, refine=True)
    labels, stats, wall = P.cluster_batch(small_graphs, cfg, concurrency=8)
    assert wall > 0
    for g, lab, st in zip(small_graphs, labels, stats):
        ref, rst = _single(ctx, g, cfg, 0)
        np.testing.assert_array_equal(lab, ref)
        assert st["objective"] == rst["objective"]
        assert st["edge_visits"] == rst["edge_visits"] and st["rounds"] == rst["rounds"]
        assert st["kernel_launches"] == rst["kernel_launches"]


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
