"""CPU tests of the oracle (the C++ restatement of the reference path).

The oracle is pinned by
  * golden clusterings from an independent pure-Python restatement
    (tests/golden/make_golden.py, fixtures in golden_clusterings.json);
  * the objective's definition (clustering/config.proto:66-93), enumerated
    by brute force on tiny graphs;
  * the move-delta identity: a best move's value equals the objective after
    the move minus the objective before it;
  * hand-derived answers on known graphs.
"""

import itertools
import json
import os
import sys

import numpy as np
import pytest

import oracle as O
import pcc_gb300 as P
import pcc_graphs as G

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden as MG  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    O.set_threads(4)
    yield


def _csr(n, edges, weights=None):
    src = [a for a, b in edges]
    dst = [b for a, b in edges]
    return P.CsrGraph.from_edges(n, src, dst, weights)


def _cfg(d):
    return P.make_config(resolution=d["resolution"], edge_weight_offset=d.get("edge_weight_offset", 0.0),
                         refine=d.get("refine", False), move_method=d.get("move_method", 0),
                         louvain_num_iterations=d.get("louvain_num_iterations", 0),
                         louvain_num_inner_iterations=d.get("louvain_num_inner_iterations", 0),
                         clustering_moves_method=d.get("clustering_moves_method", P.LOUVAIN),
                         num_iterations=d.get("num_iterations", 0))


with open(os.path.join(HERE, "golden", "golden_clusterings.json")) as _f:
    GOLDEN = json.load(_f)


@pytest.mark.parametrize("fx", GOLDEN, ids=[f"{g['graph']}-{i % 10}" for i, g in enumerate(GOLDEN)])
def test_oracle_matches_golden(fx):
    g = _csr(fx["n"], fx["edges"], fx["weights"])
    og = O.OracleGraph(g)
    cfg = _cfg(fx["config"])
    if fx["config"]["kind"] == "modularity":
        lab, st = O.modularity_cluster(og, cfg)
    else:
        lab, st = O.correlation_cluster(og, cfg)
    assert lab.tolist() == fx["labels"]
    assert st["edge_visits"] == fx["edge_visits"]
    assert st["rounds"] == fx["rounds"]
    assert st["objective"] == pytest.approx(fx["objective"], rel=1e-12, abs=1e-12)


def _objective_by_definition(n, edges, weights, labels, k, res, off):
    """sum over unordered same-cluster pairs of w'_uv (config.proto:66-93)."""
    w = {}
    for i, (a, b) in enumerate(edges):
        w[(min(a, b), max(a, b))] = weights[i] if weights is not None else 1.0
    tot = 0.0
    for u, v in itertools.combinations(range(n), 2):
        if labels[u] != labels[v]:
            continue
        if (u, v) in w:
            tot += w[(u, v)] - off - res * k[u] * k[v]
        else:
            tot += -res * k[u] * k[v]
    return tot


@pytest.mark.parametrize("seed", range(6))
def test_objective_brute_force(seed):
    rng = np.random.default_rng(seed)
    n = 8
    edges = [(a, b) for a, b in itertools.combinations(range(n), 2) if rng.random() < 0.4]
    weights = [float(x) for x in rng.integers(1, 4, size=len(edges))]
    g = _csr(n, edges, weights)
    og = O.OracleGraph(g)
    k = rng.integers(1, 3, size=n).astype(np.float64)
    for _ in range(10):
        labels = rng.integers(0, 4, size=n).astype(np.uint32)
        for res, off in ((0.1, 0.0), (0.5, 0.25)):
            cfg = P.make_config(resolution=res, edge_weight_offset=off)
            got = O.objective(og, cfg, labels, k)
            want = _objective_by_definition(n, edges, weights, labels, k, res, off)
            assert got == pytest.approx(want, abs=1e-9)


def test_best_clustering_brute_force():
    """On a tiny graph the local search reaches the brute-force optimum."""
    edges = [(0, 1), (1, 2), (0, 2), (3, 4), (4, 5), (3, 5), (2, 3)]
    n = 6
    g = _csr(n, edges)
    og = O.OracleGraph(g)
    res = 0.3
    cfg = P.make_config(resolution=res, refine=False, move_method=P.ALL_MOVE)
    lab, st = O.correlation_cluster(og, cfg)
    best = max(_objective_by_definition(n, edges, None, labels, [1.0] * n, res, 0.0)
               for labels in itertools.product(range(3), repeat=n))
    assert st["objective"] == pytest.approx(best)
    assert len(set(lab.tolist())) == 2


@pytest.mark.parametrize("seed", range(4))
def test_move_delta_identity(seed):
    """EfficientBestMove's value for the chosen cluster equals the objective
    change of that single move, computed from scratch."""
    rng = np.random.default_rng(seed)
    n = 40
    edges = [(a, b) for a, b in itertools.combinations(range(n), 2) if rng.random() < 0.15]
    weights = [float(x) for x in rng.integers(1, 4, size=len(edges))]
    g = _csr(n, edges, weights)
    og = O.OracleGraph(g)
    C = rng.integers(0, 8, size=n).astype(np.uint32)
    k = rng.integers(1, 3, size=n).astype(np.float64)
    s = np.bincount(C, minlength=n).astype(np.uint32)
    K = np.bincount(C, weights=k, minlength=n)
    res = 0.05
    cfg = P.make_config(resolution=res)
    t, v, _ = O.best_moves(og, cfg, C, s, k, K)
    base = O.objective(og, cfg, C, k)
    free = [c for c in range(n) if s[c] == 0]
    checked = 0
    for u in range(n):
        if t[u] == C[u]:
            # Own cluster: its value carries the -res * k_v^2 bias of the
            # reference's formula (K_C includes k_v), so the identity is for
            # D != C(v) only.
            assert v[u] == pytest.approx(-res * k[u] * k[u], abs=1e-9)
            continue
        checked += 1
        C2 = C.copy()
        C2[u] = free[0] if t[u] == n else t[u]
        delta = O.objective(og, cfg, C2, k) - base
        assert v[u] == pytest.approx(delta, abs=1e-9)


def test_known_answers():
    # Two disjoint 5-cliques: two clusters at small resolution.
    e = [(a, b) for a in range(5) for b in range(a + 1, 5)] + [(a, b) for a in range(5, 10) for b in range(a + 1, 10)]
    og = O.OracleGraph(_csr(10, e))
    lab, _ = O.correlation_cluster(og, P.make_config(resolution=0.1, move_method=P.ALL_MOVE))
    assert lab.tolist() == [0] * 5 + [1] * 5
    # refine with one level only: the reference returns singletons (the
    # refinement block needs iter > 0).
    lab, st = O.correlation_cluster(og, P.make_config(resolution=0.1, refine=True, move_method=P.ALL_MOVE,
                                                      louvain_num_iterations=1))
    assert lab.tolist() == list(range(10))
    # a path at a high resolution stays singletons
    og = O.OracleGraph(_csr(6, [(i, i + 1) for i in range(5)]))
    lab, _ = O.correlation_cluster(og, P.make_config(resolution=2.0, move_method=P.ALL_MOVE))
    assert lab.tolist() == list(range(6))


@pytest.mark.parametrize("seed", range(3))
def test_compress_matches_pure_python(seed):
    rng = np.random.default_rng(seed)
    n = 200
    edges = [(a, b) for a, b in itertools.combinations(range(n), 2) if rng.random() < 0.05]
    weights = [float(x) for x in rng.uniform(0.5, 1.5, size=len(edges))]
    g = _csr(n, edges, weights)
    og = O.OracleGraph(g)
    C = rng.integers(0, 30, size=n).astype(np.uint32)
    k = rng.integers(1, 4, size=n).astype(np.float64)
    got, got_k = O.compress(og, C, k)
    pg = MG.from_edges(n, edges, weights)
    want, want_k = MG.compress(pg, C.tolist(), k.tolist())
    assert got.n == want.n
    for u in range(want.n):
        row = [(int(got.neighbors[j]), float(got.weights[j])) for j in range(int(got.offsets[u]), int(got.offsets[u + 1]))]
        assert row == [(a, float(np.float32(b))) for a, b in want.adj[u]]
    np.testing.assert_array_equal(got_k, np.array(want_k))


def test_move_nodes_new_cluster_ids():
    """MoveNodesToCluster: new clusters take the ascending empty ids in
    ascending node order (parallel-correlation-clusterer-internal.cc:339-366)."""
    n = 6
    C = np.array([0, 0, 0, 3, 3, 5], np.uint32)
    s = np.bincount(C, minlength=n).astype(np.uint32)
    k = np.ones(n)
    K = s.astype(np.float64)
    moves = np.full(n, 0xFFFFFFFF, np.uint32)
    moves[2] = n      # 2 -> new cluster
    moves[4] = n      # 4 -> new cluster
    moves[5] = 0      # 5 joins cluster 0 (5 becomes empty)
    C2, s2, K2, mod = O.move_nodes(C, s, k, K, moves)
    # empty ids after leaves/joins: 1, 2, 4, 5 -> node 2 gets 1, node 4 gets 2
    assert C2.tolist() == [0, 0, 1, 3, 2, 0]
    assert s2.tolist() == [3, 1, 1, 1, 0, 0]
    assert mod.tolist() == [1, 1, 1, 1, 0, 1]


def test_oracle_async_cluster_moves():
    """Async whole-cluster moves: two triangles joined by an edge end as the
    two triangles (the vertex moves form them; no whole-cluster move pays)."""
    g = _csr(6, [(0, 1), (1, 2), (0, 2), (3, 4), (4, 5), (3, 5), (2, 3)])
    og = O.OracleGraph(g)
    for seed in range(3):
        cfg = P.make_config(resolution=0.3, clustering_moves_method=P.DEFAULT_CLUSTER_MOVES, async_=True,
                            random_seed=seed + 1)
        lab, st = O.correlation_cluster(og, cfg)
        assert lab[0] == lab[1] == lab[2] and lab[3] == lab[4] == lab[5] and lab[0] != lab[3], lab


def _blocked_sum(xs):
    """pbbs::reduce_add order: serial fold of <= 1024 items, else folds of
    1024-item blocks and the same reduce over the block sums."""
    if not xs:
        return 0.0
    if len(xs) <= 1024:
        r = xs[0]
        for x in xs[1:]:
            r += x
        return r
    return _blocked_sum([_blocked_sum(xs[i:i + 1024]) for i in range(0, len(xs), 1024)])


def _compare_brute(labels, communities):
    """CompareCommunities (cluster-in-memory_main.cc:172-225) by definition:
    intersections as Python sets, first largest in cluster order."""
    clusters = {}
    for v, c in enumerate(labels):
        clusters.setdefault(int(c), set()).add(v)
    order = [clusters[c] for c in sorted(clusters)]
    prec, rec = [], []
    for comm in communities:
        cs = set(int(v) for v in comm)
        best, idx = 0, 0
        for i, cl in enumerate(order):
            k = len(cl & cs)
            if k > best:
                best, idx = k, i
        prec.append(best / len(order[idx]) if order else 0.0)
        rec.append(best / len(comm) if len(comm) else 0.0)
    nc = len(communities)
    sizes = [len(c) for c in order]
    return ({"avg_precision": _blocked_sum(prec) / nc if nc else float("nan"),
             "avg_recall": _blocked_sum(rec) / nc if nc else float("nan"),
             "num_clusters": len(order), "min_size": min(sizes) if sizes else 0xFFFFFFFF,
             "max_size": max(sizes) if sizes else 0,
             "avg_size": sum(sizes) / len(sizes) if sizes else float("nan")}, prec, rec)


def community_cases():
    """Seeded (labels, communities) cases: repeated members, ids no cluster
    holds, empty communities, labels that are not dense, ties, and more
    than 1024 communities (the blocked reduce)."""
    rng = np.random.default_rng(11)
    out = []
    for n, k, nc in ((40, 7, 9), (300, 25, 40), (2000, 300, 2500)):
        labels = rng.choice(rng.permutation(n)[:k], size=n)            # sparse label values
        comms = []
        for j in range(nc):
            size = int(rng.integers(0, 12))
            c = rng.integers(0, n + 5, size=size).tolist()             # ids >= n too
            if size and rng.random() < 0.3:
                c += c[:2]                                              # repeats
            comms.append(c)
        comms.append([])
        out.append((labels.astype(np.uint32), comms))
    return out


@pytest.mark.parametrize("ci", range(3))
def test_oracle_compare_communities_brute_force(ci):
    labels, comms = community_cases()[ci]
    got, gp, gr = O.compare_communities(labels, comms)
    want, wp, wr = _compare_brute(labels, comms)
    assert gp.tolist() == wp and gr.tolist() == wr
    for key, val in want.items():
        assert got[key] == val, key


def _py_subclusters(g, C, method, res, offset):
    """Independent restatement of ComputeSubcluster over every cluster
    (parallel-correlation-clusterer-internal.cc:784-1120, with components
    labelled by their smallest member's local index): (ids, block starts)."""
    off = g.offsets.astype(np.int64)
    nbr = g.neighbors.astype(np.int64)
    rows = [set(nbr[off[v]:off[v + 1]].tolist()) for v in range(g.n)]
    clusters = sorted(set(int(c) for c in C))
    members = {c: [v for v in range(g.n) if C[v] == c] for c in clusters}
    blocks, labels = [], {}
    for c in clusters:
        mem = members[c]
        local = {v: x for x, v in enumerate(mem)}
        if method in (1, 2):
            parent = list(range(len(mem)))

            def find(x):
                while parent[x] != x:
                    x = parent[x]
                return x
            for x, v in enumerate(mem):
                for j in range(off[v], off[v + 1]):
                    u = int(nbr[j])
                    if C[u] != c:
                        continue
                    if method == 1:
                        ratio = len(rows[v] & rows[u]) / float(len(rows[v]) + len(rows[u]))
                        if not ratio > 0.25:
                            continue
                    a, b = find(x), find(local[u])
                    if a != b:
                        parent[max(a, b)] = min(a, b)
            lab = [find(x) for x in range(len(mem))]
            block = len(mem) if method == 2 else max(lab) + 1
        else:
            size = len(mem)
            tmp = list(range(size))
            single = [0] * size
            outside = lambda u: C[u] != c  # noqa: E731
            for i in range(size):
                if single[i]:
                    continue
                cv = mem[i]
                if sum(1 for u in nbr[off[cv]:off[cv + 1]] if outside(int(u))) < size - 1:
                    continue
                groups = {}
                for x, t in enumerate(tmp):
                    groups.setdefault(t, []).append(x)
                glist = [groups[t] for t in sorted(groups)]
                valid = []
                for curr in glist:
                    if curr[0] == i:
                        valid.append(False)
                        continue
                    ne = sum(1 for x in curr for u in nbr[off[mem[x]]:off[mem[x] + 1]] if outside(int(u)))
                    valid.append(ne >= len(curr) * (size - len(curr)))
                if not any(valid):
                    continue
                best, idx, any_left = 0.0, 0, False
                for j, curr in enumerate(glist):
                    if not valid[j]:
                        continue
                    cs = set(mem[x] for x in curr)
                    weight = float(sum(1 for u in nbr[off[cv]:off[cv + 1]] if int(u) in cs))
                    o = offset * len(curr) + res * len(curr)
                    if weight < o:
                        continue
                    any_left = True
                    if weight - o >= best:
                        best, idx = weight - o, j
                if not any_left:
                    continue
                tmp[i] = tmp[glist[idx][0]]
                single[i] = 1
                single[glist[idx][0]] = 1
            lab = tmp
            block = max(lab) + 1
        blocks.append(block)
        labels[c] = lab
    nxt = np.zeros(len(clusters) + 1, np.uint64)
    nxt[1:] = np.cumsum(blocks)
    ids = np.zeros(g.n, np.uint32)
    for gi, c in enumerate(clusters):
        for x, v in enumerate(members[c]):
            ids[v] = nxt[gi] + labels[c][x]
    return ids, nxt


@pytest.mark.parametrize("method", [1, 2, 3])
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_subclusters_match_pure_python(method, seed):
    """Subcluster ids (triangle, connectivity, slow connectivity) of the
    oracle against an independent Python restatement, on SBM graphs with
    random coarse clusterings (so clusters hold several components)."""
    rng = np.random.default_rng(seed)
    g, blocks = G.sbm(120, 6, 0.25, 0.02, seed)
    C = np.where(rng.random(g.n) < 0.8, blocks, rng.integers(0, 6, g.n)).astype(np.uint32) * 3
    og = O.OracleGraph(g)
    res = [0.0, 0.5, 2.0][seed - 1]
    ids, nxt = O.subclusters(og, C, method, res, 0.0)
    want_ids, want_next = _py_subclusters(g, C, method, res, 0.0)
    np.testing.assert_array_equal(nxt, want_next)
    np.testing.assert_array_equal(ids, want_ids)


def test_subclusters_known_answers():
    """Two 4-cliques joined by one edge, all in one cluster: connectivity
    keeps one component (block of 8); the triangle filter keeps the clique
    edges (ratio 2/6 or 2/7 > 0.25) and cuts the bridge (0/8), giving the two
    cliques labelled 0 and 4 (block 5).  Two triangles joined by an edge
    have clique-edge ratios of exactly 1/4, which does not pass."""
    k4 = [(a, b) for a in range(4) for b in range(a + 1, 4)]
    g = _csr(8, k4 + [(a + 4, b + 4) for a, b in k4] + [(3, 4)])
    og = O.OracleGraph(g)
    C = np.zeros(8, np.uint32)
    ids, nxt = O.subclusters(og, C, 2)
    assert ids.tolist() == [0] * 8 and nxt.tolist() == [0, 8]
    ids, nxt = O.subclusters(og, C, 1)
    assert ids.tolist() == [0, 0, 0, 0, 4, 4, 4, 4] and nxt.tolist() == [0, 5]
    t = _csr(6, [(0, 1), (1, 2), (0, 2), (3, 4), (4, 5), (3, 5), (2, 3)])
    ids, nxt = O.subclusters(O.OracleGraph(t), np.zeros(6, np.uint32), 1)
    assert ids.tolist() == [0, 1, 2, 3, 4, 5] and nxt.tolist() == [0, 6]
    # Two clusters, one of them disconnected: components inside each cluster
    # (cluster 5 = {0, 1, 5}: {0, 1} and {5}; cluster 9 = {2, 3, 4} joined
    # through 2-3 and 3-4).
    C2 = np.array([5, 5, 9, 9, 9, 5], np.uint32)
    ids, nxt = O.subclusters(O.OracleGraph(t), C2, 2)
    assert nxt.tolist() == [0, 3, 6]
    assert ids.tolist() == [0, 0, 3, 3, 3, 2]
