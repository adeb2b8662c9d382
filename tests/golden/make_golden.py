"""Generates tests/golden/*.json: golden clusterings of small graphs.

An independent pure-Python restatement of the reference's parallel
correlation / modularity clustering path (loops over dicts and sorted lists,
no shared code with oracle/pcc_oracle.cc), written from:
  parallel-correlation-clusterer.cc:115-365, 476-653   (rounds, levels, refine,
                                                        whole-cluster moves)
  parallel-correlation-clusterer-internal.cc:50-149, 256-369, 448-583, 644-782
  correlation-clusterer-util.h:26-113
  parallel/parallel-graph-utils.cc:33-243, parallel-sequence-ops.h:161-209
  parallel-modularity-clusterer.cc:36-111
The fixtures pin the C++ oracle (tests/test_oracle.py).  The reference
itself cannot be built here, so these are the pinned answers.

Run:  python tests/golden/make_golden.py
"""

import json
import os
import struct

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def f32(x):
    """Round a Python float to IEEE single precision."""
    return struct.unpack("f", struct.pack("f", x))[0]


def pbbs_reduce(xs, op):
    """pbbs::reduce: serial fold for <= 1024 items, else blocked."""
    if len(xs) <= 1024:
        r = xs[0]
        for x in xs[1:]:
            r = op(r, x)
        return r
    sums = [pbbs_reduce(xs[i:i + 1024], op) for i in range(0, len(xs), 1024)]
    return pbbs_reduce(sums, op)


class G:
    def __init__(self, n, adj):
        self.n = n
        self.adj = adj  # list of lists of (nbr, weight float32 value)


def efficient_best_move(g, C, k, K, v, res, off):
    deg = len(g.adj[v])
    c = C[v]
    kv = k[v]
    mnw = 0.0 + kv
    if deg <= 1000:
        together = 0.0
        per = {}
        for (u, w) in g.adj[v]:
            x = float(w) - off
            if u != v:
                if C[u] == c:
                    together += x
                per[C[u]] = per.get(C[u], 0.0) + x
        change = 0.0 - (together - res * (kv * (K[c] - kv)))
        best_id, best = None, change
        for cid in sorted(per):
            val = change + (per[cid] - res * (mnw * K[cid]))
            if val > best or (val == best and best_id is not None and cid < best_id):
                best_id, best = cid, val
        return (g.n if best_id is None else best_id), best
    seq = [0.0] * deg
    per = {}
    for j, (u, w) in enumerate(g.adj[v]):
        x = f32(float(w) - off)
        if u != v:
            if C[u] == c:
                seq[j] = x
            per[C[u]] = per.get(C[u], 0.0) + x
    change = 0.0 - (pbbs_reduce(seq, lambda a, b: a + b) - res * (kv * (K[c] - kv)))
    cands = [(change + (per[cid] - res * (mnw * K[cid])), cid) for cid in per]
    if not cands:
        mv, mid = 0.0, 0
    else:
        mv = max(x for x, _ in cands)
        mid = min(cid for x, cid in cands if x == mv)
    if change >= mv:
        return g.n, change
    return mid, mv


def move_nodes(C, s, k, K, n, moves):
    modified = [False] * n
    movers = [v for v in range(n) if moves[v] is not None and moves[v] != C[v]]
    if not movers:
        return modified
    by_old = sorted(movers, key=lambda v: C[v])
    i = 0
    while i < len(by_old):
        j = i
        cid = C[by_old[i]]
        while j < len(by_old) and C[by_old[j]] == cid:
            j += 1
        s[cid] -= j - i
        modified[cid] = True
        for t in range(i, j):
            K[cid] -= k[by_old[t]]
        i = j
    by_new = sorted(movers, key=lambda v: moves[v])
    i = 0
    while i < len(by_new):
        j = i
        t = moves[by_new[i]]
        while j < len(by_new) and moves[by_new[j]] == t:
            j += 1
        if t != n:
            s[t] += j - i
            modified[t] = True
            for q in range(i, j):
                C[by_new[q]] = t
                K[t] += k[by_new[q]]
        i = j
    newc = [v for v in by_new if moves[v] == n]
    if newc:
        zeros = [i for i in range(n) if s[i] == 0]
        for r, v in enumerate(newc):
            cid = zeros[r]
            C[v] = cid
            s[cid] = 1
            modified[cid] = True
            K[cid] = k[v]
    return modified


def cluster_moves(g, C, s, k, K, res, off):
    """Whole-cluster moves of one synchronous round (DEFAULT_CLUSTER_MOVES,
    subclustering NONE): parallel-correlation-clusterer.cc:167-297 with
    BestMove(moving_nodes) (internal.cc:644-707) and BestMoveFromStats
    (correlation-clusterer-util.h:70-113).  Returns the modified clusters."""
    n = g.n
    moves = [None] * n
    for members in groups_by_id(C):
        c = C[members[0]]
        inside = set(members)
        weight, weight_c = 0.0, 0.0       # moving_nodes_weight, cluster_moving_weights[c]
        after = {}                        # class_1_together_after: cluster -> sum
        for v in members:
            weight_c += k[v]
            weight += k[v]
            for (u, w) in g.adj[v]:
                wf = f32(w - off)         # float weight -= double offset
                if u in inside:
                    continue              # class 2, both ends in c: not separate
                after[C[u]] = after.get(C[u], 0.0) + wf
        half_square = lambda x: x * x / 2
        change = 0.0
        change += 0.0 / 2 - res * (half_square(weight) - half_square(weight_c))
        change -= 0.0 - res * (weight_c * (K[c] - weight_c))
        best_id, best_val = None, change
        for d, total in after.items():
            val = change + (total - res * (weight * (K[d] - 0.0)))
            if val > best_val or (val == best_val and best_id is not None and d < best_id):
                best_id, best_val = d, val
        target = best_id if best_id is not None else n
        if target < n and c >= target:
            best_val = 0.0
        if best_val > 0:
            for v in members:
                moves[v] = target
    return move_nodes(C, s, k, K, n, moves)


def best_moves_round(g, C, s, k, K, frontier, res, off, move_method, whole_clusters=False):
    n = g.n
    moves = [None] * n
    moved_vertex = [False] * n
    for v in frontier:
        t, val = efficient_best_move(g, C, k, K, v, res, off)
        cur = C[v]
        if t < n and s[t] == 1 and s[cur] == 1 and cur >= t:
            t, val = cur, 0.0
        if val > 0:
            moves[v] = t
            moved_vertex[v] = True
    modified = move_nodes(C, s, k, K, n, moves)
    if whole_clusters:
        extra = cluster_moves(g, C, s, k, K, res, off)
        modified = [a or b for a, b in zip(modified, extra)]
    if move_method == 1:  # ALL_MOVE
        return list(range(n))
    if move_method == 0:
        marked = [modified[C[v]] for v in range(n)]
    else:
        marked = moved_vertex
    nxt = set()
    for v in range(n):
        if marked[v]:
            for (u, _) in g.adj[v]:
                nxt.add(u)
    return sorted(nxt)


def iterate(g, C, s, k, K, inner, res, off, mm, ctr, whole_clusters=False):
    frontier = list(range(g.n))
    moved = False
    local = True
    it = 0
    while it < inner and local:
        ctr["ev"] += sum(len(g.adj[v]) for v in frontier)
        ctr["rounds"] += 1
        frontier = best_moves_round(g, C, s, k, K, frontier, res, off, mm, whole_clusters)
        local = len(frontier) > 0
        moved |= local
        it += 1
    return moved


def compress(g, C, k):
    n2 = max(C) + 1 if g.n else 1
    ents = []
    for u in range(g.n):
        for (v, w) in g.adj[u]:
            if v <= u or C[v] != C[u]:
                ents.append((C[u], C[v], w))
    ents.sort(key=lambda e: (e[0], e[1]))  # Python sort is stable
    adj = [[] for _ in range(n2)]
    i = 0
    while i < len(ents):
        j = i
        while j < len(ents) and ents[j][:2] == ents[i][:2]:
            j += 1
        w = pbbs_reduce([ents[t][2] for t in range(i, j)], lambda a, b: f32(a + b))
        adj[ents[i][0]].append((ents[i][1], w))
        i = j
    nk = [0.0] * n2
    order = sorted(range(g.n), key=lambda v: C[v])
    i = 0
    while i < len(order):
        j = i
        while j < len(order) and C[order[j]] == C[order[i]]:
            j += 1
        nk[C[order[i]]] = pbbs_reduce([k[order[t]] for t in range(i, j)], lambda a, b: a + b)
        i = j
    return G(n2, adj), nk


def groups_by_id(ids):
    d = {}
    for i, x in enumerate(ids):
        d.setdefault(x, []).append(i)
    return [d[x] for x in sorted(d)]


def cluster(g, cfg, node_weights=None):
    res, off = cfg["resolution"], cfg.get("edge_weight_offset", 0.0)
    whole = cfg.get("clustering_moves_method", 1) == 0  # DEFAULT_CLUSTER_MOVES
    if whole:   # one level, num_iterations rounds (:487-492)
        iters = 1
        inner = cfg.get("num_iterations", 0) or 20
    else:
        iters = cfg.get("louvain_num_iterations", 0) or 10
        inner = cfg.get("louvain_num_inner_iterations", 0) or 10
    refine = cfg.get("refine", False)
    mm = cfg.get("move_method", 0)
    n = g.n
    k = list(node_weights) if node_weights is not None else [1.0] * n
    helpers = [None] * iters
    graphs = [None] * iters
    cur = g
    C, s, K = list(range(n)), [1] * n, list(k)
    hk = list(k)
    ids = list(range(n))
    ctr = {"ev": 0, "rounds": 0}
    it = 0
    while it < iters:
        moved = iterate(cur, C, s, hk, K, inner, res, off, mm, ctr, whole)
        if not moved:
            it -= 1
            break
        if not refine:
            ids = [C[x] for x in ids]
        elif it == iters - 1:
            helpers[it] = (C, s, hk, K)
            graphs[it] = cur
        if it == iters - 1:
            break
        ng, nk = compress(cur, C, hk)
        if refine:
            helpers[it] = (C, s, hk, K)
            graphs[it] = cur
        cur = ng
        C, s, hk, K = list(range(ng.n)), [1] * ng.n, nk, list(nk)
        it += 1
    if refine and it > 0:
        for i in range(it - 1, -1, -1):
            Ci, si, ki, Ki = helpers[i]
            Cu = helpers[i + 1][0]
            flat = [Cu[Ci[j]] for j in range(len(Ci))]
            grps = groups_by_id(flat)
            for q in range(len(si)):
                si[q] = 0
                Ki[q] = 0.0
            for gi, members in enumerate(grps):
                si[gi] = len(members)
                for j in members:
                    Ci[j] = gi
                    Ki[gi] += ki[j]
            iterate(graphs[i], Ci, si, ki, Ki, inner, res, off, mm, ctr, whole)
        ids = helpers[0][0]
    grps = groups_by_id(ids)
    labels = [0] * n
    for gi, members in enumerate(grps):
        for v in members:
            labels[v] = gi
    return labels, ctr


def objective(g, labels, k, res, off):
    K = {}
    for v, c in enumerate(labels):
        K[c] = K.get(c, 0.0) + k[v]
    e = 0.0
    for v in range(g.n):
        for (u, w) in g.adj[v]:
            if labels[u] == labels[v]:
                e += (float(w) - off) / 2
    r = sum(k[v] * (K[labels[v]] - k[v]) for v in range(g.n))
    return e - res * r / 2


def from_edges(n, edges, weights=None):
    adj = [[] for _ in range(n)]
    for i, (a, b) in enumerate(edges):
        w = f32(weights[i]) if weights is not None else 1.0
        adj[a].append((b, w))
        if a != b:
            adj[b].append((a, w))
    for row in adj:
        row.sort(key=lambda x: x[0])
    return G(n, adj)


def sbm_edges(n, blocks, p_in, p_out, seed):
    rng = np.random.default_rng(seed)
    blk = rng.integers(0, blocks, size=n)
    edges = []
    for i in range(n):
        for j in range(i + 1, n):
            p = p_in if blk[i] == blk[j] else p_out
            if rng.random() < p:
                edges.append((i, j))
    return edges


def cases():
    out = []
    # Two triangles joined by one edge.
    out.append(("two_triangles", 6, [(0, 1), (1, 2), (0, 2), (3, 4), (4, 5), (3, 5), (2, 3)], None))
    # A path of 8 vertices.
    out.append(("path8", 8, [(i, i + 1) for i in range(7)], None))
    # Two 5-cliques, an isolated vertex (10) and a pendant (11 - 0).
    e = [(a, b) for a in range(5) for b in range(a + 1, 5)] + [(a, b) for a in range(5, 10) for b in range(a + 1, 10)]
    out.append(("two_cliques_isolated", 12, e + [(0, 11), (4, 5)], None))
    # Star with a hub above the 1000-degree threshold (the reference's hub path).
    out.append(("star1200", 1201, [(0, i) for i in range(1, 1201)] + [(1, 2), (3, 4)], None))
    # Seeded SBMs.
    out.append(("sbm60", 60, sbm_edges(60, 4, 0.5, 0.03, 1), None))
    out.append(("sbm150", 150, sbm_edges(150, 6, 0.3, 0.01, 2), None))
    # Integer and real weights.
    e = sbm_edges(80, 4, 0.4, 0.04, 3)
    rng = np.random.default_rng(4)
    out.append(("sbm80_intw", 80, e, [float(x) for x in rng.integers(1, 5, size=len(e))]))
    out.append(("sbm80_realw", 80, e, [float(x) for x in rng.uniform(0.5, 1.5, size=len(e))]))
    return out


CONFIGS = [
    {"kind": "correlation", "resolution": 0.01, "refine": True, "move_method": 1},
    {"kind": "correlation", "resolution": 0.1, "refine": False, "move_method": 0},
    {"kind": "correlation", "resolution": 0.3, "refine": True, "move_method": 2,
     "louvain_num_iterations": 3, "louvain_num_inner_iterations": 5},
    {"kind": "correlation", "resolution": 0.05, "edge_weight_offset": 0.5, "refine": True, "move_method": 2},
    {"kind": "modularity", "resolution": 1.0, "refine": True, "move_method": 2},
    {"kind": "modularity", "resolution": 0.5, "refine": False, "move_method": 0},
    # Whole-cluster moves (one level).  With refine the reference's level loop
    # returns the identity clustering (refinement needs a second level).
    {"kind": "correlation", "resolution": 0.05, "refine": False, "move_method": 1,
     "clustering_moves_method": 0},
    {"kind": "correlation", "resolution": 0.2, "edge_weight_offset": 0.5, "refine": False, "move_method": 0,
     "clustering_moves_method": 0, "num_iterations": 6},
    {"kind": "correlation", "resolution": 0.01, "refine": True, "move_method": 2,
     "clustering_moves_method": 0},
    {"kind": "modularity", "resolution": 1.0, "refine": False, "move_method": 2,
     "clustering_moves_method": 0},
]


def main():
    fixtures = []
    for name, n, edges, weights in cases():
        g = from_edges(n, edges, weights)
        for cfg in CONFIGS:
            if cfg["kind"] == "modularity":
                k = [float(len(g.adj[v])) for v in range(n)]
                total = pbbs_reduce(k, lambda a, b: a + b) if n else 0.0
                c2 = dict(cfg, resolution=cfg["resolution"] / total, edge_weight_offset=0.0)
                labels, ctr = cluster(g, c2, k)
                obj = objective(g, labels, k, c2["resolution"], 0.0)
            else:
                labels, ctr = cluster(g, cfg)
                obj = objective(g, labels, [1.0] * n, cfg["resolution"], cfg.get("edge_weight_offset", 0.0))
            fixtures.append({"graph": name, "n": n, "edges": edges, "weights": weights, "config": cfg,
                             "labels": labels, "edge_visits": ctr["ev"], "rounds": ctr["rounds"],
                             "objective": obj})
    with open(os.path.join(HERE, "golden_clusterings.json"), "w") as f:
        json.dump(fixtures, f)
    print(f"wrote {len(fixtures)} fixtures")


if __name__ == "__main__":
    main()
