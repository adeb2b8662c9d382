"""CPU tests of the C++ host mirror: the text-format ClustererConfig parser,
the GBBS adjacency reader, CompareCommunities and the CLI's error paths."""

import os
import subprocess

import numpy as np
import pytest

import pcc_gb300 as P
import pcc_graphs as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "parallel-correlation-clustering_gb300", "_build", "cluster-in-memory_main")


def test_parse_full_config(built):
    text = """
      # every field of CorrelationClustererConfig
      correlation_clusterer_config {
        resolution: 0.01
        edge_weight_offset: -1.5e-1
        random_seed: 77
        num_iterations: 3
        louvain_config { num_iterations: 10 num_inner_iterations: 12 }
        clustering_moves_method: LOUVAIN
        subclustering_method: NONE_SUBCLUSTERING
        preclustering_method: KCORE_PRECLUSTERING
        kcore_config < kcore_cutoff: 3, fix_preclusters: true; percent_cutoff: 0.5 >
        refine: true
        async: false
        connect_stats: t
        move_method: ALL_MOVE
        all_iter: 1
        permute: True
      }
    """
    cfg, case = G.parse_config(text)
    assert case == 7
    assert cfg.resolution == 0.01 and cfg.edge_weight_offset == -0.15
    assert cfg.random_seed == 77 and cfg.num_iterations == 3
    assert cfg.louvain_num_iterations == 10 and cfg.louvain_num_inner_iterations == 12
    assert cfg.clustering_moves_method == P.LOUVAIN
    assert cfg.preclustering_method == 1
    assert cfg.refine == 1 and cfg.async_ == 0 and cfg.all_iter == 1 and cfg.permute == 1
    assert cfg.move_method == P.ALL_MOVE


def test_parse_whole_cluster_moves(built):
    """DEFAULT_CLUSTER_MOVES with its round count (num_iterations) reaches the
    library config as the engine reads it."""
    cfg, _ = G.parse_config("correlation_clusterer_config { resolution: 0.2 "
                            "clustering_moves_method: DEFAULT_CLUSTER_MOVES num_iterations: 6 "
                            "move_method: NBHR_MOVE }")
    assert cfg.clustering_moves_method == P.DEFAULT_CLUSTER_MOVES
    assert cfg.num_iterations == 6 and cfg.move_method == P.NBHR_MOVE and cfg.resolution == 0.2


def test_parse_defaults_and_numbers(built):
    cfg, case = G.parse_config("")
    assert case == 0
    d = P.make_config()
    assert cfg.move_method == d.move_method == P.NBHR_CLUSTER_MOVE
    assert cfg.clustering_moves_method == P.LOUVAIN
    cfg, case = G.parse_config("correlation_clusterer_config: { move_method: 2 resolution: 1 }")
    assert case == 7 and cfg.move_method == P.NBHR_MOVE and cfg.resolution == 1.0
    cfg, case = G.parse_config('parameter_string: "a b" " c"')
    assert case == 1
    cfg, case = G.parse_config("affinity_clusterer_config { weight_threshold: 0.5 }")
    assert case == 4


@pytest.mark.parametrize("text,needle", [
    ("correlation_clusterer_config { resolutoin: 1 }", "resolutoin"),
    ("correlation_clusterer_config { move_method: SIDEWAYS }", "SIDEWAYS"),
    ("correlation_clusterer_config { move_method: 7 }", "7"),
    ("correlation_clusterer_config { refine: maybe }", "bool"),
    ("correlation_clusterer_config { resolution: 1", "expected '}'"),
    ("correlation_clusterer_config { random_seed: -1 }", "random_seed"),
    ("correlation_clusterer_config { louvain_config: 3 }", "louvain_config"),
    ("bogus_config { }", "bogus_config"),
])
def test_parse_errors(built, text, needle):
    with pytest.raises(P.PccError) as e:
        G.parse_config(text)
    assert e.value.code == 3
    assert needle in str(e.value)


@pytest.mark.parametrize("weighted", [False, True])
def test_gbbs_reader_matches_python(built, tmp_path, weighted):
    if weighted:
        g, _ = G.lfr(3000, mean_degree=12, dmax=200, seed=4)
    else:
        g = G.rmat(10, 8, seed=2)
    path = str(tmp_path / "g.adj")
    G.write_gbbs(path, g)
    h = G.read_gbbs_native(path, float_weighted=weighted)
    np.testing.assert_array_equal(h.offsets, g.offsets)
    np.testing.assert_array_equal(h.neighbors, g.neighbors)
    if weighted:
        np.testing.assert_array_equal(h.weights, g.weights)
    else:
        assert h.weights is None


def test_gbbs_reader_errors(built, tmp_path):
    g = G.rmat(8, 4, seed=1)
    path = str(tmp_path / "g.adj")
    G.write_gbbs(path, g)
    with pytest.raises(P.PccError) as e:
        G.read_gbbs_native(path, float_weighted=True)   # header mismatch
    assert e.value.code == 3
    with pytest.raises(P.PccError) as e:
        G.read_gbbs_native(str(tmp_path / "missing.adj"))
    assert e.value.code == 5
    bad = tmp_path / "bad.adj"
    bad.write_text("AdjacencyGraph\n2\n2\n0\n1\n1\n5\n")   # neighbour id 5 >= n
    with pytest.raises(P.PccError):
        G.read_gbbs_native(str(bad))


def _compare_reference(communities, clustering):
    """CompareCommunities restated in Python (cluster-in-memory_main.cc:
    167-222): largest intersection, first cluster on ties, cluster 0 when
    none intersects."""
    ps, rs = [], []
    for comm in communities:
        best, best_idx = 0, 0
        cs = set(comm)
        for i, cl in enumerate(clustering):
            inter = len(cs.intersection(cl))
            if inter > best:
                best, best_idx = inter, i
        ps.append(best / len(clustering[best_idx]))
        rs.append(0.0 if not comm else best / len(comm))
    sizes = [len(c) for c in clustering]
    return [np.mean(ps), np.mean(rs), len(clustering), min(sizes), max(sizes), np.mean(sizes)]


def test_compare_communities(built, tmp_path):
    rng = np.random.default_rng(5)
    n = 400
    labels = rng.integers(0, 37, size=n)
    _, labels = np.unique(labels, return_inverse=True)
    clustering = P.labels_to_clustering(labels)
    truth = rng.integers(0, 20, size=n)
    communities = [sorted(np.flatnonzero(truth == c).tolist()) for c in range(20)]
    communities.append([])                       # an empty line
    communities.append([n + 3])                  # a node no cluster holds
    path = tmp_path / "comm.txt"
    path.write_text("".join("".join(f"{v}\t" for v in c) + "\n" for c in communities))
    got = G.compare_communities(str(path), labels)
    want = _compare_reference(communities, clustering)
    np.testing.assert_allclose([got[k] for k in ("avg_precision", "avg_recall", "num_clusters", "min_size",
                                                 "max_size", "avg_size")], want, rtol=1e-12)


def _cli(*args):
    return subprocess.run([CLI, *args], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=120)


def test_cli_error_paths(built, tmp_path):
    g = G.rmat(8, 4, seed=1)
    path = str(tmp_path / "g.adj")
    G.write_gbbs(path, g)
    r = _cli("--clusterer_name=ParallelAffinityClusterer", "--input_graph", path)
    assert r.returncode != 0 and "UNIMPLEMENTED" in r.stderr
    r = _cli("--clusterer_name=ParallelCorrelationClusterer", "--clusterer_config=oops {",
             "--input_graph", path)
    assert r.returncode != 0 and "Cannot parse --clusterer_config" in r.stderr
    r = _cli("--clusterer_name=ParallelCorrelationClusterer", "--bogus_flag=1")
    assert r.returncode != 0 and "unknown flag" in r.stderr
    import torch
    if not torch.cuda.is_available():
        r = _cli("--clusterer_name=ParallelModularityClusterer",
                 "--clusterer_config=correlation_clusterer_config { resolution: 1 }", "--input_graph", path)
        assert r.returncode != 0 and "UNAVAILABLE" in r.stderr


def test_compare_communities_matches_oracle(built, tmp_path):
    """The host library's CompareCommunities (CPU path of the CLI) equals the
    oracle's reading of the reference bit for bit, repeats and ids outside
    the graph included."""
    from test_oracle import community_cases
    import oracle as O
    for labels, comms in community_cases():
        path = tmp_path / "comm.txt"
        path.write_text("".join("".join(f"{v}\t" for v in c) + "\n" for c in comms))
        got = G.compare_communities(str(path), labels)
        want, _, _ = O.compare_communities(labels, [sorted(c) for c in comms])
        for key in ("avg_precision", "avg_recall", "num_clusters", "min_size", "max_size", "avg_size"):
            assert got[key] == want[key], key
