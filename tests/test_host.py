"""CPU tests of the host side: the C-ABI libraries load and export every
declared symbol, the generators are deterministic and well-formed, and the
GBBS adjacency format round-trips."""

import ctypes
import os
import re

import numpy as np
import pytest

import pcc_gb300 as P
import pcc_graphs as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:[\w\s\*]+?)\b(pc\w+)\s*\(", text, flags=re.M)))


@pytest.mark.parametrize("header,lib", [("pcc_gb300.h", "libpcc_gb300.so"), ("pcc_host.h", "libpcc_host.so")])
def test_library_exports_every_declared_symbol(built, header, lib):
    names = _declared_functions(header)
    assert len(names) >= 3
    so = ctypes.CDLL(os.path.join(ROOT, "parallel-correlation-clustering_gb300", "_build", lib))
    missing = [nm for nm in names if not hasattr(so, nm)]
    assert not missing, missing


def test_config_defaults_match_proto(built):
    lib = P.load_library()
    c = P.PccConfig()
    lib.pcc_config_default(ctypes.byref(c))
    assert c.clustering_moves_method == P.LOUVAIN
    assert c.move_method == P.NBHR_CLUSTER_MOVE
    assert c.resolution == 0 and c.refine == 0 and c.async_ == 0


def test_context_without_gpu_fails_cleanly(built):
    """On a machine without a GPU, creating a context is an UNAVAILABLE
    error, not a CPU fallback."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(P.PccError) as e:
        P.Context(0)
    assert e.value.code == 14


def _check_graph(g):
    off, nbr = g.offsets.astype(np.int64), g.neighbors.astype(np.int64)
    assert off[0] == 0 and off[-1] == g.m
    assert np.all(np.diff(off) >= 0)
    src = np.repeat(np.arange(g.n), np.diff(off))
    assert not np.any(src == nbr), "self-loop"
    key = src * g.n + nbr
    assert np.all(np.diff(key) > 0), "rows sorted, no duplicates"
    rev = np.sort(nbr * g.n + src)
    np.testing.assert_array_equal(np.sort(key), rev)  # symmetric


def test_sbm_generator(built):
    g, blk = G.sbm(2000, 10, 0.05, 0.001, 3)
    _check_graph(g)
    g2, blk2 = G.sbm(2000, 10, 0.05, 0.001, 3)
    np.testing.assert_array_equal(g.neighbors, g2.neighbors)
    np.testing.assert_array_equal(blk, blk2)
    src = np.repeat(np.arange(g.n), np.diff(g.offsets).astype(np.int64))
    frac_in = np.mean(blk[src] == blk[g.neighbors])
    assert frac_in > 0.8


def test_rmat_generator(built):
    g = G.rmat(12, 16, seed=2)
    _check_graph(g)
    assert g.n == 4096
    assert g.degrees().max() > 20 * g.degrees().mean()  # skewed
    g2 = G.rmat(12, 16, seed=2)
    np.testing.assert_array_equal(g.offsets, g2.offsets)


def test_lfr_generator(built):
    g, comm = G.lfr(20000, mean_degree=20, dmax=500, seed=5)
    _check_graph(g)
    assert 12 < g.degrees().mean() < 25
    assert g.weights is not None and 0.5 <= g.weights.min() and g.weights.max() <= 1.5
    # weights are symmetric
    src = np.repeat(np.arange(g.n), np.diff(g.offsets).astype(np.int64))
    d = dict(zip(zip(src.tolist(), g.neighbors.tolist()), g.weights.tolist()))
    for (a, b), w in list(d.items())[:2000]:
        assert d[(b, a)] == w


def test_gbbs_roundtrip(tmp_path, built):
    g, _ = G.sbm(300, 5, 0.1, 0.01, 1)
    p = tmp_path / "g.adj"
    G.write_gbbs(str(p), g)
    h = G.read_gbbs(str(p))
    np.testing.assert_array_equal(g.offsets, h.offsets)
    np.testing.assert_array_equal(g.neighbors, h.neighbors)
    gw = P.CsrGraph(g.offsets, g.neighbors, np.linspace(0.5, 1.5, g.m).astype(np.float32))
    G.write_gbbs(str(p), gw)
    h = G.read_gbbs(str(p))
    np.testing.assert_array_equal(gw.weights, h.weights)
    bad = tmp_path / "bad.adj"
    bad.write_text("AdjacencyGraph\n3\n4\n0\n")
    with pytest.raises(P.PccError):
        G.read_gbbs(str(bad))
