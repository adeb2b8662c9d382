"""ctypes binding of the oracle (oracle/pcc_oracle.cc).

TEST AND BASELINE INFRASTRUCTURE ONLY.  Imported by tests/, by the smoke
check in __graft_entry__.py and by bench.py's CPU-baseline leg, where it is
the checker or the timed CPU baseline -- never a path of the product.
Parity of the oracle itself is unpinned against the reference binary (it
cannot be built here); it is pinned against hand-derived answers and an
independent pure-Python restatement (tests/golden/).
"""

from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_ROOT = os.path.dirname(_HERE)
sys.path.insert(0, os.path.join(_ROOT, "parallel-correlation-clustering_gb300"))
from pcc_gb300 import CsrGraph, PccConfig, PccStats  # noqa: E402

SRC = os.path.join(_HERE, "pcc_oracle.cc")
LIB = os.path.join(_HERE, "_build", "libpcc_oracle.so")


def build(force: bool = False) -> str:
    """Compiles the oracle with g++ (-ffp-contract=off, OpenMP, portable)."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(SRC),
            os.path.getmtime(os.path.join(_ROOT, "include", "pcc_gb300.h"))):
        return LIB
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC",
           "-shared", "-Wall", "-I" + os.path.join(_ROOT, "include"), SRC, "-o", LIB]
    subprocess.run(cmd, check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        P = ctypes.POINTER
        vp = ctypes.c_void_p
        L.pcco_set_threads.argtypes = [ctypes.c_int]
        L.pcco_get_threads.restype = ctypes.c_int
        L.pcco_graph_create.argtypes = [ctypes.c_uint32, ctypes.c_uint64,
                                        P(ctypes.c_uint64), P(ctypes.c_uint32),
                                        P(ctypes.c_float)]
        L.pcco_graph_create.restype = vp
        L.pcco_graph_free.argtypes = [vp]
        L.pcco_graph_info.argtypes = [vp, P(ctypes.c_uint32), P(ctypes.c_uint64)]
        L.pcco_graph_copy.argtypes = [vp, P(ctypes.c_uint64), P(ctypes.c_uint32),
                                      P(ctypes.c_float), P(ctypes.c_double)]
        L.pcco_correlation_cluster.argtypes = [vp, P(PccConfig), P(ctypes.c_double),
                                               P(ctypes.c_uint32), P(ctypes.c_uint32),
                                               P(PccStats)]
        L.pcco_modularity_cluster.argtypes = [vp, P(PccConfig), P(ctypes.c_uint32),
                                              P(ctypes.c_uint32), P(PccStats)]
        L.pcco_objective.argtypes = [vp, P(PccConfig), P(ctypes.c_double),
                                     P(ctypes.c_uint32), P(ctypes.c_double)]
        L.pcco_modularity.argtypes = [vp, ctypes.c_double, P(ctypes.c_uint32),
                                      P(ctypes.c_double)]
        L.pcco_best_moves.argtypes = [vp, P(PccConfig), P(ctypes.c_uint32),
                                      P(ctypes.c_uint32), P(ctypes.c_double),
                                      P(ctypes.c_double), P(ctypes.c_uint32),
                                      P(ctypes.c_double), P(ctypes.c_uint32)]
        L.pcco_move_nodes.argtypes = [ctypes.c_uint32, P(ctypes.c_uint32),
                                      P(ctypes.c_uint32), P(ctypes.c_double),
                                      P(ctypes.c_double), P(ctypes.c_uint32),
                                      P(ctypes.c_uint8)]
        L.pcco_compress.argtypes = [vp, P(ctypes.c_uint32), P(ctypes.c_double)]
        L.pcco_compare_communities.argtypes = [ctypes.c_uint32, P(ctypes.c_uint32), ctypes.c_uint32,
                                               P(ctypes.c_uint64), P(ctypes.c_uint32),
                                               P(ctypes.c_double), P(ctypes.c_double), P(ctypes.c_double)]
        L.pcco_compress.restype = vp
        L.pcco_gen_rmat.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_double, ctypes.c_uint64]
        L.pcco_gen_rmat.restype = vp
        L.pcco_subclusters.argtypes = [vp, P(ctypes.c_uint32), ctypes.c_int32, ctypes.c_double, ctypes.c_double,
                                       P(ctypes.c_uint32), P(ctypes.c_uint64), P(ctypes.c_uint32)]
        _lib = L
    return _lib


def set_threads(t: int):
    lib().pcco_set_threads(int(t))


def get_threads() -> int:
    return int(lib().pcco_get_threads())


def _p(a, t):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(t))


class OracleGraph:
    def __init__(self, g: CsrGraph = None, handle=None):
        L = lib()
        if handle is not None:
            self.h = handle
        else:
            self._off = np.ascontiguousarray(g.offsets, dtype=np.uint64)
            self._nbr = np.ascontiguousarray(g.neighbors, dtype=np.uint32)
            self._w = None if g.weights is None else np.ascontiguousarray(g.weights, np.float32)
            self.h = L.pcco_graph_create(g.n, g.m, _p(self._off, ctypes.c_uint64),
                                         _p(self._nbr, ctypes.c_uint32),
                                         _p(self._w, ctypes.c_float))

    def __del__(self):
        try:
            lib().pcco_graph_free(self.h)
        except Exception:
            pass

    def info(self):
        n = ctypes.c_uint32()
        m = ctypes.c_uint64()
        lib().pcco_graph_info(self.h, ctypes.byref(n), ctypes.byref(m))
        return int(n.value), int(m.value)

    def to_csr(self):
        """(CsrGraph with float weights, node weights attached by compression)."""
        n, m = self.info()
        off = np.empty(n + 1, np.uint64)
        nbr = np.empty(m, np.uint32)
        w = np.empty(m, np.float32)
        nw = np.empty(n, np.float64)
        lib().pcco_graph_copy(self.h, _p(off, ctypes.c_uint64), _p(nbr, ctypes.c_uint32),
                              _p(w, ctypes.c_float), _p(nw, ctypes.c_double))
        return CsrGraph(off, nbr, w), nw


def _check(st):
    if st != 0:
        raise RuntimeError(f"oracle status {st}")


def correlation_cluster(g: OracleGraph, cfg: PccConfig, node_weights=None,
                        initial_labels=None):
    n, _ = g.info()
    out = np.empty(n, np.uint32)
    st = PccStats()
    k = None if node_weights is None else np.ascontiguousarray(node_weights, np.float64)
    lab = None if initial_labels is None else np.ascontiguousarray(initial_labels, np.uint32)
    _check(lib().pcco_correlation_cluster(g.h, ctypes.byref(cfg), _p(k, ctypes.c_double),
                                          _p(lab, ctypes.c_uint32), _p(out, ctypes.c_uint32),
                                          ctypes.byref(st)))
    return out, st.as_dict()


def modularity_cluster(g: OracleGraph, cfg: PccConfig, initial_labels=None):
    n, _ = g.info()
    out = np.empty(n, np.uint32)
    st = PccStats()
    lab = None if initial_labels is None else np.ascontiguousarray(initial_labels, np.uint32)
    _check(lib().pcco_modularity_cluster(g.h, ctypes.byref(cfg), _p(lab, ctypes.c_uint32),
                                         _p(out, ctypes.c_uint32), ctypes.byref(st)))
    return out, st.as_dict()


def objective(g: OracleGraph, cfg: PccConfig, labels, node_weights=None) -> float:
    out = ctypes.c_double()
    lab = np.ascontiguousarray(labels, np.uint32)
    k = None if node_weights is None else np.ascontiguousarray(node_weights, np.float64)
    _check(lib().pcco_objective(g.h, ctypes.byref(cfg), _p(k, ctypes.c_double),
                                _p(lab, ctypes.c_uint32), ctypes.byref(out)))
    return float(out.value)


def modularity(g: OracleGraph, resolution: float, labels) -> float:
    out = ctypes.c_double()
    lab = np.ascontiguousarray(labels, np.uint32)
    _check(lib().pcco_modularity(g.h, resolution, _p(lab, ctypes.c_uint32),
                                 ctypes.byref(out)))
    return float(out.value)


def best_moves(g: OracleGraph, cfg: PccConfig, C, s, k, K):
    n, _ = g.info()
    C = np.ascontiguousarray(C, np.uint32)
    s = np.ascontiguousarray(s, np.uint32)
    k = np.ascontiguousarray(k, np.float64)
    K = np.ascontiguousarray(K, np.float64)
    t = np.empty(n, np.uint32)
    v = np.empty(n, np.float64)
    mv = np.empty(n, np.uint32)
    _check(lib().pcco_best_moves(g.h, ctypes.byref(cfg), _p(C, ctypes.c_uint32),
                                 _p(s, ctypes.c_uint32), _p(k, ctypes.c_double),
                                 _p(K, ctypes.c_double), _p(t, ctypes.c_uint32),
                                 _p(v, ctypes.c_double), _p(mv, ctypes.c_uint32)))
    return t, v, mv


def move_nodes(C, s, k, K, moves):
    """MoveNodesToCluster on copies; returns (C, s, K, modified)."""
    C = np.array(C, np.uint32)
    s = np.array(s, np.uint32)
    K = np.array(K, np.float64)
    k = np.ascontiguousarray(k, np.float64)
    mv = np.ascontiguousarray(moves, np.uint32)
    mod = np.zeros(C.size, np.uint8)
    _check(lib().pcco_move_nodes(C.size, _p(C, ctypes.c_uint32), _p(s, ctypes.c_uint32),
                                 _p(k, ctypes.c_double), _p(K, ctypes.c_double),
                                 _p(mv, ctypes.c_uint32), _p(mod, ctypes.c_uint8)))
    return C, s, K, mod


def compress(g: OracleGraph, C, node_weights=None):
    """CompressGraph; returns (CsrGraph, new node weights)."""
    C = np.ascontiguousarray(C, np.uint32)
    k = None if node_weights is None else np.ascontiguousarray(node_weights, np.float64)
    h = lib().pcco_compress(g.h, _p(C, ctypes.c_uint32), _p(k, ctypes.c_double))
    og = OracleGraph(handle=h)
    return og.to_csr()


def rmat(scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19,
         seed: int = 1) -> OracleGraph:
    """Seeded RMAT graph built inside the oracle (symmetrised, deduplicated,
    no self-loops, unit weights): the same graph as the package's generator
    for the same arguments, without loading any library of the package."""
    return OracleGraph(handle=lib().pcco_gen_rmat(scale, edge_factor, a, b, c, seed))


def subclusters(g: OracleGraph, C, method: int, resolution: float = 0.0, edge_weight_offset: float = 0.0):
    """Subcluster ids of clustering C on g (one level of the subclustering
    before compression); returns (ids, block starts + total)."""
    n, _ = g.info()
    C = np.ascontiguousarray(C, np.uint32)
    ids = np.empty(n, np.uint32)
    nxt = np.empty(n + 1, np.uint64)
    G = ctypes.c_uint32()
    _check(lib().pcco_subclusters(g.h, _p(C, ctypes.c_uint32), method, resolution, edge_weight_offset,
                                  _p(ids, ctypes.c_uint32), _p(nxt, ctypes.c_uint64), ctypes.byref(G)))
    return ids, nxt[:G.value + 1].copy()


def compare_communities(labels, communities):
    """CompareCommunities on host lists; returns (scores dict, precision,
    recall).  communities: a list of vertex-id sequences."""
    labels = np.ascontiguousarray(labels, np.uint32)
    sizes = [len(c) for c in communities]
    off = np.zeros(len(communities) + 1, np.uint64)
    off[1:] = np.cumsum(sizes, dtype=np.uint64)
    mem = (np.concatenate([np.asarray(c, np.uint32) for c in communities]) if sum(sizes)
           else np.zeros(1, np.uint32))
    mem = np.ascontiguousarray(mem, np.uint32)
    prec = np.zeros(max(len(communities), 1), np.float64)
    rec = np.zeros(max(len(communities), 1), np.float64)
    out = np.zeros(6, np.float64)
    _check(lib().pcco_compare_communities(labels.size, _p(labels, ctypes.c_uint32), len(communities),
                                          _p(off, ctypes.c_uint64), _p(mem, ctypes.c_uint32),
                                          _p(prec, ctypes.c_double), _p(rec, ctypes.c_double),
                                          _p(out, ctypes.c_double)))
    scores = {"avg_precision": out[0], "avg_recall": out[1], "num_clusters": int(out[2]),
              "min_size": int(out[3]), "max_size": int(out[4]), "avg_size": out[5]}
    return scores, prec[:len(communities)], rec[:len(communities)]
