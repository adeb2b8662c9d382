"""Synthetic graphs and GBBS adjacency I/O (bindings of libpcc_host.so).

The generators make the seeded stand-ins for the reference's evaluation
graphs: stochastic block models, RMAT (Graph500 quadrant recursion) and
LFR-like planted partitions.  Outputs are deterministic for a seed on any
machine and thread count.
"""

from __future__ import annotations

import ctypes
import os

import numpy as np

from pcc_gb300 import CsrGraph, PccError

_HERE = os.path.dirname(os.path.abspath(__file__))
HOST_LIB = os.path.join(_HERE, "_build", "libpcc_host.so")


class _PcchGraph(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_uint32),
        ("m", ctypes.c_uint64),
        ("off", ctypes.POINTER(ctypes.c_uint64)),
        ("nbr", ctypes.POINTER(ctypes.c_uint32)),
        ("w", ctypes.POINTER(ctypes.c_float)),
        ("truth", ctypes.POINTER(ctypes.c_uint32)),
    ]


_lib = None


def host_lib():
    global _lib
    if _lib is None:
        if not os.path.exists(HOST_LIB):
            raise PccError(14, f"host library not built: {HOST_LIB}")
        L = ctypes.CDLL(HOST_LIB)
        GP = ctypes.POINTER(_PcchGraph)
        L.pcch_graph_free.argtypes = [GP]
        L.pcch_gen_sbm.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_uint64]
        L.pcch_gen_sbm.restype = GP
        L.pcch_gen_rmat.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_uint64]
        L.pcch_gen_rmat.restype = GP
        L.pcch_gen_lfr.argtypes = [ctypes.c_uint32, ctypes.c_double, ctypes.c_uint32, ctypes.c_double,
                                   ctypes.c_uint32, ctypes.c_uint32, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_double, ctypes.c_uint64]
        L.pcch_gen_lfr.restype = GP
        L.pcch_parse_config.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32),
                                        ctypes.c_char_p, ctypes.c_size_t]
        L.pcch_parse_config.restype = ctypes.c_int32
        L.pcch_read_gbbs.argtypes = [ctypes.c_char_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]
        L.pcch_read_gbbs.restype = GP
        L.pcch_compare_communities.argtypes = [ctypes.c_char_p, ctypes.c_uint32, ctypes.c_void_p,
                                               ctypes.POINTER(ctypes.c_double)]
        L.pcch_compare_communities.restype = ctypes.c_int32
        _lib = L
    return _lib


def _take(gp):
    """Copies a library-owned graph into numpy arrays and frees it."""
    g = gp.contents
    n, m = int(g.n), int(g.m)
    off = np.ctypeslib.as_array(g.off, shape=(n + 1,)).copy()
    nbr = np.ctypeslib.as_array(g.nbr, shape=(max(m, 1),))[:m].copy()
    w = np.ctypeslib.as_array(g.w, shape=(max(m, 1),))[:m].copy() if g.w else None
    truth = np.ctypeslib.as_array(g.truth, shape=(max(n, 1),))[:n].copy() if g.truth else None
    host_lib().pcch_graph_free(gp)
    return CsrGraph(off, nbr, w), truth


def sbm(n: int, blocks: int, p_in: float, p_out: float, seed: int):
    """Stochastic block model; returns (CsrGraph, block of each vertex)."""
    return _take(host_lib().pcch_gen_sbm(n, blocks, p_in, p_out, seed))


def rmat(scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19,
         seed: int = 1) -> CsrGraph:
    """RMAT graph (symmetrised, deduplicated, no self-loops, unit weights)."""
    g, _ = _take(host_lib().pcch_gen_rmat(scale, edge_factor, a, b, c, seed))
    return g


def lfr(n: int, mean_degree: float = 20.0, dmax: int = 2000, tau1: float = 2.2, cmin: int = 5,
        cmax: int = 5000, tau2: float = 2.5, mu: float = 0.3, w_lo: float = 0.5, w_hi: float = 1.5,
        seed: int = 1):
    """LFR-like planted partition; returns (CsrGraph, community of each vertex)."""
    return _take(host_lib().pcch_gen_lfr(n, mean_degree, dmax, tau1, cmin, cmax, tau2, mu, w_lo, w_hi, seed))


def write_gbbs(path: str, g: CsrGraph) -> None:
    """Writes the GBBS text adjacency format (AdjacencyGraph /
    WeightedAdjacencyGraph: header, n, m, n offsets, m targets, [m weights])."""
    with open(path, "w") as f:
        f.write("WeightedAdjacencyGraph\n" if g.weights is not None else "AdjacencyGraph\n")
        f.write(f"{g.n}\n{g.m}\n")
        np.savetxt(f, g.offsets[:-1].astype(np.uint64), fmt="%d")
        np.savetxt(f, g.neighbors.astype(np.uint32), fmt="%d")
        if g.weights is not None:
            np.savetxt(f, g.weights.astype(np.float32), fmt="%.9g")


def parse_config(text: str):
    """Text-format ClustererConfig -> (PccConfig, config_case) via the C++
    parser (config_case: 0 unset, 1 parameter_string, 4 affinity, 7
    correlation).  Raises PccError(3) with the parser's message."""
    from pcc_gb300 import PccConfig
    cfg = PccConfig()
    case = ctypes.c_int32(0)
    err = ctypes.create_string_buffer(512)
    st = host_lib().pcch_parse_config(text.encode(), ctypes.byref(cfg), ctypes.byref(case), err, 512)
    if st != 0:
        raise PccError(st, err.value.decode(errors="replace"))
    return cfg, case.value


def read_gbbs_native(path: str, float_weighted: bool = False) -> CsrGraph:
    """Reads a GBBS adjacency file with the C++ reader of the CLI."""
    st = ctypes.c_int32(0)
    gp = host_lib().pcch_read_gbbs(path.encode(), 1 if float_weighted else 0, ctypes.byref(st))
    if not gp:
        raise PccError(st.value, f"cannot read GBBS graph {path}")
    g, _ = _take(gp)
    return g


def compare_communities(path: str, labels) -> dict:
    """CompareCommunities of the CLI: average precision / recall of the
    clustering (labels = cluster index per node) against a communities file."""
    lab = np.ascontiguousarray(labels, dtype=np.uint32)
    out = (ctypes.c_double * 6)()
    st = host_lib().pcch_compare_communities(path.encode(), lab.size, lab.ctypes.data_as(ctypes.c_void_p), out)
    if st != 0:
        raise PccError(st, f"cannot score against {path}")
    keys = ("avg_precision", "avg_recall", "num_clusters", "min_size", "max_size", "avg_size")
    return dict(zip(keys, list(out)))


def read_gbbs(path: str) -> CsrGraph:
    """Reads the GBBS text adjacency format."""
    with open(path) as f:
        header = f.readline().strip()
        if header not in ("AdjacencyGraph", "WeightedAdjacencyGraph"):
            raise PccError(3, f"not a GBBS adjacency graph: {header!r}")
        data = np.array(f.read().split(), dtype=np.float64)
    n, m = int(data[0]), int(data[1])
    need = 2 + n + m + (m if header.startswith("Weighted") else 0)
    if data.size < need:
        raise PccError(3, f"truncated GBBS file: {data.size} numbers, need {need}")
    off = np.empty(n + 1, dtype=np.uint64)
    off[:n] = data[2:2 + n].astype(np.uint64)
    off[n] = m
    nbr = data[2 + n:2 + n + m].astype(np.uint32)
    w = data[2 + n + m:2 + n + 2 * m].astype(np.float32) if header.startswith("Weighted") else None
    return CsrGraph(off, nbr, w)


def batch_sbm_spec(count: int, seed: int = 7, n_lo: int = 200, n_hi: int = 50000):
    """Parameters of the batched SBM workload: n log-uniform in [n_lo, n_hi],
    blocks uniform in [2, 200] (at most n / 2), mean degree uniform in
    [8, 32], p_out / p_in = 0.02.  Returns a list of (n, blocks, p_in, p_out,
    seed) tuples; p_in solves
    mean degree = p_in * (n / B - 1) + p_out * (n - n / B)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(round(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi)))))
        blocks = int(min(rng.integers(2, 201), max(2, n // 2)))
        deg = rng.uniform(8.0, 32.0)
        size = n / blocks
        p_in = deg / max((size - 1.0) + 0.02 * (n - size), 1e-9)
        p_in = float(min(p_in, 1.0))
        out.append((n, blocks, p_in, 0.02 * p_in, int(rng.integers(1, 2**62))))
    return out


def batch_sbm_graphs(count: int, seed: int = 7, n_lo: int = 200, n_hi: int = 50000):
    """The batched SBM workload's graphs (unit weights)."""
    return [sbm(n, b, pi, po, s)[0] for (n, b, pi, po, s) in batch_sbm_spec(count, seed, n_lo, n_hi)]


def serving_requests(count: int, seed: int = 11, rmat_scale: int = 20, n_hi: int = 50000,
                     distinct_rmat: int = 0):
    """Serving workload: 95% graphs of the batched SBM distribution, 5% RMAT
    (edge factor 16); resolution from {0.01, 0.1, 0.5}; objective modularity
    (1) or correlation (0) with equal probability.  distinct_rmat > 0 reuses
    that many RMAT graphs (generation time) instead of one per request.
    Returns a list of dicts (graph, resolution, objective, kind)."""
    rng = np.random.default_rng(seed)
    spec = batch_sbm_spec(count, seed + 1, n_hi=n_hi)
    out = []
    rmats = []
    for i in range(count):
        if rng.random() < 0.05:
            rseed = int(rng.integers(1, 2**62))
            if distinct_rmat and len(rmats) >= distinct_rmat:
                g = rmats[len(out) % distinct_rmat]
            else:
                g = rmat(rmat_scale, 16, seed=rseed)
                rmats.append(g)
            kind = f"rmat{rmat_scale}"
        else:
            n, b, pi, po, s = spec[i]
            g = sbm(n, b, pi, po, s)[0]
            kind = "sbm"
        out.append({"graph": g, "resolution": float(rng.choice([0.01, 0.1, 0.5])),
                    "objective": int(rng.integers(0, 2)), "kind": kind})
    return out
