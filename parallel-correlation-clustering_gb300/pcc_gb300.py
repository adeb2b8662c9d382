"""Python host binding of libpcc_gb300.so (the GB300 clustering C ABI).

Mirrors the reference's operator interface for the clustering hot path:
``ParallelCorrelationClusterer`` / ``ParallelModularityClusterer`` from
clustering/clusterers/parallel-correlation-clusterer.h:44-95 and
parallel-modularity-clusterer.h:45-56, whose ``Cluster(config)`` returns a
``Clustering`` (list of clusters, each a sorted list of node ids, clusters
ordered by internal id -- clustering/in-memory-clusterer.h:77).

Everything here calls the CUDA library through ctypes.  There is no CPU
path: if the shared library is missing or has no usable GPU, construction
raises ``PccError``.
"""

from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libpcc_gb300.so")

# absl::StatusCode numbering (clustering/status_macros.h uses absl::Status).
STATUS_NAMES = {
    0: "OK", 1: "CANCELLED", 2: "UNKNOWN", 3: "INVALID_ARGUMENT",
    4: "DEADLINE_EXCEEDED", 5: "NOT_FOUND", 6: "ALREADY_EXISTS",
    7: "PERMISSION_DENIED", 8: "RESOURCE_EXHAUSTED", 9: "FAILED_PRECONDITION",
    10: "ABORTED", 11: "OUT_OF_RANGE", 12: "UNIMPLEMENTED", 13: "INTERNAL",
    14: "UNAVAILABLE", 15: "DATA_LOSS",
}

DEFAULT_CLUSTER_MOVES, LOUVAIN = 0, 1
NONE_SUBCLUSTERING = 0
NBHR_CLUSTER_MOVE, ALL_MOVE, NBHR_MOVE = 0, 1, 2
NO_MOVE = 0xFFFFFFFF


class PccError(RuntimeError):
    """A non-OK status from the C ABI; ``code`` is the absl status code."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {message}")
        self.code = code
        self.message = message


class PccConfig(ctypes.Structure):
    """pcc_config: CorrelationClustererConfig (clustering/config.proto:94-165)."""

    _fields_ = [
        ("resolution", ctypes.c_double),
        ("edge_weight_offset", ctypes.c_double),
        ("num_iterations", ctypes.c_int64),
        ("louvain_num_iterations", ctypes.c_int64),
        ("louvain_num_inner_iterations", ctypes.c_int64),
        ("clustering_moves_method", ctypes.c_int32),
        ("subclustering_method", ctypes.c_int32),
        ("preclustering_method", ctypes.c_int32),
        ("move_method", ctypes.c_int32),
        ("refine", ctypes.c_int32),
        ("async_", ctypes.c_int32),
        ("permute", ctypes.c_int32),
        ("all_iter", ctypes.c_int32),
        ("random_seed", ctypes.c_uint64),
    ]


class PccCommunityScores(ctypes.Structure):
    _fields_ = [("avg_precision", ctypes.c_double), ("avg_recall", ctypes.c_double),
                ("num_clusters", ctypes.c_uint64), ("min_size", ctypes.c_uint64),
                ("max_size", ctypes.c_uint64), ("avg_size", ctypes.c_double)]


class PccStats(ctypes.Structure):
    _fields_ = [
        ("edge_visits", ctypes.c_uint64),
        ("vertex_visits", ctypes.c_uint64),
        ("moves", ctypes.c_uint64),
        ("levels", ctypes.c_int32),
        ("rounds", ctypes.c_int32),
        ("refine_passes", ctypes.c_int32),
        ("num_clusters", ctypes.c_int32),
        ("objective", ctypes.c_double),
        ("modularity", ctypes.c_double),
        ("ms_total", ctypes.c_double),
        ("ms_best_moves", ctypes.c_double),
        ("ms_compress", ctypes.c_double),
        ("ms_apply", ctypes.c_double),
        ("ms_frontier", ctypes.c_double),
        ("kernel_launches", ctypes.c_uint64),
        ("algo_bytes_best_moves", ctypes.c_uint64),
        ("family_ms", ctypes.c_double * 4),
        ("family_launches", ctypes.c_uint64 * 4),
        ("family_entries", ctypes.c_uint64 * 4),
        ("family_vertices", ctypes.c_uint64 * 4),
        ("algo_bytes_compress", ctypes.c_uint64),
        ("algo_bytes_frontier", ctypes.c_uint64),
    ]

    FAMILIES = ("groups", "warps", "small_hubs", "big_hubs")

    def as_dict(self) -> dict:
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if isinstance(v, ctypes.Array) else v
        return out


def make_config(resolution: float = 0.0, edge_weight_offset: float = 0.0,
                num_iterations: int = 0, louvain_num_iterations: int = 0,
                louvain_num_inner_iterations: int = 0,
                clustering_moves_method: int = LOUVAIN,
                subclustering_method: int = NONE_SUBCLUSTERING,
                move_method: int = NBHR_CLUSTER_MOVE, refine: bool = False,
                async_: bool = False, permute: bool = False,
                all_iter: bool = False, random_seed: int = 0) -> PccConfig:
    """A PccConfig with the proto defaults for every field not given."""
    c = PccConfig()
    c.resolution = resolution
    c.edge_weight_offset = edge_weight_offset
    c.num_iterations = num_iterations
    c.louvain_num_iterations = louvain_num_iterations
    c.louvain_num_inner_iterations = louvain_num_inner_iterations
    c.clustering_moves_method = clustering_moves_method
    c.subclustering_method = subclustering_method
    c.preclustering_method = 0
    c.move_method = move_method
    c.refine = int(bool(refine))
    c.async_ = int(bool(async_))
    c.permute = int(bool(permute))
    c.all_iter = int(bool(all_iter))
    c.random_seed = random_seed
    return c


@dataclass
class CsrGraph:
    """Host symmetric CSR graph: offsets uint64[n+1], neighbors uint32[m],
    weights float32[m] or None (unit weights)."""

    offsets: np.ndarray
    neighbors: np.ndarray
    weights: Optional[np.ndarray] = None

    @property
    def n(self) -> int:
        return int(self.offsets.shape[0] - 1)

    @property
    def m(self) -> int:
        return int(self.neighbors.shape[0])

    def degrees(self) -> np.ndarray:
        return np.diff(self.offsets).astype(np.int64)

    @staticmethod
    def from_edges(n: int, src, dst, w=None, symmetrize: bool = True,
                   dedupe: bool = True, drop_self_loops: bool = False) -> "CsrGraph":
        """Builds CSR from an edge list (rows sorted by neighbour id)."""
        src = np.asarray(src, dtype=np.int64)
        dst = np.asarray(dst, dtype=np.int64)
        ww = None if w is None else np.asarray(w, dtype=np.float32)
        if drop_self_loops:
            keep = src != dst
            src, dst = src[keep], dst[keep]
            ww = None if ww is None else ww[keep]
        if symmetrize:
            loops = src == dst
            s2 = np.concatenate([src, dst[~loops]])
            d2 = np.concatenate([dst, src[~loops]])
            ww = None if ww is None else np.concatenate([ww, ww[~loops]])
            src, dst = s2, d2
        key = src * (n + 1) + dst
        order = np.argsort(key, kind="stable")
        src, dst, key = src[order], dst[order], key[order]
        ww = None if ww is None else ww[order]
        if dedupe and key.size:
            first = np.ones(key.size, dtype=bool)
            first[1:] = key[1:] != key[:-1]
            src, dst = src[first], dst[first]
            ww = None if ww is None else ww[first]
        counts = np.bincount(src, minlength=n).astype(np.uint64)
        offsets = np.zeros(n + 1, dtype=np.uint64)
        np.cumsum(counts, out=offsets[1:])
        return CsrGraph(offsets, dst.astype(np.uint32),
                        None if ww is None else ww.astype(np.float32))


def _ptr(a: Optional[np.ndarray], ctype):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctype))


_lib = None


def load_library(path: str = LIB_PATH) -> ctypes.CDLL:
    """Loads libpcc_gb300.so; raises PccError when it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise PccError(14, f"CUDA library not built: {path} (run __graft_entry__.build())")
    lib = ctypes.CDLL(path)
    P = ctypes.POINTER
    vp = ctypes.c_void_p
    lib.pcc_create.argtypes = [P(vp), ctypes.c_int, ctypes.c_uint64]
    lib.pcc_create.restype = ctypes.c_int
    lib.pcc_destroy.argtypes = [vp]
    lib.pcc_destroy.restype = None
    lib.pcc_last_error.argtypes = [vp]
    lib.pcc_last_error.restype = ctypes.c_char_p
    lib.pcc_version.argtypes = []
    lib.pcc_version.restype = ctypes.c_char_p
    lib.pcc_device_bytes_in_use.argtypes = [vp]
    lib.pcc_device_bytes_in_use.restype = ctypes.c_uint64
    lib.pcc_device_peak_bytes.argtypes = [vp, ctypes.c_int32]
    lib.pcc_device_peak_bytes.restype = ctypes.c_uint64
    lib.pcc_cluster_batch.argtypes = [ctypes.c_int, ctypes.c_uint32, vp, P(PccConfig), ctypes.c_uint32,
                                      vp, ctypes.c_uint32, ctypes.c_uint64, vp, vp, P(ctypes.c_double)]
    lib.pcc_cluster_batch.restype = ctypes.c_int
    lib.pcc_set_detailed_timing.argtypes = [vp, ctypes.c_int32]
    lib.pcc_set_detailed_timing.restype = None
    lib.pcc_set_launch_tuning.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float]
    lib.pcc_set_launch_tuning.restype = ctypes.c_int32
    lib.pcc_cluster_union.argtypes = [vp, ctypes.c_uint32, vp, vp, ctypes.c_uint32, vp, ctypes.c_uint64, vp, vp,
                                      vp]
    lib.pcc_cluster_union.restype = ctypes.c_int
    lib.pcc_server_create.argtypes = [P(vp), ctypes.c_int, ctypes.c_uint32, ctypes.c_uint64]
    lib.pcc_server_create.restype = ctypes.c_int
    lib.pcc_server_submit.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint64, P(ctypes.c_uint64),
                                      P(ctypes.c_uint32), P(ctypes.c_float), P(ctypes.c_double),
                                      P(PccConfig), ctypes.c_int32, P(ctypes.c_uint64)]
    lib.pcc_server_submit.restype = ctypes.c_int
    lib.pcc_server_wait.argtypes = [vp, ctypes.c_uint64, ctypes.c_int32, P(ctypes.c_uint32), P(PccStats),
                                    P(ctypes.c_double), P(ctypes.c_double)]
    lib.pcc_server_wait.restype = ctypes.c_int
    lib.pcc_server_destroy.argtypes = [vp]
    lib.pcc_server_destroy.restype = None
    lib.pcc_request_bytes_estimate.argtypes = [ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int32]
    lib.pcc_request_bytes_estimate.restype = ctypes.c_uint64
    lib.pcc_config_default.argtypes = [P(PccConfig)]
    lib.pcc_config_default.restype = None
    lib.pcc_graph_upload.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint64,
                                     P(ctypes.c_uint64), P(ctypes.c_uint32),
                                     P(ctypes.c_float), P(vp)]
    lib.pcc_graph_upload.restype = ctypes.c_int
    lib.pcc_graph_upload_device.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint64,
                                            vp, vp, vp, P(vp)]
    lib.pcc_graph_upload_device.restype = ctypes.c_int
    lib.pcc_graph_free.argtypes = [vp, vp]
    lib.pcc_graph_free.restype = None
    lib.pcc_graph_info.argtypes = [vp, P(ctypes.c_uint32), P(ctypes.c_uint64),
                                   P(ctypes.c_int32)]
    lib.pcc_graph_info.restype = ctypes.c_int
    lib.pcc_graph_download.argtypes = [vp, vp, P(ctypes.c_uint64),
                                       P(ctypes.c_uint32), P(ctypes.c_float)]
    lib.pcc_graph_download.restype = ctypes.c_int
    lib.pcc_graph_node_weights.argtypes = [vp, vp, P(ctypes.c_double)]
    lib.pcc_graph_node_weights.restype = ctypes.c_int
    lib.pcc_correlation_cluster.argtypes = [vp, vp, P(PccConfig), P(ctypes.c_double),
                                            P(ctypes.c_uint32), P(ctypes.c_uint32),
                                            P(PccStats)]
    lib.pcc_correlation_cluster.restype = ctypes.c_int
    lib.pcc_modularity_cluster.argtypes = [vp, vp, P(PccConfig), P(ctypes.c_uint32),
                                           P(ctypes.c_uint32), P(PccStats)]
    lib.pcc_modularity_cluster.restype = ctypes.c_int
    lib.pcc_cluster_host_csr.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint64,
                                         P(ctypes.c_uint64), P(ctypes.c_uint32),
                                         P(ctypes.c_float), P(PccConfig), ctypes.c_int32,
                                         P(ctypes.c_double), P(ctypes.c_uint32),
                                         P(PccStats)]
    lib.pcc_cluster_host_csr.restype = ctypes.c_int
    lib.pcc_objective.argtypes = [vp, vp, P(PccConfig), P(ctypes.c_double),
                                  P(ctypes.c_uint32), P(ctypes.c_double)]
    lib.pcc_objective.restype = ctypes.c_int
    lib.pcc_modularity.argtypes = [vp, vp, ctypes.c_double, P(ctypes.c_uint32),
                                   P(ctypes.c_double)]
    lib.pcc_modularity.restype = ctypes.c_int
    lib.pcc_compare_communities.argtypes = [vp, ctypes.c_uint32, P(ctypes.c_uint32), ctypes.c_uint32,
                                            P(ctypes.c_uint64), P(ctypes.c_uint32), P(ctypes.c_double),
                                            P(ctypes.c_double), P(PccCommunityScores)]
    lib.pcc_compare_communities.restype = ctypes.c_int
    lib.pcc_best_moves.argtypes = [vp, vp, P(PccConfig), P(ctypes.c_uint32),
                                   P(ctypes.c_uint32), P(ctypes.c_double),
                                   P(ctypes.c_double), P(ctypes.c_uint32),
                                   P(ctypes.c_double), P(ctypes.c_uint32)]
    lib.pcc_best_moves.restype = ctypes.c_int
    lib.pcc_compress.argtypes = [vp, vp, P(ctypes.c_uint32), P(ctypes.c_double), P(vp)]
    lib.pcc_compress.restype = ctypes.c_int
    lib.pcc_graph_parse_gbbs.argtypes = [vp, ctypes.c_char_p, ctypes.c_uint64, ctypes.c_int32, P(vp)]
    lib.pcc_graph_parse_gbbs.restype = ctypes.c_int
    lib.pcc_graph_read_gbbs.argtypes = [vp, ctypes.c_char_p, ctypes.c_int32, P(vp)]
    lib.pcc_graph_read_gbbs.restype = ctypes.c_int
    lib.pcc_format_clustering.argtypes = [vp, ctypes.c_uint32, P(ctypes.c_uint32), ctypes.c_char_p,
                                          ctypes.c_uint64, P(ctypes.c_uint64)]
    lib.pcc_format_clustering.restype = ctypes.c_int
    lib.pcc_write_clustering.argtypes = [vp, ctypes.c_char_p, ctypes.c_uint32, P(ctypes.c_uint32)]
    lib.pcc_write_clustering.restype = ctypes.c_int
    _lib = lib
    return lib


class Context:
    """One GPU context (device, stream, memory pool).  Owns uploaded graphs."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0):
        self.lib = load_library()
        self._h = ctypes.c_void_p()
        self.detailed_timing = False
        st = self.lib.pcc_create(ctypes.byref(self._h), device, hbm_budget_bytes)
        if st != 0:
            raise PccError(st, "pcc_create failed (no usable GPU?)")

    def close(self):
        if self._h:
            self.lib.pcc_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def check(self, st: int):
        if st != 0:
            msg = self.lib.pcc_last_error(self._h)
            raise PccError(st, msg.decode() if msg else "")

    def set_detailed_timing(self, on: bool):
        """pcc_set_detailed_timing: host-driven rounds with per-phase and
        per-kernel-family CUDA events (on), or the device-side round loop
        (off, the default)."""
        self.lib.pcc_set_detailed_timing(self._h, 1 if on else 0)
        self.detailed_timing = bool(on)

    def set_launch_tuning(self, group_max_degree: int = 0, cta_min_degree: int = 0, grid_waves: float = 0.0):
        """pcc_set_launch_tuning: lane-group bins above group_max_degree on
        the warp kernel, certified warp bins above cta_min_degree on one CTA
        per vertex, grid_waves waves of resident CTAs per best-move launch;
        (0, 0, 0) returns to the compiled-in table."""
        self.check(self.lib.pcc_set_launch_tuning(self._h, int(group_max_degree), int(cta_min_degree),
                                                  float(grid_waves)))

    def bytes_in_use(self) -> int:
        return int(self.lib.pcc_device_bytes_in_use(self._h))

    def upload(self, g: CsrGraph) -> "DeviceGraph":
        off = np.ascontiguousarray(g.offsets, dtype=np.uint64)
        nbr = np.ascontiguousarray(g.neighbors, dtype=np.uint32)
        w = None if g.weights is None else np.ascontiguousarray(g.weights, dtype=np.float32)
        h = ctypes.c_void_p()
        self.check(self.lib.pcc_graph_upload(
            self._h, g.n, g.m, _ptr(off, ctypes.c_uint64), _ptr(nbr, ctypes.c_uint32),
            _ptr(w, ctypes.c_float), ctypes.byref(h)))
        return DeviceGraph(self, h)


    def parse_gbbs(self, text: bytes, float_weighted: bool) -> "DeviceGraph":
        """pcc_graph_parse_gbbs: GBBS adjacency text (bytes) parsed on the
        device into a resident graph."""
        h = ctypes.c_void_p()
        self.check(self.lib.pcc_graph_parse_gbbs(self._h, text, len(text), 1 if float_weighted else 0,
                                                 ctypes.byref(h)))
        return DeviceGraph(self, h)

    def read_gbbs(self, path: str, float_weighted: bool) -> "DeviceGraph":
        """pcc_graph_read_gbbs: a GBBS adjacency file parsed on the device."""
        h = ctypes.c_void_p()
        self.check(self.lib.pcc_graph_read_gbbs(self._h, os.fsencode(path), 1 if float_weighted else 0,
                                                ctypes.byref(h)))
        return DeviceGraph(self, h)

    def format_clustering(self, labels) -> bytes:
        """pcc_format_clustering: the clustering file's text (WriteClustering
        format) for labels (cluster index per node)."""
        lab = np.ascontiguousarray(labels, dtype=np.uint32)
        length = ctypes.c_uint64()
        self.check(self.lib.pcc_format_clustering(self._h, lab.size, _ptr(lab, ctypes.c_uint32), None, 0,
                                                  ctypes.byref(length)))
        buf = ctypes.create_string_buffer(max(int(length.value), 1))
        self.check(self.lib.pcc_format_clustering(self._h, lab.size, _ptr(lab, ctypes.c_uint32), buf,
                                                  length.value, ctypes.byref(length)))
        return buf.raw[:int(length.value)]

    def write_clustering(self, path: str, labels) -> None:
        """pcc_write_clustering: WriteClustering formatted on the device."""
        lab = np.ascontiguousarray(labels, dtype=np.uint32)
        self.check(self.lib.pcc_write_clustering(self._h, os.fsencode(path), lab.size, _ptr(lab, ctypes.c_uint32)))


class DeviceGraph:
    """A graph resident in HBM (pcc_graph*)."""

    def __init__(self, ctx: Context, handle: ctypes.c_void_p):
        self.ctx = ctx
        self._h = handle

    @property
    def handle(self):
        return self._h

    def free(self):
        if self._h:
            self.ctx.lib.pcc_graph_free(self.ctx.handle, self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            if self.ctx.handle:
                self.free()
        except Exception:
            pass

    def info(self):
        n = ctypes.c_uint32()
        m = ctypes.c_uint64()
        hw = ctypes.c_int32()
        self.ctx.check(self.ctx.lib.pcc_graph_info(self._h, ctypes.byref(n), ctypes.byref(m),
                                                   ctypes.byref(hw)))
        return int(n.value), int(m.value), bool(hw.value)

    def download(self) -> CsrGraph:
        n, m, hw = self.info()
        off = np.empty(n + 1, dtype=np.uint64)
        nbr = np.empty(m, dtype=np.uint32)
        w = np.empty(m, dtype=np.float32) if hw else None
        self.ctx.check(self.ctx.lib.pcc_graph_download(
            self.ctx.handle, self._h, _ptr(off, ctypes.c_uint64), _ptr(nbr, ctypes.c_uint32),
            _ptr(w, ctypes.c_float)))
        return CsrGraph(off, nbr, w)

    def node_weights(self) -> np.ndarray:
        n, _, _ = self.info()
        out = np.empty(n, dtype=np.float64)
        self.ctx.check(self.ctx.lib.pcc_graph_node_weights(self.ctx.handle, self._h,
                                                           _ptr(out, ctypes.c_double)))
        return out


def _u32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.uint32)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def correlation_cluster(g: DeviceGraph, config: PccConfig, node_weights=None,
                        initial_labels=None):
    """Returns (labels uint32[n], stats dict).  labels[v] = index of v's
    cluster in the reference's Clustering order."""
    n, _, _ = g.info()
    out = np.empty(n, dtype=np.uint32)
    st = PccStats()
    k = _f64(node_weights)
    lab = _u32(initial_labels)
    g.ctx.check(g.ctx.lib.pcc_correlation_cluster(
        g.ctx.handle, g.handle, ctypes.byref(config), _ptr(k, ctypes.c_double),
        _ptr(lab, ctypes.c_uint32), _ptr(out, ctypes.c_uint32), ctypes.byref(st)))
    return out, st.as_dict()


def modularity_cluster(g: DeviceGraph, config: PccConfig, initial_labels=None):
    n, _, _ = g.info()
    out = np.empty(n, dtype=np.uint32)
    st = PccStats()
    lab = _u32(initial_labels)
    g.ctx.check(g.ctx.lib.pcc_modularity_cluster(
        g.ctx.handle, g.handle, ctypes.byref(config), _ptr(lab, ctypes.c_uint32),
        _ptr(out, ctypes.c_uint32), ctypes.byref(st)))
    return out, st.as_dict()


def cluster_host_csr(ctx: Context, g: CsrGraph, config: PccConfig, objective: int = 0,
                     node_weights=None):
    """End-to-end call on host buffers (upload + cluster + download)."""
    off = np.ascontiguousarray(g.offsets, dtype=np.uint64)
    nbr = np.ascontiguousarray(g.neighbors, dtype=np.uint32)
    w = None if g.weights is None else np.ascontiguousarray(g.weights, dtype=np.float32)
    out = np.empty(g.n, dtype=np.uint32)
    st = PccStats()
    k = _f64(node_weights)
    ctx.check(ctx.lib.pcc_cluster_host_csr(
        ctx.handle, g.n, g.m, _ptr(off, ctypes.c_uint64), _ptr(nbr, ctypes.c_uint32),
        _ptr(w, ctypes.c_float), ctypes.byref(config), objective, _ptr(k, ctypes.c_double),
        _ptr(out, ctypes.c_uint32), ctypes.byref(st)))
    return out, st.as_dict()


def objective(g: DeviceGraph, config: PccConfig, labels, node_weights=None) -> float:
    out = ctypes.c_double()
    lab = _u32(labels)
    k = _f64(node_weights)
    g.ctx.check(g.ctx.lib.pcc_objective(g.ctx.handle, g.handle, ctypes.byref(config),
                                        _ptr(k, ctypes.c_double), _ptr(lab, ctypes.c_uint32),
                                        ctypes.byref(out)))
    return float(out.value)


def modularity(g: DeviceGraph, resolution: float, labels) -> float:
    out = ctypes.c_double()
    lab = _u32(labels)
    g.ctx.check(g.ctx.lib.pcc_modularity(g.ctx.handle, g.handle, resolution,
                                         _ptr(lab, ctypes.c_uint32), ctypes.byref(out)))
    return float(out.value)


def compare_communities(ctx: "Context", labels, communities=None, offsets=None, members=None):
    """Ground-truth scoring (CompareCommunities, cluster-in-memory_main.cc:
    172-225) on the device.  communities: a list of vertex-id sequences, or
    offsets (uint64[C+1]) and members (uint32) in CSR form.  Returns (scores
    dict, precision per community, recall per community)."""
    lab = _u32(labels)
    if communities is not None:
        sizes = [len(c) for c in communities]
        offsets = np.zeros(len(communities) + 1, np.uint64)
        offsets[1:] = np.cumsum(sizes, dtype=np.uint64)
        members = (np.concatenate([np.asarray(c, np.uint32) for c in communities]) if sum(sizes)
                   else np.zeros(1, np.uint32))
    off = np.ascontiguousarray(offsets, np.uint64)
    mem = np.ascontiguousarray(members if len(members) else np.zeros(1, np.uint32), np.uint32)
    nc = off.size - 1
    prec = np.zeros(max(nc, 1), np.float64)
    rec = np.zeros(max(nc, 1), np.float64)
    out = PccCommunityScores()
    ctx.check(ctx.lib.pcc_compare_communities(ctx.handle, lab.size, _ptr(lab, ctypes.c_uint32), nc,
                                              _ptr(off, ctypes.c_uint64), _ptr(mem, ctypes.c_uint32),
                                              _ptr(prec, ctypes.c_double), _ptr(rec, ctypes.c_double),
                                              ctypes.byref(out)))
    scores = {name: getattr(out, name) for name, _ in out._fields_}
    return scores, prec[:nc], rec[:nc]


def best_moves(g: DeviceGraph, config: PccConfig, cluster_ids, cluster_sizes, node_weights,
               cluster_weights):
    """One sync best-move pass over all vertices; returns (targets, values, moves)."""
    n, _, _ = g.info()
    C, s = _u32(cluster_ids), _u32(cluster_sizes)
    k, K = _f64(node_weights), _f64(cluster_weights)
    t = np.empty(n, dtype=np.uint32)
    v = np.empty(n, dtype=np.float64)
    mv = np.empty(n, dtype=np.uint32)
    g.ctx.check(g.ctx.lib.pcc_best_moves(
        g.ctx.handle, g.handle, ctypes.byref(config), _ptr(C, ctypes.c_uint32),
        _ptr(s, ctypes.c_uint32), _ptr(k, ctypes.c_double), _ptr(K, ctypes.c_double),
        _ptr(t, ctypes.c_uint32), _ptr(v, ctypes.c_double), _ptr(mv, ctypes.c_uint32)))
    return t, v, mv


def compress(g: DeviceGraph, cluster_ids, node_weights=None) -> DeviceGraph:
    C = _u32(cluster_ids)
    k = _f64(node_weights)
    h = ctypes.c_void_p()
    g.ctx.check(g.ctx.lib.pcc_compress(g.ctx.handle, g.handle, _ptr(C, ctypes.c_uint32),
                                       _ptr(k, ctypes.c_double), ctypes.byref(h)))
    return DeviceGraph(g.ctx, h)


class _BatchGraph(ctypes.Structure):
    _fields_ = [("n", ctypes.c_uint32), ("m", ctypes.c_uint64), ("offsets", ctypes.c_void_p),
                ("neighbors", ctypes.c_void_p), ("weights", ctypes.c_void_p), ("node_weights", ctypes.c_void_p)]


def _batch_arrays(graphs, node_weights):
    """The pcc_batch_graph array (and the numpy arrays it points into) and
    one label array per graph."""
    ng = len(graphs)
    keep = []
    arr = (_BatchGraph * max(ng, 1))()
    labels = []
    for i, g in enumerate(graphs):
        off = np.ascontiguousarray(g.offsets, dtype=np.uint64)
        nbr = np.ascontiguousarray(g.neighbors, dtype=np.uint32)
        w = None if g.weights is None else np.ascontiguousarray(g.weights, dtype=np.float32)
        k = None if node_weights is None or node_weights[i] is None else \
            np.ascontiguousarray(node_weights[i], dtype=np.float64)
        keep.append((off, nbr, w, k))
        arr[i].n = g.n
        arr[i].m = g.m
        arr[i].offsets = off.ctypes.data
        arr[i].neighbors = nbr.ctypes.data if g.m else None
        arr[i].weights = None if w is None else w.ctypes.data
        arr[i].node_weights = None if k is None else k.ctypes.data
        labels.append(np.empty(max(g.n, 1), dtype=np.uint32))
    return arr, keep, labels


def cluster_union(ctx: "Context", graphs: Sequence[CsrGraph], configs, objectives=None, node_weights=None,
                  max_union_entries: int = 0):
    """pcc_cluster_union: independent graphs as disjoint-union engine runs on
    `ctx`.  configs: one PccConfig or one per graph (differing in resolution
    only); objectives: None (correlation) or 0/1 per graph.  Returns (label
    arrays, per-graph stats dicts, batch stats dict)."""
    lib = load_library()
    ng = len(graphs)
    arr, keep, labels = _batch_arrays(graphs, node_weights)
    if isinstance(configs, PccConfig):
        cfgs = (PccConfig * 1)(configs)
        ncfg = 1
    else:
        cfgs = (PccConfig * ng)(*configs)
        ncfg = ng
    objs = None if objectives is None else np.ascontiguousarray(objectives, dtype=np.int32)
    outs = (ctypes.c_void_p * max(ng, 1))(*[lab.ctypes.data for lab in labels])
    stats = (PccStats * max(ng, 1))()
    tot = PccStats()
    st = lib.pcc_cluster_union(ctx.handle, ng, ctypes.cast(arr, ctypes.c_void_p), ctypes.cast(cfgs, ctypes.c_void_p),
                               ncfg, None if objs is None else objs.ctypes.data, max_union_entries,
                               ctypes.cast(outs, ctypes.c_void_p), ctypes.cast(stats, ctypes.c_void_p),
                               ctypes.byref(tot))
    del keep
    ctx.check(st)
    return [labels[i][:graphs[i].n] for i in range(ng)], [stats[i].as_dict() for i in range(ng)], tot.as_dict()


def cluster_batch(graphs: Sequence[CsrGraph], configs, objectives=None, node_weights=None, concurrency: int = 16,
                  hbm_budget: int = 0, device: int = 0):
    """pcc_cluster_batch: clusters independent graphs on one GPU (disjoint
    unions for one shared correlation config, else the concurrent worker
    pool).  configs: one PccConfig or one per graph; objectives: None
    (correlation) or 0/1 per graph.  Returns (list of label arrays, list of
    stats dicts, wall ms)."""
    lib = load_library()
    ng = len(graphs)
    arr, keep, labels = _batch_arrays(graphs, node_weights)
    if isinstance(configs, PccConfig):
        cfgs = (PccConfig * 1)(configs)
        ncfg = 1
    else:
        cfgs = (PccConfig * ng)(*configs)
        ncfg = ng
    objs = None if objectives is None else np.ascontiguousarray(objectives, dtype=np.int32)
    outs = (ctypes.c_void_p * max(ng, 1))(*[lab.ctypes.data for lab in labels])
    stats = (PccStats * max(ng, 1))()
    wall = ctypes.c_double(0)
    st = lib.pcc_cluster_batch(device, ng, ctypes.cast(arr, ctypes.c_void_p), cfgs, ncfg,
                               None if objs is None else objs.ctypes.data, concurrency, hbm_budget,
                               ctypes.cast(outs, ctypes.c_void_p), ctypes.cast(stats, ctypes.c_void_p),
                               ctypes.byref(wall))
    if st != 0:
        raise PccError(st, "pcc_cluster_batch failed")
    return [labels[i][:graphs[i].n] for i in range(ng)], [stats[i].as_dict() for i in range(ng)], wall.value


class Server:
    """The serving loop (pcc_server_*): submit requests, wait for results."""

    def __init__(self, slots: int = 8, hbm_budget: int = 0, device: int = 0):
        self.lib = load_library()
        self.handle = ctypes.c_void_p()
        st = self.lib.pcc_server_create(ctypes.byref(self.handle), device, slots, hbm_budget)
        if st != 0:
            raise PccError(st, "pcc_server_create failed")
        self.sizes = {}

    def submit(self, g: CsrGraph, config: PccConfig, objective: int = 0, node_weights=None) -> int:
        off = np.ascontiguousarray(g.offsets, dtype=np.uint64)
        nbr = np.ascontiguousarray(g.neighbors, dtype=np.uint32)
        w = None if g.weights is None else np.ascontiguousarray(g.weights, dtype=np.float32)
        k = None if node_weights is None else np.ascontiguousarray(node_weights, dtype=np.float64)
        t = ctypes.c_uint64(0)
        st = self.lib.pcc_server_submit(self.handle, g.n, g.m, _ptr(off, ctypes.c_uint64),
                                        _ptr(nbr, ctypes.c_uint32), _ptr(w, ctypes.c_float),
                                        _ptr(k, ctypes.c_double), ctypes.byref(config), objective, ctypes.byref(t))
        if st != 0:
            raise PccError(st, "pcc_server_submit failed")
        self.sizes[t.value] = g.n
        return t.value

    def wait(self, ticket: int, wait_ms: int = -1):
        """Returns (labels, stats dict, latency ms, queue ms), or None while
        the request is still queued or running (wait_ms >= 0)."""
        n = self.sizes[ticket]
        lab = np.empty(max(n, 1), dtype=np.uint32)
        stt = PccStats()
        lat = ctypes.c_double(0)
        qms = ctypes.c_double(0)
        st = self.lib.pcc_server_wait(self.handle, ticket, wait_ms, _ptr(lab, ctypes.c_uint32), ctypes.byref(stt),
                                      ctypes.byref(lat), ctypes.byref(qms))
        if st == 4:  # DEADLINE_EXCEEDED
            return None
        del self.sizes[ticket]
        if st != 0:
            raise PccError(st, "request failed")
        return lab[:n], stt.as_dict(), lat.value, qms.value

    def close(self):
        if self.handle:
            self.lib.pcc_server_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def request_bytes_estimate(n: int, m: int, weighted: bool) -> int:
    return int(load_library().pcc_request_bytes_estimate(n, m, 1 if weighted else 0))


def labels_to_clustering(labels: Sequence[int]) -> List[List[int]]:
    """InMemoryClusterer::Clustering from group labels (groups by label)."""
    labels = np.asarray(labels)
    if labels.size == 0:
        return []
    order = np.argsort(labels, kind="stable")
    bounds = np.flatnonzero(np.diff(labels[order])) + 1
    return [list(map(int, grp)) for grp in np.split(order, bounds)]


class ParallelCorrelationClustererGB300:
    """Drop-in for ParallelCorrelationClusterer: holds a device graph and
    clusters it with ``cluster(config)`` / ``refine_clusters(config, clustering)``."""

    objective_kind = 0

    def __init__(self, ctx: Optional[Context] = None):
        self.ctx = ctx or Context()
        self.graph: Optional[DeviceGraph] = None

    def set_graph(self, g: CsrGraph):
        if self.graph is not None:
            self.graph.free()
        self.graph = self.ctx.upload(g)

    def _run(self, config: PccConfig, initial_labels):
        return correlation_cluster(self.graph, config, None, initial_labels)

    def cluster(self, config: PccConfig) -> List[List[int]]:
        labels, self.last_stats = self._run(config, None)
        return labels_to_clustering(labels)

    def refine_clusters(self, config: PccConfig, clustering: List[List[int]]) -> List[List[int]]:
        n, _, _ = self.graph.info()
        init = np.empty(n, dtype=np.uint32)
        seen = np.zeros(n, dtype=bool)
        for cid, members in enumerate(clustering):
            for v in members:
                if seen[v]:
                    raise PccError(3, f"node {v} appears twice in the initial clustering")
                seen[v] = True
                init[v] = cid
        if not seen.all():
            raise PccError(3, "initial clustering must cover every node exactly once")
        labels, self.last_stats = self._run(config, init)
        return labels_to_clustering(labels)


class ParallelModularityClustererGB300(ParallelCorrelationClustererGB300):
    """Drop-in for ParallelModularityClusterer."""

    objective_kind = 1

    def _run(self, config: PccConfig, initial_labels):
        return modularity_cluster(self.graph, config, initial_labels)
