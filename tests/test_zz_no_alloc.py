"""pcc_best_moves_static (the entry point that allocates no device memory)
against pcc_best_moves on the same states, two calls in a row.

Collected last so it also runs after every other GPU test in one process;
it passes alone in a fresh process as well.
"""

import ctypes

import numpy as np
import pytest

import pcc_gb300 as P
import pcc_graphs as G
from conftest import rand_state

pytestmark = pytest.mark.gpu

REL_TOL = 1e-9
MAX_DEGREE_LIMIT = (1 << 20) - 1


def _fn(lib):
    fn = lib.pcc_best_moves_static
    fn.restype = ctypes.c_int
    vp = ctypes.c_void_p
    fn.argtypes = [ctypes.c_uint32, vp, vp, vp, vp, vp, vp, ctypes.c_double, ctypes.c_double, vp,
                   ctypes.c_uint32, ctypes.c_uint32, vp, vp, vp]
    return fn


def _graphs():
    out = {}
    g, _ = G.sbm(2000, 20, 0.05, 0.001, 7)
    out["sbm2k"] = g
    out["rmat14"] = G.rmat(14, 16, seed=3)      # hub rows (degree > 1000)
    lg, _ = G.lfr(20000, mean_degree=20, dmax=1500, seed=9)
    out["lfr20k_real"] = lg                     # real weights
    rng = np.random.default_rng(11)
    gi, _ = G.sbm(3000, 10, 0.03, 0.002, 13)
    src = np.repeat(np.arange(gi.n), np.diff(gi.offsets).astype(np.int64))
    keep = src < gi.neighbors
    w = rng.integers(1, 6, size=int(keep.sum())).astype(np.float32)
    out["sbm3k_int"] = P.CsrGraph.from_edges(gi.n, src[keep], gi.neighbors[keep].astype(np.int64), w)
    return out


class _Dev:
    """Device copies of a graph and a clustering state (torch-owned memory)."""

    def __init__(self, torch, g, C, k, K):
        dev = "cuda:0"
        self.off = torch.from_numpy(g.offsets.view(np.int64).copy()).to(dev)
        self.nbr = torch.from_numpy(g.neighbors.view(np.int32).copy()).to(dev)
        self.w = None if g.weights is None else torch.from_numpy(g.weights.copy()).to(dev)
        self.C = torch.from_numpy(C.view(np.int32).copy()).to(dev)
        self.k = torch.from_numpy(k.copy()).to(dev)
        self.K = torch.from_numpy(K.copy()).to(dev)

    def call(self, torch, fn, g, res, offset, verts=None, max_degree=None):
        nv = g.n if verts is None else int(verts.numel())
        t = torch.empty(max(nv, 1), dtype=torch.int32, device="cuda:0")
        v = torch.empty(max(nv, 1), dtype=torch.float64, device="cuda:0")
        md = int(g.degrees().max()) if max_degree is None else max_degree
        st = fn(g.n, self.off.data_ptr(), self.nbr.data_ptr(),
                None if self.w is None else self.w.data_ptr(), self.C.data_ptr(), self.k.data_ptr(),
                self.K.data_ptr(), res, offset, None if verts is None else verts.data_ptr(), nv, md,
                t.data_ptr(), v.data_ptr(), torch.cuda.current_stream().cuda_stream)
        return st, t[:nv].cpu().numpy().view(np.uint32), v[:nv].cpu().numpy()


@pytest.fixture(scope="module")
def setup(built):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ctx = P.Context(0)
    yield torch, ctx, _fn(ctx.lib), _graphs()
    ctx.close()


def _check(g, t_ref, v_ref, t, v):
    integral = g.weights is None or np.all(g.weights == np.round(g.weights))
    if integral:
        np.testing.assert_array_equal(t, t_ref)
        np.testing.assert_array_equal(v.view(np.uint64), v_ref.view(np.uint64))
    else:
        np.testing.assert_allclose(v, v_ref, rtol=REL_TOL, atol=1e-12)
        assert np.mean(t == t_ref) >= 0.999


@pytest.mark.parametrize("name", ["sbm2k", "rmat14", "lfr20k_real", "sbm3k_int"])
@pytest.mark.parametrize("nclusters_div", [1, 7, 300])
def test_static_matches_context_path(setup, name, nclusters_div):
    torch, ctx, fn, graphs = setup
    g = graphs[name]
    C, s, k, K = rand_state(g.n, max(1, g.n // nclusters_div), seed=nclusters_div)
    dg = ctx.upload(g)
    d = _Dev(torch, g, C, k, K)
    for res, off in ((0.01, 0.0), (0.3, 0.0), (0.05, 1.0)):
        cfg = P.make_config(resolution=res, edge_weight_offset=off)
        t_ref, v_ref, _ = P.best_moves(dg, cfg, C, s, k, K)
        for _ in range(2):   # the second call sees the scratch the first one left
            st, t, v = d.call(torch, fn, g, res, off)
            assert st == 0
            _check(g, t_ref, v_ref, t, v)
        # A vertex subset, in reverse order.
        verts = torch.arange(g.n - 1, -1, -3, dtype=torch.int32, device="cuda:0")
        st, t, v = d.call(torch, fn, g, res, off, verts=verts)
        assert st == 0
        idx = verts.cpu().numpy()
        _check(g, t_ref[idx], v_ref[idx], t, v)
    dg.free()


def test_static_limits(setup):
    torch, ctx, fn, graphs = setup
    g = graphs["rmat14"]
    C, s, k, K = rand_state(g.n, g.n // 7, seed=7)
    d = _Dev(torch, g, C, k, K)
    # Above the scratch limit: refused before any launch.
    st, _, _ = d.call(torch, fn, g, 0.01, 0.0, max_degree=MAX_DEGREE_LIMIT + 1)
    assert st == 11  # OUT_OF_RANGE
    # A stated max_degree below a listed vertex's degree.
    st, t, _ = d.call(torch, fn, g, 0.01, 0.0, max_degree=8)
    assert st == 11
    assert np.any(t == 0xFFFFFFFF)
    # A vertex id >= n.
    bad = torch.tensor([0, g.n + 5], dtype=torch.int32, device="cuda:0")
    st, _, _ = d.call(torch, fn, g, 0.01, 0.0, verts=bad)
    assert st == 3  # INVALID_ARGUMENT
    # The scratch is still clean: a normal call matches the context path.
    dg = ctx.upload(g)
    cfg = P.make_config(resolution=0.01)
    t_ref, v_ref, _ = P.best_moves(dg, cfg, C, s, k, K)
    st, t, v = d.call(torch, fn, g, 0.01, 0.0)
    assert st == 0
    _check(g, t_ref, v_ref, t, v)
    dg.free()
