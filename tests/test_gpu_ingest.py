"""Device-side GBBS ingest and clustering output against the host side.

* pcc_graph_parse_gbbs / pcc_graph_read_gbbs must give the graph the host
  reader (pcch_read_gbbs, the CLI's reader) gives on the same file, bit for
  bit (offsets, ids, float weights), and the same status code on bad input;
* weights must round exactly as strtof (libc, called through ctypes) on
  hard cases: exact float midpoints (ties to even), values a hair off a
  midpoint, subnormals, the overflow threshold, long digit strings;
* pcc_format_clustering / pcc_write_clustering must produce the reference's
  WriteClustering text (cluster-in-memory_main.cc:132-145).
"""

import ctypes
import math
import os
import random
import struct
from fractions import Fraction

import numpy as np
import pytest

import pcc_gb300 as P
import pcc_graphs as G

pytestmark = pytest.mark.gpu

_libc = ctypes.CDLL(None)
_libc.strtof.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_char_p)]
_libc.strtof.restype = ctypes.c_float


def _strtof_bits(tok: str) -> int:
    return struct.unpack("<I", struct.pack("<f", _libc.strtof(tok.encode(), None)))[0]


def _bits(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def _same_graph(got: P.CsrGraph, want: P.CsrGraph):
    assert got.n == want.n and got.m == want.m
    np.testing.assert_array_equal(got.offsets, want.offsets)
    np.testing.assert_array_equal(got.neighbors, want.neighbors)
    assert (got.weights is None) == (want.weights is None)
    if want.weights is not None:
        np.testing.assert_array_equal(_bits(got.weights), _bits(want.weights))


def _graphs():
    g1, _ = G.sbm(3000, 20, 0.02, 0.001, 5)
    g2, _ = G.lfr(20000, mean_degree=20, dmax=1500, seed=9)  # real weights
    g3 = G.rmat(14, 16, seed=3)                               # hubs
    g4 = P.CsrGraph(np.zeros(6, np.uint64), np.zeros(0, np.uint32), None)  # isolated vertices only
    return {"sbm3k": g1, "lfr20k": g2, "rmat14": g3, "isolated5": g4}


@pytest.mark.parametrize("name", ["sbm3k", "lfr20k", "rmat14", "isolated5"])
def test_parse_equals_host_reader(ctx, built, tmp_path, name):
    g = _graphs()[name]
    path = str(tmp_path / f"{name}.adj")
    G.write_gbbs(path, g)
    weighted = g.weights is not None
    want = G.read_gbbs_native(path, weighted)
    dg = ctx.read_gbbs(path, weighted)
    _same_graph(dg.download(), want)
    dg.free()
    with open(path, "rb") as f:
        dg = ctx.parse_gbbs(f.read(), weighted)
    _same_graph(dg.download(), want)
    # The device graph clusters exactly as an uploaded one.
    cfg = P.make_config(resolution=0.05, refine=True)
    lab_a, st_a = P.correlation_cluster(dg, cfg)
    du = ctx.upload(want)
    lab_b, st_b = P.correlation_cluster(du, cfg)
    np.testing.assert_array_equal(lab_a, lab_b)
    assert st_a["objective"] == st_b["objective"]
    dg.free()
    du.free()


def _weight_tokens():
    rng = random.Random(12345)
    toks = ["1", "1.0", "+1.5", "-2.25", ".5", "5.", "0", "-0", "0.000", "1e5", "1E+05", "2.5e-3", "123456789",
            "0.1", "0.2", "0.3", "3.14159265358979323846264338327950288419716939937510",
            "inf", "-inf", "INF", "Infinity", "-infinity", "nan", "NaN", "-nan",
            "1e39", "-1e39", "1e-46", "1e-45", "7e-46", "7.1e-46", "1.4e-45", "3.4028235e38", "3.4028236e38",
            "340282356779733661637539395458142568448", "340282356779733661637539395458142568447.999",
            "340282356779733661637539395458142568448.001",
            "1.17549435e-38", "1.1754942e-38", "00000000000000000000000123.456000000000000000000",
            "9007199254740993", "9007199254740993e-10", "1e22", "1e23", "4.9406564584124654e-324"]
    # Exact float midpoints (ties to even) and values just off them, normal
    # and subnormal, with long exact decimal expansions.
    for _ in range(300):
        e = rng.randint(-149, 127)
        mant = rng.randint(1, (1 << 24) - 1)
        f = Fraction(mant) * Fraction(2) ** (e - 23)
        if f > Fraction(struct.unpack("<f", struct.pack("<I", 0x7F7FFFFF))[0]):
            continue
        x = float(f)
        a = np.float32(x)
        b = np.nextafter(a, np.float32(np.inf))
        if not np.isfinite(b):
            continue
        mid = (Fraction(float(a)) + Fraction(float(b))) / 2
        for delta in (Fraction(0), Fraction(1, 10 ** 60) * mid, -Fraction(1, 10 ** 60) * mid):
            # The exact midpoint (its decimal expansion ends within 150
            # significant digits), or 120 digits of a value a hair off it.
            toks.append(_decimal(mid + delta, 150 if delta == 0 else 120))
    for _ in range(400):
        digits = "".join(rng.choice("0123456789") for _ in range(rng.randint(1, 30)))
        dot = rng.randint(0, len(digits))
        t = digits[:dot] + "." + digits[dot:] if rng.random() < 0.7 else digits
        if t == ".":
            t = "0"
        if rng.random() < 0.5:
            t += rng.choice("eE") + rng.choice(["", "+", "-"]) + str(rng.randint(0, 50))
        if rng.random() < 0.3:
            t = "-" + t
        toks.append(t)
    return toks


def _decimal(v: Fraction, sig: int) -> str:
    """Decimal string of a positive fraction: exact when its expansion ends
    within `sig` significant digits, else truncated there."""
    e = math.floor(math.log10(v.numerator) - math.log10(v.denominator))
    while Fraction(10) ** e > v:
        e -= 1
    while Fraction(10) ** (e + 1) <= v:
        e += 1
    scaled = v / Fraction(10) ** (e - sig + 1)
    q = scaled.numerator // scaled.denominator
    s = str(q).rstrip("0") or "0"
    return f"{s[0]}.{s[1:] or '0'}e{e}"


def test_weights_round_as_strtof(ctx, built):
    toks = _weight_tokens()
    m = len(toks)
    text = "WeightedAdjacencyGraph\n2\n%d\n0\n%d\n%s\n%s\n" % (m, m, "\n".join(["1"] * m), "\n".join(toks))
    dg = ctx.parse_gbbs(text.encode(), True)
    got = dg.download()
    dg.free()
    want = np.array([_strtof_bits(t) for t in toks], np.uint32)
    bad = [(t, hex(int(a)), hex(int(b))) for t, a, b in zip(toks, _bits(got.weights), want) if a != b]
    assert not bad, bad[:10]


def _host_status(path, weighted):
    try:
        G.read_gbbs_native(path, weighted)
        return 0
    except P.PccError as e:
        return e.code


@pytest.mark.parametrize("text,weighted", [
    ("", False),
    ("Graph\n1\n0\n0\n", False),
    ("AdjacencyGraph\n2\n2\n0\n1\n1\n0\n", True),        # float_weighted mismatch
    ("AdjacencyGraph\nx\n2\n", False),
    ("AdjacencyGraph\n2\n2\n0\n1a\n1\n0\n", False),       # bad offset token
    ("AdjacencyGraph\n2\n2\n0\n1\n1\n", False),           # missing id
    ("AdjacencyGraph\n2\n2\n0\n1\n1\n2\n", False),        # id >= n
    ("AdjacencyGraph\n2\n2\n1\n1\n1\n0\n", False),        # offsets start at 1
    ("AdjacencyGraph\n3\n2\n0\n2\n1\n1\n0\n", False),     # decreasing offsets
    ("AdjacencyGraph\n2\n2\n0\n1\n1\n0\n77 trailing tokens\n", False),  # ignored
    ("WeightedAdjacencyGraph\n2\n2\n0\n1\n1\n0\n1.5\n", True),           # missing weight
    ("WeightedAdjacencyGraph\n2\n2\n0\n1\n1\n0\n1.5\n1e\n", True),       # bad weight
    ("WeightedAdjacencyGraph\n2\n2\n0\n1\n1\n0\n1.5\n1.2.3\n", True),
    ("WeightedAdjacencyGraph\n2\n2\n0\n1\n1\n0\n1\n1.0\n", True),        # all ones -> unit
    ("WeightedAdjacencyGraph\n2\n2\n0\n1\n1\n0\n-0.5\ninf\n", True),
    ("AdjacencyGraph\n0\n0\n", False),
    ("AdjacencyGraph \t\r\n 3\f\v2 0 1 1\n\n1 0", False),
])
def test_errors_match_host_reader(ctx, built, tmp_path, text, weighted):
    path = str(tmp_path / "g.adj")
    with open(path, "w") as f:
        f.write(text)
    want = _host_status(path, weighted)
    try:
        dg = ctx.read_gbbs(path, weighted)
        got = 0
        ref = G.read_gbbs_native(path, weighted)
        _same_graph(dg.download(), ref)
        dg.free()
    except P.PccError as e:
        got = e.code
    assert got == want, (text, got, want)


def test_hex_weights_are_rejected_by_the_device_reader(ctx, built):
    text = b"WeightedAdjacencyGraph\n2\n2\n0\n1\n1\n0\n0x1p3\n1.5\n"
    with pytest.raises(P.PccError) as e:
        ctx.parse_gbbs(text, True)
    assert e.value.code == 3 and "device reader" in e.value.message


def _host_clustering_text(labels) -> bytes:
    labels = np.asarray(labels)
    if labels.size == 0:
        return b""
    out = []
    for c in range(int(labels.max()) + 1):
        out.append("".join(f"{v}\t" for v in np.flatnonzero(labels == c)) + "\n")
    return "".join(out).encode()


@pytest.mark.parametrize("case", ["clustered", "sparse_labels", "singletons", "one", "empty"])
def test_format_clustering_matches_write_clustering(ctx, built, tmp_path, case):
    rng = np.random.default_rng(4)
    if case == "clustered":
        g, _ = G.sbm(5000, 25, 0.03, 0.001, 2)
        labels, _ = P.correlation_cluster(ctx.upload(g), P.make_config(resolution=0.05, refine=True))
    elif case == "sparse_labels":
        labels = rng.choice([0, 3, 7, 1000], size=20000).astype(np.uint32)
    elif case == "singletons":
        labels = rng.permutation(123457).astype(np.uint32)
    elif case == "one":
        labels = np.zeros(1, np.uint32)
    else:
        labels = np.zeros(0, np.uint32)
    want = _host_clustering_text(labels)
    assert ctx.format_clustering(labels) == want
    path = str(tmp_path / "out.txt")
    ctx.write_clustering(path, labels)
    with open(path, "rb") as f:
        assert f.read() == want
