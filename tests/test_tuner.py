"""CPU tests of the launch-shape autotuner's host logic: the choice of a size
class's shape from timed workloads, and the table it writes (the one the
library compiles in)."""

import os
import re

import tune_launch as T

CSRC = os.path.join(os.path.dirname(T.__file__), "csrc")

SHAPES = [f"{g}/{c}/{w}" for g in T.GROUP_MAX for c in T.CTA_MIN for w in T.WAVES]


def _rows(ms_by_shape):
    return {k: ms_by_shape.get(k, 10.0) for k in SHAPES}


def test_pick_best_weighs_workloads_by_their_default_time():
    """A 20% win on a 10 ms workload beats a 4% loss on a 100 ms one: the
    score is the sum of time / default time, not of absolute times."""
    fast = "16/512/2.0"
    small = _rows({T.DEFAULT: 10.0, fast: 8.0})
    big = {k: 100.0 for k in SHAPES}
    big[fast] = 104.0
    best, score = T.pick_best({"small": small, "big": big})
    assert best == fast
    assert abs(score[fast] - (0.8 + 1.04)) < 1e-12
    assert abs(score[T.DEFAULT] - 2.0) < 1e-12


def test_pick_best_keeps_the_default_on_ties():
    flat = {k: 10.0 for k in SHAPES}
    best, _ = T.pick_best({"a": flat, "b": dict(flat)})
    assert best == T.DEFAULT
    # Another shape as fast as the default, not faster: still the default.
    tie = dict(flat)
    tie["8/256/0.5"] = 10.0
    assert T.pick_best({"a": tie})[0] == T.DEFAULT


def test_pick_best_covers_every_shape():
    _, score = T.pick_best({"a": {k: 1.0 + i for i, k in enumerate(SHAPES)}})
    assert sorted(score) == sorted(SHAPES)
    assert len(SHAPES) == 27


def test_write_table_reproduces_the_committed_table(tmp_path):
    """The committed csrc/tuning_table.cuh is exactly what the writer emits
    for its rows, and its rows are valid launch shapes in ascending size
    classes ending with the catch-all row."""
    path = os.path.join(CSRC, "tuning_table.cuh")
    text = open(path).read()
    rows = [(int(n), int(g), int(c), float(w))
            for n, g, c, w in re.findall(r"\{(\d+)u, (\d+)u, (\d+)u, ([0-9.]+)f\}", text)]
    assert len(rows) >= 2
    out = tmp_path / "table.cuh"
    T.write_table(str(out), rows)
    assert out.read_text() == text
    sizes = [r[0] for r in rows]
    assert sizes == sorted(sizes) and sizes[-1] == 0xFFFFFFFF
    for _, g, c, w in rows:
        assert g in (4, 8, 16, 32)
        assert c in (64, 128, 256, 512, 1000)
        assert 0.125 <= w <= 16.0
