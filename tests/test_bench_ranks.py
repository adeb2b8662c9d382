"""The multi-process path of bench.py on CPU: N replicas report the
slowest rank's time and the sum of their edge visits (gloo, world size 2),
and the reference arm's other ranks exit without work."""

import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        times, counts = bench.reduce_over_ranks(dist, [1.0 + rank, 0.5 * rank], [10 * rank + 1, 7], "cpu")
        with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
            json.dump({"times": times, "counts": counts}, f)
    finally:
        dist.destroy_process_group()


def test_reduce_over_ranks_gloo(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    for rank in range(2):
        with open(tmp_path / f"r{rank}.json") as f:
            got = json.load(f)
        assert got["times"] == [2.0, 0.5]      # max over ranks
        assert got["counts"] == [12.0, 14.0]   # sum over ranks


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
