"""CPU tests of bench.py's reference arm: it times the oracle on the GPU
arm's own graph and config, and the process loads no library of the GPU
package (the graph comes from the oracle's own RMAT generator, which must
equal the package's generator entry for entry)."""

import json
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle as O
import pcc_graphs as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("scale,ef,abc,seed", [
    (10, 16, (0.57, 0.19, 0.19), 1),
    (14, 16, (0.57, 0.19, 0.19), 1),
    (12, 8, (0.45, 0.15, 0.15), 7),
])
def test_oracle_rmat_equals_package_generator(built, scale, ef, abc, seed):
    want = G.rmat(scale, ef, *abc, seed=seed)
    got, _ = O.rmat(scale, ef, *abc, seed=seed).to_csr()
    assert got.n == want.n and got.m == want.m
    np.testing.assert_array_equal(got.offsets, want.offsets)
    np.testing.assert_array_equal(got.neighbors, want.neighbors)


def test_reference_arm_same_config_without_package_libraries(built):
    code = (
        "import runpy, sys, json\n"
        f"sys.argv = ['bench.py', '--impl', 'reference', '--scale', '11', '--steps', '2', '--warmup', '1']\n"
        f"runpy.run_path({os.path.join(ROOT, 'bench.py')!r}, run_name='__main__')\n"
        "maps = [l.split()[-1] for l in open('/proc/self/maps') if l.rstrip().endswith('.so')]\n"
        "print(json.dumps({'maps': sorted(set(maps))}))\n"
    )
    env = dict(os.environ)
    env.pop("RANK", None)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr
    lines = [json.loads(x) for x in r.stdout.strip().splitlines() if x.startswith("{")]
    line, maps = lines[0], lines[1]["maps"]
    assert line["impl"] == "reference"
    assert line["config"]["workload"] == "rmat11_ef16_modularity_refine_nbhr_sync"
    assert line["config"]["n"] == 2048
    assert line["config"]["m_entries"] == G.rmat(11, 16, seed=1).m
    assert line["steps"] == 2 and line["warmup"] == 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0
    assert not [p for p in maps if "libpcc_gb300" in p or "libpcc_host" in p], maps
    assert any("libpcc_oracle" in p for p in maps), maps
