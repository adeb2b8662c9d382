"""Build recipe of the native parts of the package (no cmake).

* libpcc_gb300.so -- the CUDA library (csrc/*.cu) for sm_103a, exporting the
  C ABI of include/pcc_gb300.h.
* libpcc_host.so  -- the C++ host side: InMemoryClusterer mirror, text-format
  config parser, GBBS adjacency I/O and synthetic graph generators.
* cluster-in-memory_main -- the CLI with the reference's flags.

Translation units compile in parallel; outputs go to _build/ next to this
file.  Rebuilds only what is older than its sources.
"""

from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")

CUDA_LIB = os.path.join(BUILD, "libpcc_gb300.so")
HOST_LIB = os.path.join(BUILD, "libpcc_host.so")
CLI = os.path.join(BUILD, "cluster-in-memory_main")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build_cuda(force: bool = False, jobs: int = 0, extra_flags=None) -> str:
    os.makedirs(os.path.join(BUILD, "obj"), exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = sorted(glob.glob(os.path.join(CSRC, "*.cuh"))) + [os.path.join(INCLUDE, "pcc_gb300.h")]
    nvcc = _nvcc()
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC",
                    "-Xcompiler", "-ffp-contract=off", "-I" + INCLUDE, "-I" + CSRC]
    flags += list(extra_flags or [])
    objs = []
    todo = []
    for src in sources:
        obj = os.path.join(BUILD, "obj", os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            todo.append([nvcc] + flags + ["-c", src, "-o", obj])
    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(8, len(todo))) as ex:
            list(ex.map(_run, todo))
    if force or todo or _stale(CUDA_LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", CUDA_LIB] + objs + ["-lcudart"])
    return CUDA_LIB


def build_host(force: bool = False) -> str:
    """C++ host library + CLI (g++, portable flags, OpenMP for generators)."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(HOST, "*.cc")))
    lib_srcs = [s for s in srcs if not s.endswith("_main.cc")]
    main_srcs = [s for s in srcs if s.endswith("_main.cc")]
    hdrs = sorted(glob.glob(os.path.join(HOST, "*.h"))) + sorted(glob.glob(os.path.join(INCLUDE, "*.h")))
    if not lib_srcs:
        return ""
    cflags = ["-O3", "-std=c++17", "-fopenmp", "-fPIC", "-Wall", "-ffp-contract=off", "-I" + INCLUDE,
              "-I" + HOST]
    if force or _stale(HOST_LIB, lib_srcs + hdrs):
        _run(["g++"] + cflags + ["-shared", "-o", HOST_LIB] + lib_srcs +
             ["-L" + BUILD, "-lpcc_gb300", "-Wl,-rpath,$ORIGIN"])
    if main_srcs and (force or _stale(CLI, main_srcs + hdrs + [HOST_LIB])):
        _run(["g++"] + cflags + ["-o", CLI] + main_srcs +
             ["-L" + BUILD, "-lpcc_host", "-lpcc_gb300", "-Wl,-rpath,$ORIGIN"])
    return HOST_LIB


def build_all(force: bool = False) -> None:
    build_cuda(force)
    build_host(force)


if __name__ == "__main__":
    import sys
    build_all(force="--force" in sys.argv)
    print("built", CUDA_LIB)
