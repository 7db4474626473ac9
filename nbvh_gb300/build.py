"""Builds libnbvh.so in-tree: every CUDA/C++ translation unit of nbvh_gb300/csrc compiled for
sm_103a in parallel, then linked (CUDA runtime linked statically, so the library loads on a
machine without a GPU and reports NBVH_EDEVICE there)."""

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libnbvh.so")

SOURCES = [
    "k_classic.cu",
    "k_neural.cu",
    "k_train.cu",
    "k_misc.cu",
    "k_mlp_tc.cu",
    "k_path.cu",
    "k_query.cu",
    "nbvh_api.cpp",
    "nbvh_server.cpp",
    "nbvh_format.cpp",
    "nbvh_tree_cut.cpp",
    "nbvh_scene.cpp",
    "k_tree_cut.cu",
    "bvh_builder.cpp",
]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no FMA contraction (aarch64 GCC contracts a*b+c by default), so that host-side
# precomputation (dilated boxes, camera frames) rounds exactly like the device intrinsics
COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-O3,-ffp-contract=off",
          "-I", os.path.join(HERE, "..", "include")]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _stale(obj, src, headers):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + headers)


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "nbvh.h"))
    jobs = []
    objs = []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if force or _stale(obj, path, headers):
            jobs.append([nvcc] + COMMON + ARCH + ["-c", path, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        if verbose:
            sys.stderr.write(r.stdout + r.stderr)
        return r

    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    if jobs or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        run([nvcc] + ARCH + ["-shared", "-Xcompiler", "-fPIC", "-o", LIB] + objs)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
