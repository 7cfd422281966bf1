"""Builds libcuacd.so (the engine's C-ABI library) in-tree with nvcc for sm_103a.

The tree and hull kernels compile with --fmad=false so their float32
arithmetic rounds every multiply and add separately (the CPU oracle does the
same); the Hausdorff kernels and the host driver use the default contraction.

    python cuacd-web_gb300/build.py [--force] [--verbose]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcuacd.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + INCLUDE, "--expt-relaxed-constexpr"]
UNITS = {
    "tree_kernels.cu": ["--fmad=false"],
    "hull_kernel.cu": ["--fmad=false"],
    "hausdorff_kernels.cu": [],
    "cuacd_host.cu": [],
    # the GPU capped cut rounds every double operation as the host cut does
    "cut_kernels.cu": ["--fmad=false"],
    "concave_kernels.cu": ["--fmad=false"],
    # host geometry of the decomposition loop: double arithmetic rounded as
    # the reference's JavaScript rounds it, so no contraction into FMA
    "host_mesh.cpp": ["-Xcompiler", "-ffp-contract=off"],
    "plane_cut.cpp": ["-Xcompiler", "-ffp-contract=off"],
    "decompose.cpp": ["-Xcompiler", "-ffp-contract=off"],
    "cpu_hull.cpp": ["-Xcompiler", "-ffp-contract=off"],
}
HEADERS = ["cuacd_dev.cuh", "host_mesh.h", "cut_engine.h", "dev_scan.cuh", "concave_engine.h", "dev_ptr.h", "tree_internal.h"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra=None) -> str:
    os.makedirs(OBJ, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "cuacd.h")]
    jobs = []
    objs = []
    for unit, flags in UNITS.items():
        src = os.path.join(CSRC, unit)
        obj = os.path.join(OBJ, os.path.splitext(unit)[0] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src, __file__] + hdrs):
            cmd = [nvcc()] + ARCH + COMMON + flags + list(extra or []) + ["-c", src, "-o", obj]
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, flush=True)

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs
        run(cmd)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="--verbose" in sys.argv)
    print(LIB)
