"""In-tree build of the CUDA library lbm_gb300/_build/liblbm_gpu.so.

Every translation unit is compiled by nvcc for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, and linked into one
shared library with the CUDA runtime linked statically.  The reference-table
engine is compiled with ``-fmad=false`` so that its FP64 arithmetic keeps the
reference's separately rounded multiplies and adds; the throughput kernels use
fused multiply-adds.  The host-only grid builder (grid.cpp) is compiled without
floating-point contraction for the same reason.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liblbm_gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include")]
UNITS = {
    "table_engine.cu": ["-fmad=false"],
    "reduce.cu": [],
    "box.cu": [],
    "box_tma.cu": [],
    "box_rows.cu": [],
    "capi.cu": [],
    "noalloc.cu": [],
    "batch.cu": [],
    "unet.cu": [],
    "conv_tc.cu": [],
    # host-only grid and table build: no floating-point contraction, so that
    # the cut tests round as the reference's do on either host architecture
    "grid.cpp": ["-Xcompiler", "-ffp-contract=off"],
    # the multi-level generator (same geometry code, same rule)
    "grid_tree.cpp": ["-Xcompiler", "-ffp-contract=off"],
    # its device counterpart: the same geometry code, no contraction either
    "grid_device.cu": ["-fmad=false", "-Xcompiler", "-ffp-contract=off"],
    # particle step: the reference's separately rounded FP64 operations
    "lpt.cu": ["-fmad=false"],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))] + [
        os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))
    ]


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    newest_header = max(os.path.getmtime(h) for h in _headers())
    cc = nvcc()
    jobs = []
    for unit, extra in UNITS.items():
        src = os.path.join(CSRC, unit)
        obj = os.path.join(BUILD, unit + ".o")
        stale = force or not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), newest_header)
        if stale:
            jobs.append([cc] + ARCH + COMMON + extra + ["-c", src, "-o", obj])
    if verbose:
        for j in jobs:
            print(" ".join(j))

    def run(cmd):
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
        return p.stderr

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for warn in ex.map(run, jobs):
            if verbose and warn:
                print(warn, file=sys.stderr)
    objs = [os.path.join(BUILD, u + ".o") for u in UNITS]
    if force or jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        subprocess.run([cc] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs, check=True)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
