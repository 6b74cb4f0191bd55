"""Builds libendobeams_gb300.so in-tree with nvcc (sm_103a only).

Each .cu translation unit is compiled in parallel, then linked into one
shared library under ``endobeams.jl_gb300/_build/``.  No cmake, no torch.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libendobeams_gb300.so")
SOURCES = ["eb_kernels.cu", "eb_gmres.cu", "eb_band.cu", "eb_band_tc.cu", "eb_abi.cu", "eb_testing.cu", "eb_mlp.cu",
           "eb_warm.cu", "eb_output.cu", "eb_mesh_sdf.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(verbose: bool = False, force: bool = False, extra_flags=None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(HERE, "..", "include", "endobeams_gb300.h"))
    cc = nvcc()
    flags = FLAGS + (extra_flags or [])

    def compile_one(src):
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        path = os.path.join(CSRC, src)
        if not force and _newer(obj, [path] + headers):
            return obj, ""
        cmd = [cc] + ARCH + flags + ["-c", path, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(compile_one, SOURCES))
    for _, log in results:
        if verbose and log:
            print(log, file=sys.stderr)
    objs = [o for o, _ in results]
    if force or not _newer(LIB, objs):
        # static CUDA runtime: the library loads on hosts without a GPU driver
        cmd = [cc] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
