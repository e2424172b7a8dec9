"""Builds the native library ``libaxx.so`` in-tree (sm_103a only).

Every CUDA translation unit is compiled by nvcc for ``sm_103a`` with
``-fmad=false`` (so that only the explicit fma calls in the kernels fuse and a
host build of the same arithmetic gives identical FP32 results), in parallel,
then linked with the host C++ files into one shared library whose exported
symbols are the C ABI of ``include/axx.h``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libaxx.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = [
    "walk_free.cu",
    "walk_cyl_lat.cu",
    "walk_cyl_single.cu",
    "walk_sph_lat.cu",
    "walk_sph_single.cu",
    "walk_mix.cu",
    "misc_kernels.cu",
    "noalloc.cu",
    "batch.cu",
    "mlp.cu",
    "mlp_tc.cu",
    "mlp_gemm_tc.cu",
    "mag.cu",
    "calcf.cu",
    "wc.cu",
    "mesh.cu",
    "pack.cu",
]
HOST_SOURCES = ["api.cpp", "frame.cpp", "host_plan.cpp", "plan_layout.cpp", "substrate.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libaxx.so")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compiles and links libaxx.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "axx.h"))
    common = ["-std=c++17", "-O3", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-I", CSRC, "-I", os.path.join(ROOT, "include")]
    cmds = []
    objs = []
    for src in CUDA_SOURCES + HOST_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if _newer(o, [s] + headers):
            continue
        if src.endswith(".cu"):
            cmd = [nv] + common + ARCH + ["-lineinfo", "-fmad=false", "-c", s, "-o", o]
        else:
            cmd = [nv] + common + ["-x", "c++", "-c", s, "-o", o]
        cmds.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        for out in ex.map(_run, cmds):
            if verbose and out:
                sys.stdout.write(out)
    if cmds or not os.path.exists(LIB) or not _newer(LIB, objs):
        _run([nv, "-shared"] + ARCH + ["-o", LIB] + objs + ["-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
