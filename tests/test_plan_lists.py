"""The lattice planner's cell lists on the host: tests/cpp/plan_lists.cpp
(built here with g++ against axonexa_gb300/csrc/host_plan.cpp) checks that
every periodic image of a cylinder that a move of the longest step can meet,
or that contains the move's start, is in the candidate list of the cell the
walk kernel files the start under, for random starts and starts within a
few ulps of the grid lines; hexagonal cells and random packs, planned with
the walk's table budgets (grids up to 16 times finer than one basis per
cell) and without one, and random sphere packs (Lattice::boundaryCheck tests every basis,
src/substrate/lattice.cuh:158-247, so a list that misses a reachable image
would change the walk)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cuda_include():
    for d in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        inc = os.path.join(d, "include")
        if d and os.path.exists(os.path.join(inc, "cuda_runtime.h")):
            return inc
    return None


@pytest.fixture(scope="module")
def plans():
    gxx = shutil.which("g++")
    inc = _cuda_include()
    if gxx is None or inc is None:
        pytest.skip("g++ or the CUDA headers are missing")
    out = os.path.join(ROOT, "axonexa_gb300", "_build", "plan_lists")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    subprocess.run([gxx, "-std=c++17", "-O2", "-Wall", "-Werror",
                    "-I", os.path.join(ROOT, "include"), "-I", inc,
                    os.path.join(ROOT, "tests", "cpp", "plan_lists.cpp"),
                    os.path.join(ROOT, "axonexa_gb300", "csrc", "host_plan.cpp"), "-o", out],
                   check=True)
    r = subprocess.run([out, "20000"], capture_output=True, text=True, check=True)
    rows = {}
    for line in r.stdout.splitlines():
        f = line.split()
        if f and f[0] == "plan":
            rows[(f[1], int(f[2]))] = dict(gx=int(f[3]), gy=int(f[4]), cand=float(f[5]),
                                           inst=int(f[6]), checked=int(f[7]), bad=int(f[8]))
    assert r.stdout.rstrip().endswith("done")
    return rows


def test_every_reachable_image_is_listed(plans):
    assert len(plans) == 26
    for key, p in plans.items():
        assert p["checked"] > 1000, key
        assert p["bad"] == 0, (key, p)


def test_finer_grids_leave_fewer_candidates(plans):
    for (name, budget), p in plans.items():
        if budget == 0:
            continue
        coarse = plans[(name, 0)]
        assert p["gx"] * p["gy"] > coarse["gx"] * coarse["gy"], name
        assert p["cand"] < coarse["cand"], name
        if name.startswith("hex"):
            # a hexagonal cell of four cylinders: under 1.3 candidates per
            # move at every fraction (3 to 7 at one basis per cell)
            assert p["cand"] < 1.3, (name, p)
