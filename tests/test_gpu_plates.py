"""Parallel plates (Plane bases, plane.cuh:1-40) on the GPU: physics checks
beyond the bit-exact traces and reference-order signals of
tests/test_gpu_parity.py.

Walls at x = 0 and x = l of an l-wide periodic cell (the reference's
planePhase example):
  * motion along the walls is free: gradients along y and z give exp(-b D);
  * across them, the narrow-pulse long-time limit 2 (1 - cos(q l)) / (q l)^2
    (q = gamma G delta) holds up to the finite-pulse correction, which a 1-D
    reflecting-walk estimate puts below 0.01 for delta = 0.2 ms, l = 8 um,
    D = 2 um^2/ms, q l <= pi.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

L_MM = 0.008
D = 2e-6


def _plates():
    import axonexa_gb300 as A
    lat = A.Lattice(L_MM, L_MM, L_MM, 60.0, 0.0, D, 2)
    walls = [A.Plane((0.0, 0.0, 0.0), (1.0, 0.0, 0.0)),
             A.Plane((L_MM, 0.0, 0.0), (-1.0, 0.0, 0.0))]
    return lat, walls


def test_plates_free_along_the_walls(dev):
    import axonexa_gb300 as A
    lat, walls = _plates()
    G = np.array([0.0, 40.0, 80.0, 120.0]) * 1e-6
    S = [A.RectGrad(g, 5.0, 15.0) for g in G]
    for s in S:
        s.ghat = A.Vector3(0.0, 0.6, 0.8)
    n = 1 << 16
    res = A.run_lattice(lat, walls, S, n, 12501, 0.002, 99, device=dev)
    assert res.cap_hits == 0
    want = np.exp(-np.array([s.getB() for s in S]) * D)
    assert np.all(np.abs(res.signal - want) <= 3 * res.stderr + 2e-4), (res.signal, want)


def test_plates_narrow_pulse_limit_across(dev):
    import axonexa_gb300 as A
    lat, walls = _plates()
    delta, Delta, dt = 0.2, 100.0, 0.002
    qls = [0.0, math.pi / 2, math.pi]
    S = [A.RectGrad(ql / (A.GAMMA * delta * L_MM), delta, Delta - delta) for ql in qls]
    steps = int(round((delta + Delta) / dt)) + 1
    n = 1 << 18
    res = A.run_lattice(lat, walls, S, n, steps, dt, 7, device=dev)
    assert res.cap_hits == 0
    want = np.array([1.0] + [2.0 * (1.0 - math.cos(q)) / q ** 2 for q in qls[1:]])
    assert abs(res.signal[0] - 1.0) < 1e-6
    assert np.all(np.abs(res.signal - want) <= 0.012 + 3 * res.stderr), (res.signal, want)
    # restriction: well above the free-diffusion signal exp(-b D)
    free = np.exp(-np.array([s.getB() for s in S]) * D)
    assert np.all(res.signal[1:] > free[1:] + 0.1)


def test_plane_inputs_are_checked(dev):
    import axonexa_gb300 as A
    from axonexa_gb300 import _native as N
    lat, walls = _plates()
    S = [A.RectGrad(1e-4, 5.0, 15.0)]
    with pytest.raises(N.AxxError):  # no normal
        A.run_lattice(lat, [A.Plane((0.0, 0.0, 0.0), (0.0, 0.0, 0.0))], S, 64, 10, 0.002, 1,
                      device=dev)
    with pytest.raises(N.AxxError):  # a plane is not a pore
        A.run_single(walls[0], S, 64, 10, 0.002, 1, device=dev)
    with pytest.raises(N.AxxError):  # nothing to start inside
        A.run_lattice(lat, walls, S, 64, 10, 0.002, 1, init_mode=2, init_arg=0, device=dev)
    # a region start ignores the walls (they hold no region)
    r = A.run_lattice(lat, walls, S, 64, 10, 0.002, 1, init_mode=1, init_arg=0, device=dev)
    assert r.walker_steps == 64 * 9
