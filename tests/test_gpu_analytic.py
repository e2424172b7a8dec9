"""Restricted diffusion against the Gaussian-phase analytic forms of PGSE:
Neuman's for a cylinder (gradient across the axis) and Murday and Cotts' for
a sphere,

    ln E = -2 gamma^2 G^2 sum_m [2 delta / (a^2 D) - (2 + e^{-a^2 D (Delta - delta)}
           - 2 e^{-a^2 D delta} - 2 e^{-a^2 D Delta} + e^{-a^2 D (Delta + delta)})
           / (a^2 D)^2] / (a^2 (a^2 R^2 - d)),

with a_m R the zeros of J_1' (cylinder, d = 1) or of the spherical j_1'
(sphere, d = 2).  The Gaussian-phase approximation is accurate to about 1e-3
in E at these attenuations (E >= 0.9, checked against the FP64 oracle walk
with 8,000 walkers); free diffusion would give E = exp(-b D) = 0.39 at the
largest G.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GAMMA = 267500.0


def _zeros(kind, n=60):
    sp = pytest.importorskip("scipy.special")
    if kind == "cyl":
        return sp.jnp_zeros(1, n)
    from scipy.optimize import brentq
    f = lambda x: sp.spherical_jn(1, x, derivative=True)  # noqa: E731
    xs = np.linspace(0.5, 4.0 * n, 40000)
    v = f(xs)
    out = []
    for i in range(len(xs) - 1):
        if v[i] * v[i + 1] < 0:
            out.append(brentq(f, xs[i], xs[i + 1]))
            if len(out) == n:
                break
    return np.array(out)


def gaussian_phase_pgse(kind, R, D, G, delta, Delta):
    a2 = (_zeros(kind) / R) ** 2
    d = 1.0 if kind == "cyl" else 2.0
    t = (2.0 + np.exp(-a2 * D * (Delta - delta)) - 2.0 * np.exp(-a2 * D * delta)
         - 2.0 * np.exp(-a2 * D * Delta) + np.exp(-a2 * D * (Delta + delta)))
    s = np.sum((2.0 * delta / (a2 * D) - t / (a2 * D) ** 2) / (a2 * (a2 * R * R - d)))
    return math.exp(-2.0 * GAMMA ** 2 * G ** 2 * s)


@pytest.mark.parametrize("kind", ["cyl", "sph"])
def test_restricted_pore_against_gaussian_phase(dev, kind):
    import axonexa_gb300 as A
    R, D, delta, Delta, dt = 0.005, 2e-6, 5.0, 20.0, 0.002
    steps = int(round((delta + Delta) / dt)) + 1
    Gs = [0.0, 40e-6, 80e-6, 120e-6]
    pore = (A.Cylinder_XY(0.0, 0.0, R, 0.0, 0.0, D, 1, 0.0) if kind == "cyl"
            else A.Sphere(0.0, 0.0, 0.0, R, 0.0, 0.0, D, 1, 0.0))
    seqs = [A.RectGrad(g, delta, Delta - delta) for g in Gs]  # along x: across the axis
    r = A.run_single(pore, seqs, 1 << 20, steps, dt, 11, fix_init_quirk=True, device=dev)
    want = np.array([gaussian_phase_pgse(kind, R, D, g, delta, Delta) for g in Gs])
    assert np.all(np.abs(r.signal - want) <= 3 * r.stderr + 2e-3), (r.signal, want, r.stderr)
    free = np.exp(-np.array([s.getB() for s in seqs]) * D)
    assert r.signal[-1] > free[-1] + 0.4  # restriction, not free diffusion


def test_intra_axonal_compartment_against_gaussian_phase(dev):
    """The restricted-cylinder lattice of the benchmark (radius 5 um in a
    12 um cell, T2 80/60 ms): walkers that start inside the impermeable
    cylinder stay there, so their compartment signal over its G = 0 value is
    the cylinder's Gaussian-phase signal.  The G = 0 value is the T2 weight
    exp(-TE / 80 ms) up to moves that end within an FP32 rounding of the
    wall, which the region lookup (by position, as in the reference) may
    place outside: about one move in 2,000."""
    import axonexa_gb300 as A
    c, R, D, dt = 0.012, 0.005, 2e-6, 0.002
    delta, Delta = 10.0, 40.0
    steps = int(round((delta + Delta) / dt)) + 1
    L = A.Lattice(c, c, c, 60.0, 0.0, D, 1)
    B = [A.Cylinder_XY(c / 2, c / 2, R, 80.0, 0.0, D, 1, 0.0)]
    Gs = [0.0, 20e-6, 40e-6, 60e-6]
    seqs = [A.RectGrad(g, delta, Delta - delta) for g in Gs]
    n = 1 << 20
    r = A.run_lattice(L, B, seqs, n, steps, dt, 5, relaxation=True, compartments=True,
                      device=dev)
    f = math.pi * R * R / (c * c)
    assert abs(r.n_in / n - f) < 4 * math.sqrt(f * (1 - f) / n)
    w = math.exp(-(steps - 1) * dt / 80.0)
    s0 = math.hypot(r.mx_in[0], r.my_in[0]) / r.n_in
    assert abs(s0 / w - 1.0) < 1e-3
    sig = np.hypot(r.mx_in, r.my_in) / (r.n_in * s0)
    want = np.array([gaussian_phase_pgse("cyl", R, D, g, delta, Delta) for g in Gs])
    se = 1.0 / math.sqrt(r.n_in)  # a bound: the terms are at most 1
    assert np.all(np.abs(sig - want) <= 3 * se + 2e-3), (sig, want)
