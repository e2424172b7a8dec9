"""The CPU oracle of the magnetisation (Bloch) walker against the reference's
own updateWalkersMag (src/kernels/kernelMag.cuh) compiled for the host.

* golden fixtures (tests/golden/ref_mag.npz, from tests/golden/make_golden.py)
  pin the restatement everywhere, bit for bit: per-field sums, the final M of
  the first walkers and their trajectories;
* with the reference tree present the restatement is also compared live over
  more seeds;
* free precession and the trajectory-driven integrator (orc_mag_along) check
  the restatement's pieces on their own.
"""
import math
import os

import numpy as np
import pytest

import cases
from golden.make_golden import NTRACE, TRACE_MOVES, mag_golden_cases

GOLD = os.path.join(os.path.dirname(__file__), "golden", "ref_mag.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


@pytest.mark.parametrize("case", mag_golden_cases(), ids=lambda c: c[0])
def test_mag_oracle_matches_reference_golden(orc, gold, case):
    name, var, pore, fields, p = case
    sums, mw, tr = orc.mag_walk(pore, fields, p, ntrace=NTRACE)
    np.testing.assert_array_equal(sums, gold[name + "/sums"])
    np.testing.assert_array_equal(mw, gold[name + "/m_walk"])
    if name + "/pos" in gold.files:
        np.testing.assert_array_equal(tr["init_pos"], gold[name + "/init_pos"])
        for k in ("pos", "region", "hits", "words"):
            np.testing.assert_array_equal(tr[k][:, :TRACE_MOVES], gold[name + "/" + k], err_msg=k)
        assert tr["hits"].sum() > 0  # reflections happened


@pytest.mark.parametrize("case", mag_golden_cases(), ids=lambda c: c[0])
def test_mag_oracle_matches_reference_live(orc, case):
    name, var, pore, fields, p0 = case
    if orc.reflib() is None:
        pytest.skip("the reference tree is not present here")
    for seed in (101, 202):
        p = orc.mag_params(40, 600, seed, p0.timestep, integrator=p0.integrator,
                           reject=bool(p0.flags & 4), m0=tuple(p0.m0))
        sums, mw, tr = orc.mag_walk(pore, fields, p, ntrace=3)
        ref = orc.ref_mag(var, pore, fields, p, ntrace=3)
        np.testing.assert_array_equal(sums, ref[0])
        np.testing.assert_array_equal(mw, ref[1])


def test_free_precession(orc):
    """No gradient: every walker precesses about B0 z by -gamma B0 t."""
    f = cases.mag_fields()[0]
    f.G = 0.0
    p = orc.mag_params(16, 500, 3, 0.002)
    sums, mw, _ = orc.mag_walk(cases.mag_pore(), [f], p, ntrace=2)
    ang = -p.gamma * f.B0 * p.timestep * p.steps  # steps updates of dt (t = 0 .. steps-1)
    m = sums[0] / p.num_walkers
    assert abs(m[0] - math.cos(ang)) < 1e-9 and abs(m[1] - math.sin(ang)) < 1e-9
    assert abs(m[2]) < 1e-12


def test_mag_along_reproduces_the_walk(orc):
    """The integrator driven by a walker's recorded trajectory gives the
    walk's own final M (the pieces compose as updateWalkersMag does)."""
    fields = cases.mag_fields()
    p = orc.mag_params(2, 300, 9, 0.002)
    sums, mw, tr = orc.mag_walk(cases.mag_pore(), fields, p, ntrace=2)
    for w in range(2):
        pos = np.vstack([tr["init_pos"][w][None], tr["pos"][w]])
        np.testing.assert_array_equal(orc.mag_along(fields, p, pos), mw[w])


# ---- adaptive Dormand-Prince (integrator 3; no reference build exists) ----

def test_dorp_free_precession(orc):
    """A uniform field B0 z: Dormand-Prince follows the exact precession."""
    f = cases.mag_fields()[0]
    f.G = 0.0
    p = orc.mag_params(1, 500, 3, 0.002, integrator=orc.DORP, dorp_tol=1e-9, dorp_levels=6)
    m = orc.mag_along([f], p, np.zeros((500, 3)))[0]
    ang = -p.gamma * f.B0 * p.timestep * p.steps
    assert abs(m[0] - math.cos(ang)) < 1e-7 and abs(m[1] - math.sin(ang)) < 1e-7
    assert abs(m[2]) < 1e-12


def test_dorp_matches_the_rotation_for_fields_constant_over_the_step(orc):
    """While every field is constant in time (inside the first gradient lobe)
    the rotation about B(t_i) is the exact solution of each step: the
    adaptive integrator agrees with it at its tolerance."""
    fields = cases.mag_fields()
    fields = [fields[0], fields[6]]  # QSC_GRE and RECT_GRE: lobes 0.5 ms long
    steps, dt = 200, 0.002          # t < 0.4 ms: inside the first lobe
    rng = np.random.default_rng(5)
    pos = np.cumsum(rng.normal(0, 2e-5, (steps, 3)), axis=0)
    rot = orc.mag_params(1, steps, 3, dt)
    dp = orc.mag_params(1, steps, 3, dt, integrator=orc.DORP, dorp_tol=1e-10, dorp_levels=8)
    np.testing.assert_allclose(orc.mag_along(fields, dp, pos), orc.mag_along(fields, rot, pos),
                               rtol=0, atol=2e-7)


def test_dorp_converges_on_time_varying_fields(orc):
    """Fields that vary within a step (cosine lobes, RF, ramps): the error
    against a run at tolerance 1e-10 (eight halvings) falls with the
    tolerance -- below 5e-4 after 800 steps at the default 1e-6, below 3e-6
    at 1e-8 -- and |M| stays 1."""
    fields = cases.mag_fields()
    steps, dt = 800, 0.002
    rng = np.random.default_rng(7)
    pos = np.cumsum(rng.normal(0, 2e-5, (steps, 3)), axis=0)
    loose = orc.mag_params(1, steps, 3, dt, integrator=orc.DORP)
    tight = orc.mag_params(1, steps, 3, dt, integrator=orc.DORP, dorp_tol=1e-10, dorp_levels=8)
    a, b = orc.mag_along(fields, loose, pos), orc.mag_along(fields, tight, pos)
    assert np.abs(a - b).max() < 5e-4, np.abs(a - b).max()
    mid = orc.mag_params(1, steps, 3, dt, integrator=orc.DORP, dorp_tol=1e-8, dorp_levels=6)
    assert np.abs(orc.mag_along(fields, mid, pos) - b).max() < 3e-6
    assert np.abs(np.linalg.norm(b, axis=1) - 1.0).max() < 1e-6
    # the walk itself runs with the integrator (sums over walkers)
    p = orc.mag_params(32, 300, 11, dt, integrator=orc.DORP)
    sums, mw, _ = orc.mag_walk(cases.mag_pore(), fields, p, ntrace=2)
    assert np.all(np.isfinite(sums)) and np.abs(np.linalg.norm(mw, axis=2) - 1.0).max() < 1e-4
