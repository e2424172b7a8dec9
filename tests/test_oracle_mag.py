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
