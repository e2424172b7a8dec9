"""The magnetisation (Bloch) walk on the GPU against the CPU oracle.

  1. trajectories, bit for bit: the walk of updateWalkersMag is the
     single-pore walk, so the GPU trace equals the oracle's FP32 kernel
     formulation (positions, hits, stream words);
  2. magnetisation per walker: the GPU's FP32 M of every field functor and
     integrator against the FP64 restatement of the reference's updates
     integrated along the GPU's own trajectory;
  3. sums: within 3 standard errors of the oracle's FP64 reference-order walk
     (pinned bit-exact to the reference by tests/test_oracle_mag.py);
  4. free precession exactly, and a 1.5 T field where B0 swamps the gradient
     term in FP32 unless the rotation angle is split as the kernel does.
"""
import math

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


def to_product(pore, fields):
    import axonexa_gb300 as A
    if pore.type == 1:
        P = A.Sphere(pore.cx, pore.cy, pore.cz, pore.radius, pore.T2, pore.T1, pore.D, pore.region,
                     pore.permeability, pore.eps)
    else:
        P = A.Cylinder_XY(pore.cx, pore.cy, pore.radius, pore.T2, pore.T1, pore.D, pore.region,
                          pore.permeability, pore.eps)
    F = []
    for f in fields:
        g = (f.gx, f.gy, f.gz)
        F.append({0: lambda: A.QSC_GRE(f.B0, f.G, f.duration, f.spacing),
                  1: lambda: A.QSC_PGSE(f.B0, f.G, f.duration, f.spacing, f.rf_duration, f.dtmin,
                                        f.dtmax, f.TE),
                  2: lambda: A.QSC_COS_GRE(f.B0, f.G, f.duration, f.spacing, f.num_periods),
                  3: lambda: A.QSC_GRE_TRAP(f.B0, f.G, f.duration, f.spacing, f.ramp),
                  4: lambda: A.SIN_GRE(f.B0, g, f.duration, f.spacing, f.period),
                  5: lambda: A.COS_GRE(f.B0, g, f.duration, f.spacing, f.num_periods),
                  6: lambda: A.RECT_GRE(f.B0, g, f.duration, f.spacing),
                  7: lambda: A.UCN_lowfield(f.B0, f.G, f.rf_duration, f.dtmin, f.dtmax)}[f.kind]())
    return P, F


CASES = [  # name, sph, integrator, reject, multistep fields only, m0
    ("rot_cyl", False, 0, False, False, (1.0, 0.0, 0.0)),
    ("rot_sph", True, 0, False, False, (0.6, 0.0, 0.8)),
    ("rej_cyl", False, 0, True, False, (1.0, 0.0, 0.0)),
    ("rk4_cyl", False, 1, False, False, (1.0, 0.0, 0.0)),
    ("ms_cyl", False, 2, False, True, (0.0, 0.0, 1.0)),
    ("ms_sph", True, 2, False, True, (1.0, 0.0, 0.0)),
]


def _setup(orc, sph, integ, multi):
    pore = cases.mag_pore(sph)
    fields = cases.mag_multistep_fields() if multi else cases.mag_fields()
    return pore, fields


@pytest.mark.parametrize("case", CASES, ids=lambda c: c[0])
def test_mag_trajectory_bit_exact_and_m_per_walker(dev, orc, case):
    import axonexa_gb300 as A
    name, sph, integ, reject, multi, m0 = case
    pore, fields = _setup(orc, sph, integ, multi)
    P, F = to_product(pore, fields)
    n, steps, seed, dt = 64, 800, 31, 0.002
    g = A.trace_mag(P, F, n, steps, dt, seed, m0=m0, integrator=integ, specular=not reject,
                    device=dev)
    # 1. the walk: the oracle's FP32 single-pore formulation, bit for bit
    p = cases.params(n, steps, seed, dt=dt, flags=4 if reject else 0)
    _, o, _ = orc.walk(None, [pore], [], p, orc.KERN32, ntrace=n)
    np.testing.assert_array_equal(g["init_pos"].astype(np.float64), o["init_pos"])
    np.testing.assert_array_equal(g["pos"].astype(np.float64), o["pos"])
    np.testing.assert_array_equal(g["hits"], o["hits"])
    np.testing.assert_array_equal(g["words"], o["words"])
    if not reject:
        assert o["hits"].sum() > 0
    # 2. M of every field: FP32 kernel vs FP64 updates along the same path
    mp = orc.mag_params(n, steps, seed, dt, integrator=integ, reject=reject, m0=m0)
    worst = 0.0
    for w in range(n):
        pos = np.vstack([g["init_pos"][w][None], g["pos"][w]]).astype(np.float64)
        ref = orc.mag_along(fields, mp, pos)
        worst = max(worst, float(np.abs(g["m"][w] - ref).max()))
    assert worst < 2e-4, worst
    # rotations keep |M| = 1 (the RK4 start step does not, in the reference too)
    if integ != 1:
        assert np.abs(np.linalg.norm(g["m"], axis=2) - 1.0).max() < 1e-4


@pytest.mark.parametrize("case", CASES, ids=lambda c: c[0])
def test_mag_sums_against_reference_order_fp64(dev, orc, case):
    import axonexa_gb300 as A
    name, sph, integ, reject, multi, m0 = case
    pore, fields = _setup(orc, sph, integ, multi)
    P, F = to_product(pore, fields)
    n, steps, seed, dt = 4096, 600, 47, 0.002
    r = A.run_mag(P, F, n, steps, dt, seed, m0=m0, integrator=integ, specular=not reject,
                  device=dev)
    mp = orc.mag_params(n, steps, seed, dt, integrator=integ, reject=reject, m0=m0)
    ref, mw, _ = orc.mag_walk(pore, fields, mp, nthreads=8, ntrace=512)
    got = np.stack([r.mx, r.my, r.mz], axis=1)
    se = mw.std(axis=0) / math.sqrt(n)  # [nf, 3] from 512 walkers
    # 3 standard errors, plus the FP32 arithmetic floor of the per-walker
    # check above (components that hardly vary over walkers, such as Mz
    # starting along z, have standard errors far below it)
    d = np.abs(got - ref) / n
    assert np.all(d <= 3.0 * se + 2e-4), (d - 3.0 * se).max()


def test_mag_free_precession(dev):
    import axonexa_gb300 as A
    pore = A.Cylinder_XY(0.0, 0.0, 5e-3, 0.0, 0.0, 2e-6, 1, 0.0)
    f = A.QSC_GRE(1e-3, 0.0, 0.5, 0.6)  # no gradient: B = B0 z everywhere
    n, steps, dt = 2048, 700, 0.002
    r = A.run_mag(pore, [f], n, steps, dt, 5, device=dev)
    ang = -A.GAMMA * 1e-3 * dt * steps
    assert abs(r.mx[0] / n - math.cos(ang)) < 2e-5
    assert abs(r.my[0] / n - math.sin(ang)) < 2e-5
    assert abs(r.mz[0] / n) < 1e-6


def test_mag_high_field_keeps_the_gradient_phase(dev, orc):
    """B0 = 1.5 T rotates 800 rad per step; the gradient adds ~1e-3 rad.
    The split angle keeps the per-walker M within 1e-3 of FP64."""
    import axonexa_gb300 as A
    f = orc.Field(0, 0, 1.5, 1e-2, 0, 0, 0, 0.5, 0.6, 0, 0, 0, 0, 0, 0)
    pore = cases.mag_pore()
    P, F = to_product(pore, [f])
    n, steps, dt = 32, 800, 0.002
    g = A.trace_mag(P, F, n, steps, dt, 13, device=dev)
    mp = orc.mag_params(n, steps, 13, dt)
    worst = 0.0
    spread = []
    for w in range(n):
        pos = np.vstack([g["init_pos"][w][None], g["pos"][w]]).astype(np.float64)
        ref = orc.mag_along([f], mp, pos)
        worst = max(worst, float(np.abs(g["m"][w] - ref).max()))
        spread.append(ref[0, :2])
    assert worst < 1e-3, worst
    # the walkers dephased (the gradient term mattered)
    assert np.std(np.array(spread), axis=0).max() > 1e-2


def test_mag_acquisition_stream_api(dev):
    """magAcquisitionStream.runAcquisition fills the acquisition's Mx/My/Mz
    with run_mag's sums."""
    import axonexa_gb300 as A
    pore = A.Cylinder_XY(0.0, 0.0, 5e-3, 0.0, 0.0, 2e-6, 1, 0.0)
    pas = A.magAcquisitionStream(1024)
    for i in range(3):
        acq = A.magAcquisition(1, 600, 100 + i)
        acq.addMeasurement(A.QSC_GRE(1e-3, i * 5e-4, 0.5, 0.2))
        pas.addAcquisition(acq)
    pas.runAcquisitionStream(pore, (1.0, 0.0, 0.0), 0.002)
    for i in range(3):
        acq = pas.getAcquisition(i)
        r = A.run_mag(pore, acq.getFieldFunctors(), 1024, 600, 0.002, 100 + i, device=dev)
        assert acq.getMx()[0] == r.mx[0] and acq.getMy()[0] == r.my[0]
    # stronger gradients dephase more
    s = [math.hypot(pas.getAcquisition(i).getMx()[0], pas.getAcquisition(i).getMy()[0])
         for i in range(3)]
    assert s[0] > s[1] > s[2]


def test_mag_negative_gamma_helium3(dev, orc):
    """GAMMA = -203789 (helium-3, the reference's magLF examples) reverses the
    precession; per-walker M against FP64 along the same paths."""
    import axonexa_gb300 as A
    f = orc.Field(0, 0, 1e-3, 1e-3, 0, 0, 0, 0.5, 0.6, 0, 0, 0, 0, 0, 0)
    pore = cases.mag_pore()
    P, F = to_product(pore, [f])
    n, steps, dt, gam = 32, 800, 0.002, -203789.0
    g = A.trace_mag(P, F, n, steps, dt, 17, gamma=gam, device=dev)
    mp = orc.mag_params(n, steps, 17, dt, gamma=gam)
    worst = 0.0
    for w in range(n):
        pos = np.vstack([g["init_pos"][w][None], g["pos"][w]]).astype(np.float64)
        worst = max(worst, float(np.abs(g["m"][w] - orc.mag_along([f], mp, pos)).max()))
    assert worst < 2e-4, worst
    # free precession sense: after one step My = -sin(-|gamma| B0 dt) > 0 for gamma < 0
    one = A.trace_mag(P, [A.QSC_GRE(1e-3, 0.0, 0.5, 0.6)], 1, 1, dt, 1, gamma=gam, device=dev)
    assert one["m"][0, 0, 1] > 0


# ---- adaptive Dormand-Prince (AXX_MAG_DORP) -------------------------------

def test_mag_dorp_per_walker_against_fp64(dev, orc):
    """Every field functor kind, Dormand-Prince in FP32 on the GPU against
    the oracle's FP64 Dormand-Prince along the same trajectories (the error
    control may choose other sub-steps in FP32 near its threshold; both stay
    within the tolerance's reach of the solution)."""
    import axonexa_gb300 as A
    pore, fields = _setup(orc, False, 3, False)
    P, F = to_product(pore, fields)
    n, steps, seed, dt = 32, 400, 61, 0.002
    g = A.trace_mag(P, F, n, steps, dt, seed, integrator=3, device=dev)
    p = cases.params(n, steps, seed, dt=dt, flags=0)
    _, o, _ = orc.walk(None, [pore], [], p, orc.KERN32, ntrace=n)
    np.testing.assert_array_equal(g["pos"].astype(np.float64), o["pos"])
    mp = orc.mag_params(n, steps, seed, dt, integrator=orc.DORP)
    worst = 0.0
    for w in range(n):
        pos = np.vstack([g["init_pos"][w][None], g["pos"][w]]).astype(np.float64)
        worst = max(worst, float(np.abs(g["m"][w] - orc.mag_along(fields, mp, pos)).max()))
    assert worst < 1e-3, worst
    assert np.abs(np.linalg.norm(g["m"], axis=2) - 1.0).max() < 1e-3


def test_mag_dorp_free_precession_and_sums(dev, orc):
    import axonexa_gb300 as A
    pore = A.Cylinder_XY(0.0, 0.0, 5e-3, 0.0, 0.0, 2e-6, 1, 0.0)
    f = A.QSC_GRE(1e-3, 0.0, 0.5, 0.6)  # no gradient: B = B0 z everywhere
    n, steps, dt = 2048, 700, 0.002
    r = A.run_mag(pore, [f], n, steps, dt, 5, integrator=3, device=dev)
    ang = -A.GAMMA * 1e-3 * dt * steps
    # 374.5 rad over 700 steps: the phase error may grow by up to the
    # tolerance (1e-6) per step
    assert abs(r.mx[0] / n - math.cos(ang)) < 7e-4
    assert abs(r.my[0] / n - math.sin(ang)) < 7e-4
    # sums of every functor kind against the FP64 walk with the same integrator
    cpore, fields = _setup(orc, False, 3, False)
    P, F = to_product(cpore, fields)
    n, steps, seed = 1024, 300, 47
    r = A.run_mag(P, F, n, steps, dt, seed, integrator=3, device=dev)
    mp = orc.mag_params(n, steps, seed, dt, integrator=orc.DORP)
    ref, mw, _ = orc.mag_walk(cpore, fields, mp, nthreads=8, ntrace=256)
    got = np.stack([r.mx, r.my, r.mz], axis=1)
    se = mw.std(axis=0) / math.sqrt(n)
    d = np.abs(got - ref) / n
    assert np.all(d <= 3.0 * se + 1e-3), (d - 3.0 * se).max()


def test_mag_dorp_rejects_bad_parameters(dev):
    import axonexa_gb300 as A
    from axonexa_gb300 import _native as N
    pore = A.Cylinder_XY(0.0, 0.0, 5e-3, 0.0, 0.0, 2e-6, 1, 0.0)
    f = A.QSC_GRE(1e-3, 1e-3, 0.5, 0.6)
    with pytest.raises(N.AxxError):
        A.run_mag(pore, [f], 64, 10, 0.002, 5, integrator=3, dorp_levels=9, device=dev)
    with pytest.raises(N.AxxError):
        A.run_mag(pore, [f], 64, 10, 0.002, 5, integrator=3, dorp_tol=-1.0, device=dev)
