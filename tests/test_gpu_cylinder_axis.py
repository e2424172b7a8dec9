"""Arbitrary-axis cylinders (the reference's draft Cylinder, cylinder.cuh:1-199)
run through the library's change of frame.

  * a lattice of x- or y-axis cylinders is the z-axis lattice with permuted
    axes: identical bits to that lattice run with permuted cell sides,
    centres and gradient directions;
  * a tilted single pore is a Cylinder_XY in the frame (ahat, bhat, chat):
    the same walk as that pore with rotated gradients, traces stay inside the
    tilted cylinder in simulation coordinates, and motion along the axis is
    free (exp(-b D) for a gradient along it).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

UM = 1e-3
D = 2e-6


def _seqs(A, dirs, G=(0.0, 60e-6, 120e-6)):
    out = []
    for d in dirs:
        for g in G:
            s = A.RectGrad(g, 5.0, 15.0)
            s.ghat = A.Vector3(*d)
            out.append(s)
    return out


@pytest.mark.parametrize("axis", [0, 1])
def test_lattice_of_axis_cylinders_is_the_permuted_z_lattice(dev, axis):
    import axonexa_gb300 as A
    a, b, c = 12 * UM, 10 * UM, 14 * UM
    side = (a, b, c)
    ctr = (0.5 * a, 0.45 * b, 0.55 * c)
    ax = [0.0, 0.0, 0.0]
    ax[axis] = -1.0 if axis else 1.0  # either sense
    perm = [(1, 2, 0), (2, 0, 1)][axis]  # frame axes as simulation axes
    L = A.Lattice(a, b, c, 60.0, 0.0, D, 2)
    B = [A.Cylinder(ctr, ax, 4 * UM, 80.0, 0.0, 1.5e-6, 1, 2e-5),
         A.Sphere(0.1 * a, 0.05 * b, 0.1 * c, 1.5 * UM, 70.0, 0.0, 1e-6, 2, 0.0)]
    dirs = [(1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 1.0), (0.6, 0.0, 0.8)]
    S = _seqs(A, dirs)
    Lz = A.Lattice(*(side[j] for j in perm), 60.0, 0.0, D, 2)
    cz = [ctr[j] for j in perm]
    sp = (0.1 * a, 0.05 * b, 0.1 * c)  # clear of the cylinder and its images
    Bz = [A.Cylinder_XY(cz[0], cz[1], 4 * UM, 80.0, 0.0, 1.5e-6, 1, 2e-5),
          A.Sphere(*(sp[j] for j in perm), 1.5 * UM, 70.0, 0.0, 1e-6, 2, 0.0)]
    Sz = _seqs(A, [tuple(d[j] for j in perm) for d in dirs])
    kw = dict(relaxation=True, permeable=True, device=dev)
    r = A.run_lattice(L, B, S, 4096, 1500, 0.002, 17, **kw)
    rz = A.run_lattice(Lz, Bz, Sz, 4096, 1500, 0.002, 17, **kw)
    np.testing.assert_array_equal(r.mx, rz.mx)
    np.testing.assert_array_equal(r.my, rz.my)
    # traces come back in simulation coordinates
    t = A.trace_lattice(L, B, 16, 400, 0.002, 17, relaxation=True, permeable=True, device=dev)
    tz = A.trace_lattice(Lz, Bz, 16, 400, 0.002, 17, relaxation=True, permeable=True, device=dev)
    inv = np.argsort(perm)
    np.testing.assert_array_equal(t["pos"], tz["pos"][..., inv])
    np.testing.assert_array_equal(t["region"], tz["region"])
    assert tz["hits"].sum() > 0
    # the volume fraction follows
    f, n = A.volume_fraction(L, B, 1 << 18, 5, device=dev)
    fz, nz = A.volume_fraction(Lz, Bz, 1 << 18, 5, device=dev)
    assert n == nz


def test_tilted_single_pore(dev):
    import axonexa_gb300 as A
    R = 4 * UM
    ctr = (1 * UM, -2 * UM, 0.5 * UM)
    axis = (1.0, 2.0, 2.0)
    cyl = A.Cylinder(ctr, axis, R, 0.0, 0.0, D, 1, 0.0)
    F = cyl.frame()
    u = np.array(axis) / 3.0
    perp = np.cross(u, [0.0, 0.0, 1.0])
    perp /= np.linalg.norm(perp)
    G = [0.0, 60e-6, 120e-6, 200e-6]
    S = _seqs(A, [tuple(u), tuple(perp)], G)
    n = 1 << 16
    r = A.run_single(cyl, S, n, 12501, 0.002, 23, device=dev)
    # the same pore as a Cylinder_XY in the frame, gradients rotated
    cf = F @ np.array(ctr)
    xy = A.Cylinder_XY(cf[0], cf[1], R, 0.0, 0.0, D, 1, 0.0)
    Sf = _seqs(A, [tuple(F @ u), tuple(F @ perp)], G)
    rf = A.run_single(xy, Sf, n, 12501, 0.002, 23, device=dev)
    # (the same walk unless a rounding of the frame centre differs: then the
    # same statistics)
    assert np.all(np.abs(r.signal - rf.signal) <= 3 * r.stderr + 1e-5)
    # along the axis: free diffusion
    b = np.array([s.getB() for s in S[:4]])
    assert np.all(np.abs(r.signal[:4] - np.exp(-b * D)) <= 3 * r.stderr[:4] + 2e-4)
    # across it: restricted (well above exp(-b D))
    assert np.all(r.signal[5:8] > np.exp(-b[1:] * D) + 0.05)
    # every traced position lies inside the tilted cylinder
    t = A.trace_single(cyl, 64, 2000, 0.002, 23, device=dev)
    p = t["pos"].reshape(-1, 3).astype(np.float64) - np.array(ctr)
    radial = p - np.outer(p @ u, u)
    assert np.sqrt((radial ** 2).sum(axis=1)).max() < R * (1 + 1e-5)
    assert t["hits"].sum() > 0


def test_axis_cylinder_inputs_are_checked(dev):
    import axonexa_gb300 as A
    from axonexa_gb300 import _native as N
    c = 12 * UM
    L = A.Lattice(c, c, c, 60.0, 0.0, D, 1)
    S = _seqs(A, [(1.0, 0.0, 0.0)])
    tilted = A.Cylinder((c / 2, c / 2, c / 2), (1.0, 1.0, 0.0), 3 * UM, 80.0, 0.0, D, 1, 0.0)
    with pytest.raises(N.AxxError):  # tilted cylinders do not tile the cell
        A.run_lattice(L, [tilted], S, 64, 10, 0.002, 1, device=dev)
    xcyl = A.Cylinder((c / 2, c / 2, c / 2), (1.0, 0.0, 0.0), 3 * UM, 80.0, 0.0, D, 1, 0.0)
    zcyl = A.Cylinder_XY(0.0, 0.0, 2 * UM, 80.0, 0.0, D, 2, 0.0)
    with pytest.raises(N.AxxError):  # two cylinder axes in one lattice
        A.run_lattice(L, [xcyl, zcyl], S, 64, 10, 0.002, 1, device=dev)
    with pytest.raises(N.AxxError):  # no axis
        A.run_single(A.Cylinder((0, 0, 0), (0, 0, 0), 3 * UM, 0, 0, D, 1, 0), S, 64, 10,
                     0.002, 1, device=dev)
    with pytest.raises(N.AxxError):  # the magnetisation walk takes z-cylinders and spheres
        A.run_mag(tilted, [A.QSC_GRE(1e-3, 1e-3, 0.5, 0.6)], 64, 10, 0.002, 1, device=dev)


def test_wc_walker_in_a_tilted_pore(dev):
    import axonexa_gb300 as A
    R = 4 * UM
    axis = (0.0, 0.6, 0.8)
    cyl = A.Cylinder((0.0, 0.0, 0.0), axis, R, 0.0, 0.0, D, 1, 0.0)
    n, steps, dt = 1 << 16, 5000, 0.002
    st, p0 = A.wc_start(cyl, n, 3)
    assert all(cyl.inside(q) for q in p0[:256])
    # a bipolar gradient along the axis (two lobes of T/2): free diffusion,
    # S = exp(-b D) with b = gamma^2 G^2 T^3 / 12 (rejected moves at the
    # wall slow the axial motion by ~1 %)
    G = 100e-6
    grad = np.outer(np.where(np.arange(steps) < steps // 2, 1.0, -1.0), np.array(axis) * G)
    _, sc, _ = A.run_wc(cyl, st, p0, grad, dt, device=dev)
    T = steps * dt
    want = math.exp(-(A.GAMMA * G) ** 2 * D * T ** 3 / 12.0)
    assert abs(sc / n - want) < 0.02, (sc / n, want)
