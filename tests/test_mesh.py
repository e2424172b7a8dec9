"""Closed triangle meshes as single pores (the reference's draft Mesh and
Triangle, src/primitives/mesh.cuh:1-75, triangle.cuh:1-59, which do not
compile: parity is unpinned against the reference).

The oracle restates the GPU walker in FP64 and FP32 (oracle.cpp, mesh
section).  Checks: no walker leaves a closed mesh; the outward orientation
makes the input winding irrelevant; a cube's walk across x equals the
parallel-plate walk of the same width (the same streams move x alike); the
GPU trace equals the FP32 mirror bit for bit.
"""

import numpy as np
import pytest

import cases
import axonexa_gb300.mesh as Mh

UM = 1e-3
D = 2e-6
L_SHAPE = [(0, 0), (8, 0), (8, 4), (4, 4), (4, 8), (0, 8)]


def _meshes():
    return [("cube", Mh.cube(8 * UM, D, center=(4 * UM, 4 * UM, 4 * UM))),
            ("icosphere2", Mh.icosphere(5 * UM, 2, D)),
            ("l_prism", Mh.prism(np.array(L_SHAPE) * UM, 0.0, 6 * UM, D))]


SEQS = [cases.pgse(0), cases.pgse(100, delta=2.0, Delta=10.0),
        cases.pgse(200, delta=2.0, Delta=10.0), cases.pgse(200, delta=2.0, Delta=10.0,
                                                           g=(0.0, 0.6, 0.8))]


@pytest.mark.parametrize("name,mesh", _meshes(), ids=[m[0] for m in _meshes()])
def test_oracle_mesh_walk_stays_inside(orc, name, mesh):
    p = cases.params(2000, 3001, 7)
    for mode in (orc.KERN32, orc.KERN64):
        s, tr, esc = orc.mesh_walk(mesh.vertices, mesh.triangles, D, SEQS, p, mode, nthreads=8,
                                   ntrace=8)
        assert esc == 0
        assert tr["hits"].sum() > 0
        assert abs(s[0, 0] - 2000) < 1e-9  # G = 0
    # the winding of the input does not matter: triangles are oriented outward
    # (by swapping their last two vertices where needed)
    flipped = mesh.triangles.copy()
    flipped[::2] = flipped[::2][:, [0, 2, 1]]
    a, _, _ = orc.mesh_walk(mesh.vertices, mesh.triangles, D, SEQS, p, orc.KERN32, nthreads=8)
    b, _, _ = orc.mesh_walk(mesh.vertices, flipped, D, SEQS, p, orc.KERN32, nthreads=8)
    np.testing.assert_array_equal(a, b)


def test_oracle_cube_equals_parallel_plates(orc):
    """Across x, a cube walk is the plate walk: the same streams give the same
    start x (the cube fills its bounding box) and the same x moves."""
    cube = Mh.cube(8 * UM, D, center=(4 * UM, 4 * UM, 4 * UM))
    seqs = SEQS[:3]
    p = cases.params(4000, 6001, 5)
    sc, _, esc = orc.mesh_walk(cube.vertices, cube.triangles, D, seqs, p, orc.KERN64, nthreads=8)
    lat, plates = cases.parallel_plates(l_um=8.0)
    sp, _, _ = orc.walk(lat, plates, seqs, p, orc.KERN64, nthreads=8)
    assert esc == 0
    sig = lambda s: np.hypot(s[:, 0], s[:, 1]) / 4000
    assert np.abs(sig(sc) - sig(sp)).max() < 1e-6, (sig(sc), sig(sp))


def test_oracle_rejects_open_meshes(orc):
    cube = Mh.cube(8 * UM, D)
    with pytest.raises(ValueError):
        orc.mesh_walk(cube.vertices, cube.triangles[:-1], D, SEQS, cases.params(8, 10, 1))


@pytest.mark.gpu
@pytest.mark.parametrize("name,mesh", _meshes(), ids=[m[0] for m in _meshes()])
def test_gpu_mesh_trace_bit_exact(dev, orc, name, mesh):
    import axonexa_gb300 as A
    n, steps, seed = 64, 2000, 11
    g = A.trace_mesh(mesh, n, steps, 0.002, seed, device=dev)
    _, o, esc = orc.mesh_walk(mesh.vertices, mesh.triangles, D, [], cases.params(n, steps, seed),
                              orc.KERN32, ntrace=n)
    np.testing.assert_array_equal(g["init_pos"].astype(np.float64), o["init_pos"])
    np.testing.assert_array_equal(g["pos"].astype(np.float64), o["pos"])
    np.testing.assert_array_equal(g["hits"], o["hits"])
    np.testing.assert_array_equal(g["words"], o["words"])
    assert g["escaped"] == esc == 0
    assert o["hits"].sum() > 0


@pytest.mark.gpu
def test_gpu_mesh_signals_and_physics(dev, orc):
    import axonexa_gb300 as A
    from test_gpu_parity import to_product
    n, steps = 1 << 16, 6001
    # the FP32 mirror: tight agreement of the sums; no leak at scale
    for name, mesh in _meshes():
        _, _, S = to_product(None, [], SEQS)
        r = A.run_mesh(mesh, S, n, steps, 0.002, 3, device=dev)
        assert r.escaped == 0 and r.cap_hits == 0
        k32, _, _ = orc.mesh_walk(mesh.vertices, mesh.triangles, D, SEQS,
                                  cases.params(n, steps, 3), orc.KERN32, nthreads=16)
        assert np.all(np.abs(r.mx - k32[:, 0]) <= 2e-5 * n), name
    # a cube across x is the parallel-plate walk of the same width: the same
    # walks up to FP32 rounding (the two kernels round the path after a y or z
    # reflection and sum the phase differently), far inside one standard
    # error (about 6e-4 here)
    cube = Mh.cube(8 * UM, D, center=(4 * UM, 4 * UM, 4 * UM))
    lat, plates = cases.parallel_plates(l_um=8.0)
    L, B, S = to_product(lat, plates, SEQS[:3])
    rc = A.run_mesh(cube, S, n, steps, 0.002, 5, device=dev)
    rp = A.run_lattice(L, B, S, n, steps, 0.002, 5, device=dev)
    assert np.abs(rc.signal - rp.signal).max() < 1e-4, (rc.signal, rp.signal)
    # a fine icosphere approaches the sphere pore (its volume is 0.3 % smaller)
    ico = Mh.icosphere(5 * UM, 4, D)
    sph = A.Sphere(0.0, 0.0, 0.0, 5 * UM, 0.0, 0.0, D, 1, 0.0)
    _, _, S = to_product(None, [], SEQS)
    ri = A.run_mesh(ico, S, n, steps, 0.002, 9, device=dev)
    rs = A.run_single(sph, S, n, steps, 0.002, 9, fix_init_quirk=True, device=dev)
    assert ri.escaped == 0
    assert np.all(np.abs(ri.signal - rs.signal) < 0.01 + 3 * rs.stderr), (ri.signal, rs.signal)


@pytest.mark.gpu
def test_gpu_mesh_inputs_are_checked(dev):
    import axonexa_gb300 as A
    from axonexa_gb300 import _native as N
    cube = Mh.cube(8 * UM, D)
    S = [A.RectGrad(1e-4, 2.0, 8.0)]
    with pytest.raises(N.AxxError):  # a hole
        A.run_mesh(Mh.Mesh(cube.vertices, cube.triangles[:-1], D), S, 64, 10, 0.002, 1,
                   device=dev)
    with pytest.raises(N.AxxError):  # a vertex index out of range
        bad = cube.triangles.copy()
        bad[0, 0] = 99
        A.run_mesh(Mh.Mesh(cube.vertices, bad, D), S, 64, 10, 0.002, 1, device=dev)
    with pytest.raises(N.AxxError):  # steps longer than half the mesh
        A.run_mesh(Mh.cube(0.1 * UM, D), S, 64, 10, 0.002, 1, device=dev)
