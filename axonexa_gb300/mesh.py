"""Closed triangle meshes as single pores (axx_run_mesh, axx_trace_mesh).

Mirrors the reference's draft Mesh and Triangle (src/primitives/mesh.cuh:1-75,
triangle.cuh:1-59): a mesh is a list of triangles enclosing a volume ("We
assume no holes -> a closed surface mesh") with a diffusion coefficient
inside.  `cube` and `icosphere` build common test shapes.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .acquisition import GAMMA, Device, RunResult, _params, default_device


class Triangle:
    """Triangle(p1, p2, p3) (triangle.cuh:13-19)."""

    def __init__(self, p1, p2, p3):
        self.v = np.array([p1, p2, p3], dtype=np.float64)

    def getNormal(self, r=None):
        n = np.cross(self.v[1] - self.v[0], self.v[2] - self.v[0])
        return n / np.linalg.norm(n)


class Mesh:
    """A closed triangle mesh: vertices[nvert, 3] (mm), triangles[ntri, 3]
    (vertex indices), D inside (mm^2/ms)."""

    def __init__(self, vertices, triangles, D):
        self.vertices = np.ascontiguousarray(vertices, dtype=np.float64).reshape(-1, 3)
        self.triangles = np.ascontiguousarray(triangles, dtype=np.int32).reshape(-1, 3)
        self.D = float(D)

    @classmethod
    def from_triangles(cls, tris, D):
        """From Triangle objects (each keeps its own three vertices)."""
        v = np.concatenate([t.v for t in tris])
        return cls(v, np.arange(len(v), dtype=np.int32).reshape(-1, 3), D)

    def record(self) -> N.MeshRec:
        return N.MeshRec(self.vertices.ctypes.data_as(C.POINTER(C.c_double)),
                         len(self.vertices),
                         self.triangles.ctypes.data_as(C.POINTER(C.c_int32)),
                         len(self.triangles), self.D)

    def volume(self) -> float:
        """Enclosed volume (divergence theorem; orientation-free)."""
        p = self.vertices[self.triangles]
        return abs(np.einsum("ij,ij->i", p[:, 0], np.cross(p[:, 1], p[:, 2])).sum()) / 6.0


def cube(side, D, center=(0.0, 0.0, 0.0)) -> Mesh:
    """An axis-aligned cube of 12 triangles."""
    h = side / 2.0
    c = np.asarray(center, dtype=np.float64)
    v = np.array([[x, y, z] for x in (-h, h) for y in (-h, h) for z in (-h, h)]) + c
    f = [(0, 1, 3), (0, 3, 2), (4, 6, 7), (4, 7, 5), (0, 4, 5), (0, 5, 1),
         (2, 3, 7), (2, 7, 6), (0, 2, 6), (0, 6, 4), (1, 5, 7), (1, 7, 3)]
    return Mesh(v, f, D)


def prism(polygon, z0, z1, D) -> Mesh:
    """The polygon (x, y vertices in order) extruded from z0 to z1; the caps
    are fans from the first vertex, so the polygon must be star-shaped from
    it (an L shape from its outer corner is)."""
    poly = np.asarray(polygon, dtype=np.float64).reshape(-1, 2)
    k = len(poly)
    v = np.vstack([np.column_stack([poly, np.full(k, z0)]),
                   np.column_stack([poly, np.full(k, z1)])])
    f = []
    for i in range(1, k - 1):
        f += [(0, i + 1, i), (k, k + i, k + i + 1)]
    for i in range(k):
        j = (i + 1) % k
        f += [(i, j, k + j), (i, k + j, k + i)]
    return Mesh(v, f, D)


def icosphere(radius, subdivisions, D, center=(0.0, 0.0, 0.0)) -> Mesh:
    """A sphere approximated by a subdivided icosahedron (20 * 4^k triangles),
    vertices on the sphere."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t),
         (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(p, dtype=np.float64) / np.linalg.norm(p) for p in v]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
             (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
             (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdivisions):
        mid = {}

        def midpoint(a, b):
            key = (min(a, b), max(a, b))
            if key not in mid:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                mid[key] = len(verts) - 1
            return mid[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return Mesh(np.array(verts) * radius + np.asarray(center, dtype=np.float64), faces, D)


def run_mesh(mesh: Mesh, seqs, num_walkers: int, steps: int, timestep: float, seed: int, *,
             gamma=GAMMA, walker_offset=0, device: Device = None) -> RunResult:
    """One mesh-pore walk (axx_run_mesh).  result.escaped counts walkers
    found outside the mesh after their walk."""
    dev = device or default_device()
    M = len(seqs)
    s = N.array_of(N.SequenceRec, [q.record() for q in seqs])
    p = _params(num_walkers, steps, seed, timestep, 0, gamma=gamma, offset=walker_offset)
    out = [np.zeros(max(M, 1)) for _ in range(5)]
    ptr = [o.ctypes.data_as(C.POINTER(C.c_double)) for o in out]
    st = N.Stats(ptr[2], ptr[3], ptr[4], 0, 0, 0)
    esc = C.c_int64(0)
    rec = mesh.record()
    N.check(N.lib().axx_run_mesh(dev.h, C.byref(rec), s, M, C.byref(p), ptr[0], ptr[1],
                                 C.byref(st), C.byref(esc)), dev.h)
    r = RunResult(*(o[:M] for o in out), st.reflection_cap_hits, st.walker_steps,
                  int(num_walkers), st.boundary_hits)
    r.escaped = int(esc.value)
    return r


def trace_mesh(mesh: Mesh, num_trace: int, steps: int, timestep: float, seed: int, *,
               walker_offset=0, device: Device = None):
    """Per-move record of the first walkers (axx_trace_mesh)."""
    dev = device or default_device()
    n = int(num_trace)
    nm = max(steps - 1, 0)
    p = _params(n, steps, seed, timestep, 0, offset=walker_offset)
    init = np.zeros((n, 3), np.float32)
    pos = np.zeros((n, nm, 3), np.float32)
    hits = np.zeros((n, nm), np.int32)
    words = np.zeros((n, nm), np.int32)
    esc = C.c_int64(0)
    rec = mesh.record()
    N.check(N.lib().axx_trace_mesh(dev.h, C.byref(rec), C.byref(p), n,
                                   init.ctypes.data_as(C.POINTER(C.c_float)),
                                   pos.ctypes.data_as(C.POINTER(C.c_float)),
                                   hits.ctypes.data_as(C.POINTER(C.c_int32)),
                                   words.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(esc)),
            dev.h)
    return {"init_pos": init, "pos": pos, "hits": hits, "words": words, "escaped": int(esc.value)}
