"""Host-side mirror of axonexa's acquisition API over the C ABI.

Names, argument order and meaning follow the reference's C++ classes so that
code written against them reads the same here:

* geometry  -- ``Cylinder_XY`` (src/primitives/cylinderXY.cuh:16-40),
  ``Sphere`` (src/primitives/Sphere.cuh:13-44), ``Lattice``
  (src/substrate/lattice.cuh:14-23);
* sequences -- ``RectGrad``, ``CosGFunc``, ``SinGFunc``, ``ApodCosGFunc``,
  ``SWOGSEFunc`` (src/functors/gfunctors.cuh);
* ``phaseAcquisition`` (src/acquisition/phaseAcquisition.cuh:1-86) and
  ``phaseAcquisitionStream`` (src/acquisition/phaseAcquisitionStream.cuh:4-642)
  with ``runAcquisitionLattice``, ``runAcquisition``,
  ``runAcquisitionStreamLattice``, ``runAcquisitionStream``, ``changeSeeds``,
  ``calcEveryADC`` and ``flushADC``.

The reference selects specular reflection, permeability and relaxation with
compile-time macros (SPECULAR_REFLECTION, USE_PERMEABLE, USE_RELAXATION); here
they are keyword arguments of the run calls.  The launch-shape arguments
(blocks, threads, numOfSM) are accepted and ignored: the library sizes its own
grid.  Results are the reference's unnormalised sums (getMx/getMy).
"""
from __future__ import annotations

import atexit
import ctypes as C
import math
import weakref
from typing import List, Sequence

import numpy as np

from . import _native as N

GAMMA = 267500.0  # rad / (ms * T), examples/gammadist.cu:5
PI = 3.1415926535897932384626433832795


class Vector3(tuple):
    def __new__(cls, x=0.0, y=0.0, z=0.0):
        return super().__new__(cls, (float(x), float(y), float(z)))

    x = property(lambda s: s[0])
    y = property(lambda s: s[1])
    z = property(lambda s: s[2])


# ---------------------------------------------------------------- geometry ---
class Cylinder_XY:
    """Infinite cylinder along z (cylinderXY.cuh:16-40)."""

    def __init__(self, centerX, centerY, radius, T2, T1, D, region, permeability, eps=1e-14):
        self.centerX, self.centerY, self.radius = float(centerX), float(centerY), float(radius)
        self.T2, self.T1, self.D = float(T2), float(T1), float(D)
        self.region, self.permeability, self.eps = int(region), float(permeability), float(eps)

    def inside(self, r) -> bool:
        return (r[0] - self.centerX) ** 2 + (r[1] - self.centerY) ** 2 < self.radius ** 2

    def getCenter(self):
        return Vector3(self.centerX, self.centerY, 0.0)

    def setCenter(self, v):
        self.centerX, self.centerY = float(v[0]), float(v[1])

    def setRadius(self, r):
        self.radius = float(r)

    def getRadius(self):
        return self.radius

    def setRegion(self, r):
        self.region = int(r)

    def getRegion(self):
        return self.region

    def record(self) -> N.Basis:
        return N.Basis(N.PRIM_CYLINDER_Z, self.region, self.centerX, self.centerY, 0.0,
                       self.radius, self.D, self.T2, self.T1, self.permeability, self.eps)


class Sphere:
    """Sphere (Sphere.cuh:13-44)."""

    def __init__(self, centerX, centerY, centerZ, radius, T2, T1, D, region, permeability,
                 eps=1e-14):
        self.centerX, self.centerY, self.centerZ = float(centerX), float(centerY), float(centerZ)
        self.radius, self.T2, self.T1, self.D = float(radius), float(T2), float(T1), float(D)
        self.region, self.permeability, self.eps = int(region), float(permeability), float(eps)

    def inside(self, r) -> bool:
        return ((r[0] - self.centerX) ** 2 + (r[1] - self.centerY) ** 2 +
                (r[2] - self.centerZ) ** 2 < self.radius ** 2)

    def getCenter(self):
        return Vector3(self.centerX, self.centerY, self.centerZ)

    def setCenter(self, v):
        self.centerX, self.centerY, self.centerZ = float(v[0]), float(v[1]), float(v[2])

    def getRadius(self):
        return self.radius

    def record(self) -> N.Basis:
        return N.Basis(N.PRIM_SPHERE, self.region, self.centerX, self.centerY, self.centerZ,
                       self.radius, self.D, self.T2, self.T1, self.permeability, self.eps)


class Cylinder:
    """Infinite cylinder through ``center`` along ``axis`` (cylinder.cuh:1-199;
    the reference's class is a draft that does not compile).  The library runs
    it as a Cylinder_XY in the cylinder's frame (ahat, bhat, chat) built as
    in cylinder.cuh:20-40, with gradient directions rotated into that frame:
    any axis for a single pore; in a lattice the cylinders share one axis
    along a cell axis (x, y or z)."""

    def __init__(self, center, axis, radius, T2, T1, D, region, permeability, eps=1e-14):
        self.center = tuple(float(v) for v in center)
        self.axis = tuple(float(v) for v in axis)
        self.radius, self.T2, self.T1, self.D = float(radius), float(T2), float(T1), float(D)
        self.region, self.permeability, self.eps = int(region), float(permeability), float(eps)

    def frame(self) -> np.ndarray:
        """Rows ahat, bhat, chat: r_frame = frame() @ r (cylinder.cuh:20-40)."""
        c = np.array(self.axis) / np.linalg.norm(self.axis)
        a = np.array([c[1], -c[0], 0.0])  # chat x z
        if np.hypot(a[0], a[1]) < 1e-14:
            a, b = np.array([1.0, 0.0, 0.0]), np.array([0.0, 1.0, 0.0])
        else:
            a = a / np.hypot(a[0], a[1])
            b = np.cross(c, a)
            b = b / np.linalg.norm(b)
        return np.vstack([a, b, c])

    def inside(self, r) -> bool:
        d = np.asarray(r, float) - np.array(self.center)
        c = np.array(self.axis) / np.linalg.norm(self.axis)
        p = d - np.dot(d, c) * c
        return float(np.dot(p, p)) < self.radius ** 2

    def getCenter(self):
        return Vector3(*self.center)

    def getRadius(self):
        return self.radius

    def getRegion(self):
        return self.region

    def record(self) -> N.Basis:
        c, a = self.center, self.axis
        return N.Basis(N.PRIM_CYLINDER, self.region, c[0], c[1], c[2], self.radius, self.D,
                       self.T2, self.T1, self.permeability, self.eps, a[0], a[1], a[2])


class Plane:
    """Infinite impermeable wall through ``center`` with normal ``normal``
    (plane.cuh:1-40).  It has no inside: it never holds a walker's region,
    D or T2 (getRegion 0, getT2/getD -1), reflects every crossing and
    transmits nothing.  Lattice bases only (planePhase.cu: walls at x = 0 and
    x = l of an l-wide cell make parallel plates).  The normal is normalised
    by the library."""

    def __init__(self, center, normal, eps=1e-14):
        self.center = tuple(float(v) for v in center)
        self.normal = tuple(float(v) for v in normal)
        self.eps = float(eps)
        self.region = 0

    def inside(self, r) -> bool:
        return False

    def getNormal(self, r=None):
        return Vector3(*self.normal)

    def getRegion(self, r=None):
        return 0

    def getPermeability(self):
        return 0.0

    def record(self) -> N.Basis:
        c, n = self.center, self.normal
        return N.Basis(N.PRIM_PLANE, 0, c[0], c[1], c[2], 0.0, 0.0, 0.0, 0.0, 0.0, self.eps,
                       n[0], n[1], n[2])


class Lattice:
    """Periodic a x b x c cell with the extracellular T2, T1, D (lattice.cuh:14-23)."""

    def __init__(self, a, b, c, T2, T1, D, basisSize=0):
        self.a, self.b, self.c = float(a), float(b), float(c)
        self.T2, self.T1, self.D = float(T2), float(T1), float(D)
        self.basisSize = int(basisSize)

    def getA(self):
        return self.a

    def getB(self):
        return self.b

    def getC(self):
        return self.c

    def getBasisSize(self):
        return self.basisSize

    def setBasisSize(self, n):
        self.basisSize = int(n)

    def record(self) -> N.LatticeRec:
        return N.LatticeRec(self.a, self.b, self.c, self.T2, self.T1, self.D)


# --------------------------------------------------------------- sequences ---
class _GFunc:
    kind = N.SEQ_PGSE

    def __init__(self, G, duration, spacing, num_periods, ghat):
        self.G, self.duration, self.spacing = float(G), float(duration), float(spacing)
        self.num_periods = int(num_periods)
        self.ghat = Vector3(*ghat)

    def record(self) -> N.SequenceRec:
        return N.SequenceRec(self.kind, self.num_periods, self.G, self.duration, self.spacing,
                             self.ghat[0], self.ghat[1], self.ghat[2])

    def getB(self, gamma: float = GAMMA) -> float:
        b = C.c_double()
        N.check(N.lib().axx_bvalue(C.byref(self.record()), gamma, C.byref(b)))
        return b.value

    def __call__(self, time: float) -> Vector3:
        t = (C.c_double * 1)(time)
        out = (C.c_double * 3)()
        N.check(N.lib().axx_gradient_eval(C.byref(self.record()), t, 1, out))
        return Vector3(*out)

    def getG(self):
        return self.G

    def getFreq(self):
        return self.num_periods / self.duration


class RectGrad(_GFunc):
    """PGSE (gfunctors.cuh:3-66): RectGrad(gstr, gd, gspac) along x, or
    RectGrad(b, gd, gspac, ghat) with the strength solved from the b-value."""

    kind = N.SEQ_PGSE

    def __init__(self, a, gd, gspac, ghat=None, gamma: float = GAMMA):
        if ghat is None:
            super().__init__(a, gd, gspac, 0, (1.0, 0.0, 0.0))
        else:
            g = math.sqrt(a / (gd * gd * gamma * gamma * ((2.0 / 3.0) * gd + gspac)))
            super().__init__(g, gd, gspac, 0, ghat)

    def getDiffusionTime(self):
        return self.spacing + self.duration


class CosGFunc(_GFunc):
    kind = N.SEQ_COS

    def __init__(self, G, gradientDuration, gradientSpacing, numOfPeriods, gHat=(1, 0, 0)):
        super().__init__(G, gradientDuration, gradientSpacing, numOfPeriods, gHat)


class SinGFunc(_GFunc):
    kind = N.SEQ_SIN

    def __init__(self, G, gradientDuration, gradientSpacing, numOfPeriods, gHat=(1, 0, 0)):
        super().__init__(G, gradientDuration, gradientSpacing, numOfPeriods, gHat)


class ApodCosGFunc(_GFunc):
    kind = N.SEQ_APODCOS

    def __init__(self, G, gradientDuration, gradientSpacing, numOfPeriods, gHat=(1, 0, 0)):
        super().__init__(G, gradientDuration, gradientSpacing, numOfPeriods, gHat)


class SWOGSEFunc(_GFunc):
    """Square-wave OGSE with sign (-1)^floor(2 t nu), nu = N / duration."""

    kind = N.SEQ_SQUARE

    def __init__(self, G, gradientDuration, gradientSpacing, numOfPeriods, gHat=(1, 0, 0)):
        super().__init__(G, gradientDuration, gradientSpacing, numOfPeriods, gHat)


# contexts still open at exit are closed (with their objects) before the
# CUDA runtime unloads
_LIVE_DEVICES: "weakref.WeakSet[Device]" = weakref.WeakSet()


@atexit.register
def _close_live_devices():
    for d in list(_LIVE_DEVICES):
        try:
            d.close()
        except Exception:
            pass


# ------------------------------------------------------------------ device ---
class Device:
    """One GPU context (axx_create).  Close it or use it as a context manager.

    Objects made on the context (batches, networks) register with it:
    closing the context closes them first, so that no handle outlives the
    context it was made on, whatever order the interpreter finalises them in
    (reference cycles, exit)."""

    def __init__(self, device: int = 0):
        L = N.lib()
        h = C.c_void_p()
        N.check(L.axx_create(C.byref(h), device))
        self.h = h
        self.device = device
        self._children = weakref.WeakSet()
        _LIVE_DEVICES.add(self)

    def adopt(self, obj):
        """Registers an object holding a handle made on this context; its
        close() runs before the context is destroyed."""
        self._children.add(obj)

    def close(self):
        if getattr(self, "h", None):
            for c in list(getattr(self, "_children", ())):
                try:
                    c.close()
                except Exception:
                    pass
            N.lib().axx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        n, ma, mi, mem = C.c_int(), C.c_int(), C.c_int(), C.c_size_t()
        N.check(N.lib().axx_device_info(self.h, C.byref(n), C.byref(ma), C.byref(mi),
                                        C.byref(mem)), self.h)
        return dict(num_sms=n.value, cc=(ma.value, mi.value), global_mem=mem.value)


_default_device = None


def default_device() -> Device:
    global _default_device
    if _default_device is None:
        _default_device = Device(0)
    return _default_device


def run_flags(specular=True, relaxation=False, permeable=False) -> int:
    f = 0
    if relaxation:
        f |= N.FLAG_RELAXATION
    if permeable:
        f |= N.FLAG_PERMEABLE
    if not specular:
        f |= N.FLAG_SIMPLE_REJECTION
    return f


class RunResult:
    def __init__(self, mx, my, sxx, syy, sxy, cap_hits, walker_steps, n, hits=0):
        self.mx, self.my = mx, my
        self.sxx, self.syy, self.sxy = sxx, syy, sxy
        self.cap_hits, self.walker_steps, self.n = cap_hits, walker_steps, n
        self.hits = hits
        # start-compartment sums (run_lattice(compartments=True)): walkers
        # that start inside a basis, and how many they are
        self.mx_in = self.my_in = None
        self.n_in = None

    @property
    def signal(self):
        """|M| / N per sequence."""
        return np.hypot(self.mx, self.my) / self.n

    @property
    def stderr(self):
        """Standard error of |M|/N per sequence (delta method on the walker
        terms x = cos(phi) e^{-T2f}, y = sin(phi) e^{-T2f})."""
        n = self.n
        mx, my = self.mx / n, self.my / n
        vxx = self.sxx / n - mx * mx
        vyy = self.syy / n - my * my
        vxy = self.sxy / n - mx * my
        s = np.hypot(mx, my)
        with np.errstate(invalid="ignore", divide="ignore"):
            ux = np.where(s > 0, mx / s, 1.0)
            uy = np.where(s > 0, my / s, 0.0)
        var = ux * ux * vxx + 2 * ux * uy * vxy + uy * uy * vyy
        return np.sqrt(np.maximum(var, 0.0) / n)


def _params(n, steps, seed, timestep, flags, init_mode=0, init_arg=0, gamma=GAMMA, offset=0):
    return N.RunParams(int(n), int(steps), int(init_mode), int(init_arg), int(flags),
                       int(seed) & 0xFFFFFFFFFFFFFFFF, float(timestep), float(gamma), int(offset))


def run_lattice(lattice: Lattice, basis: Sequence, seqs: Sequence, num_walkers: int, steps: int,
                timestep: float, seed: int, *, specular=True, relaxation=False, permeable=False,
                init_mode=0, init_arg=0, gamma=GAMMA, walker_offset=0, device: Device = None,
                allow_cap=False, compartments=False) -> RunResult:
    """One lattice walk (axx_run_lattice): host records in, FP64 sums out.
    compartments: also the sums over the walkers that start inside a basis
    (result.mx_in, result.my_in, result.n_in)."""
    dev = device or default_device()
    L = N.lib()
    M = len(seqs)
    b = N.array_of(N.Basis, [x.record() for x in basis])
    s = N.array_of(N.SequenceRec, [q.record() for q in seqs])
    flags = run_flags(specular, relaxation, permeable) | (N.FLAG_COMPARTMENTS if compartments
                                                          else 0)
    p = _params(num_walkers, steps, seed, timestep, flags, init_mode, init_arg, gamma,
                walker_offset)
    out = [np.zeros(max(M, 1)) for _ in range(7)]
    ptr = [o.ctypes.data_as(C.POINTER(C.c_double)) for o in out]
    st = N.Stats(ptr[2], ptr[3], ptr[4], 0, 0, 0, ptr[5], ptr[6], 0)
    rc = L.axx_run_lattice(dev.h, C.byref(lattice.record()), b, len(basis), s, M, C.byref(p),
                           ptr[0], ptr[1], C.byref(st))
    if not (allow_cap and rc == 3):
        N.check(rc, dev.h)
    r = RunResult(*(o[:M] for o in out[:5]), st.reflection_cap_hits, st.walker_steps,
                  int(num_walkers), st.boundary_hits)
    if compartments:
        r.mx_in, r.my_in, r.n_in = out[5][:M], out[6][:M], int(st.walkers_in)
    return r


def run_single(basis, seqs: Sequence, num_walkers: int, steps: int, timestep: float, seed: int,
               *, specular=True, gamma=GAMMA, fix_init_quirk=False, lattice_picking=False,
               device: Device = None, walker_offset=0) -> RunResult:
    """One single-pore walk (axx_run_single); lattice_picking: the
    LATTICE_PICKING moves of kernelPhase.cuh:31-35."""
    dev = device or default_device()
    L = N.lib()
    M = len(seqs)
    s = N.array_of(N.SequenceRec, [q.record() for q in seqs])
    flags = (run_flags(specular) | (N.FLAG_FIX_INIT_QUIRK if fix_init_quirk else 0) |
             (N.FLAG_LATTICE_PICKING if lattice_picking else 0))
    p = _params(num_walkers, steps, seed, timestep, flags, gamma=gamma, offset=walker_offset)
    out = [np.zeros(max(M, 1)) for _ in range(5)]
    ptr = [o.ctypes.data_as(C.POINTER(C.c_double)) for o in out]
    st = N.Stats(ptr[2], ptr[3], ptr[4], 0, 0, 0)
    rc = L.axx_run_single(dev.h, C.byref(basis.record()), s, M, C.byref(p), ptr[0], ptr[1],
                          C.byref(st))
    N.check(rc, dev.h)
    return RunResult(*(o[:M] for o in out), st.reflection_cap_hits, st.walker_steps,
                     int(num_walkers), st.boundary_hits)


def trace_lattice(lattice: Lattice, basis: Sequence, num_trace: int, steps: int, timestep: float,
                  seed: int, *, specular=True, relaxation=False, permeable=False, init_mode=0,
                  init_arg=0, walker_offset=0, device: Device = None):
    """Per-move record of the first walkers (axx_trace_lattice)."""
    dev = device or default_device()
    p = _params(num_trace, steps, seed, timestep, run_flags(specular, relaxation, permeable),
                init_mode, init_arg, GAMMA, walker_offset)
    return _trace(dev, p, num_trace, steps,
                  lambda ip, pos, reg, hit, wd: N.lib().axx_trace_lattice(
                      dev.h, C.byref(lattice.record()),
                      N.array_of(N.Basis, [x.record() for x in basis]), len(basis), C.byref(p),
                      num_trace, ip, pos, reg, hit, wd))


def trace_single(basis, num_trace: int, steps: int, timestep: float, seed: int, *,
                 specular=True, fix_init_quirk=False, lattice_picking=False,
                 device: Device = None):
    dev = device or default_device()
    flags = (run_flags(specular) | (N.FLAG_FIX_INIT_QUIRK if fix_init_quirk else 0) |
             (N.FLAG_LATTICE_PICKING if lattice_picking else 0))
    p = _params(num_trace, steps, seed, timestep, flags)
    return _trace(dev, p, num_trace, steps,
                  lambda ip, pos, reg, hit, wd: N.lib().axx_trace_single(
                      dev.h, C.byref(basis.record()), C.byref(p), num_trace, ip, pos, reg, hit, wd))


def _trace(dev, p, n, steps, call):
    m = n * max(steps - 1, 0)
    ip = np.zeros(n * 3, np.float32)
    pos = np.zeros(m * 3, np.float32)
    reg = np.zeros(m, np.int32)
    hit = np.zeros(m, np.int32)
    wd = np.zeros(m, np.int32)
    f = lambda a, t: a.ctypes.data_as(C.POINTER(t))
    N.check(call(f(ip, C.c_float), f(pos, C.c_float), f(reg, C.c_int32), f(hit, C.c_int32),
                 f(wd, C.c_int32)), dev.h)
    return dict(init_pos=ip.reshape(n, 3), pos=pos.reshape(n, steps - 1, 3),
                region=reg.reshape(n, steps - 1), hits=hit.reshape(n, steps - 1),
                words=wd.reshape(n, steps - 1))


def philox_words(seed: int, walker: int, n: int, device: Device = None) -> np.ndarray:
    dev = device or default_device()
    out = np.zeros(n, np.uint32)
    N.check(N.lib().axx_philox_words(dev.h, seed, walker, n,
                                     out.ctypes.data_as(C.POINTER(C.c_uint32))), dev.h)
    return out


# ------------------------------------------------------------- acquisition ---
def wc_start(basis, n: int, seed: int):
    """Per-walker non-zero 32-bit xorshift states and start points uniform
    in the pore (the host side of runAcquisitionWC, seeded generator)."""
    rng = np.random.default_rng(int(seed) & 0xFFFFFFFFFFFFFFFF)
    state = rng.integers(1, 1 << 32, size=n, dtype=np.uint64).astype(np.uint32)
    if isinstance(basis, Cylinder):
        # the same draws for the cylinder in its own frame, rotated back
        F = basis.frame()
        cf = F @ np.array(basis.center)
        xy = Cylinder_XY(cf[0], cf[1], basis.radius, basis.T2, basis.T1, basis.D,
                         basis.region, basis.permeability, basis.eps)
        st2, pf = wc_start(xy, n, seed)
        return st2, pf @ F
    R = basis.radius if hasattr(basis, "radius") else basis.getRadius()
    sph = isinstance(basis, Sphere)
    c = np.array([basis.centerX, basis.centerY, basis.centerZ if sph else 0.0])
    out = np.zeros((n, 3))
    filled = 0
    while filled < n:
        p = rng.uniform(-1.0, 1.0, size=(2 * (n - filled) + 16, 3)) * R
        if not sph:
            p[:, 2] = (p[:, 2] + R)  # z in [0, 2R) as Cylinder_XY::unifRandCPU
        q = p[:, 0] ** 2 + p[:, 1] ** 2 + (p[:, 2] ** 2 if sph else 0.0)
        p = p[q < R * R][: n - filled]
        out[filled:filled + len(p)] = p + np.array([c[0], c[1], c[2] if sph else 0.0])
        filled += len(p)
    return state, out


def run_wc(basis, rng_state, start, grad, timestep: float, *, gamma: float = GAMMA,
           return_phase: bool = False, device: Device = None):
    """The WCDMC comparison walker (axx_run_wc).  Returns (phases | None,
    sum cos(phase), sum sin(phase))."""
    dev = device or default_device()
    st = np.ascontiguousarray(rng_state, np.uint32)
    p0 = np.ascontiguousarray(start, np.float64)
    g = np.ascontiguousarray(grad, np.float64)
    n = len(st)
    ph = np.zeros(n) if return_phase else None
    sc, ss = C.c_double(), C.c_double()
    N.check(N.lib().axx_run_wc(dev.h, C.byref(basis.record()), n, len(g), float(timestep),
                               float(gamma), st.ctypes.data_as(C.POINTER(C.c_uint32)),
                               p0.ctypes.data_as(C.POINTER(C.c_double)),
                               g.ctypes.data_as(C.POINTER(C.c_double)),
                               ph.ctypes.data_as(C.POINTER(C.c_double)) if return_phase else None,
                               C.byref(sc), C.byref(ss)), dev.h)
    return ph, sc.value, ss.value


def linear_regression(y, x) -> float:
    """Slope of y on x (misc.cuh:41-59)."""
    if len(y) != len(x):
        raise ValueError("linear_regression: y.size != x.size")
    n = float(len(y))
    # plain left-to-right sums, as the reference's loop (Python's sum() of
    # floats is compensated and would round differently)
    t2 = t3 = t4 = t5 = 0.0
    for a, b in zip(x, y):
        t2 = t2 + a * b
        t3 = t3 + a
        t4 = t4 + b
        t5 = t5 + a * a
    delta = n * t5 - t3 * t3
    return (1.0 / delta) * (n * t2 - t3 * t4)


class phaseAcquisition:
    """phaseAcquisition<FieldType> (phaseAcquisition.cuh:1-86)."""

    def __init__(self, numOfMeas, numOfSteps, numOfParticles, seed):
        self.numOfMeasurements = int(numOfMeas)
        self.numOfSteps = int(numOfSteps)
        self.seed = int(seed)
        self.mx = [0.0] * self.numOfMeasurements
        self.my = [0.0] * self.numOfMeasurements
        self.gradientFunctors: List[_GFunc] = []
        self.ADC = 0.0
        self.ADCmeansquare = 0.0
        self.points = 0
        self.last: RunResult | None = None

    def addMeasurement(self, field):
        if len(self.gradientFunctors) >= self.numOfMeasurements:
            raise IndexError("more measurements than numOfMeas")
        self.gradientFunctors.append(field)

    def getGradientFunctors(self):
        return self.gradientFunctors

    def getMx(self):
        return self.mx

    def getMy(self):
        return self.my

    def getSignal(self, i):
        return math.sqrt(self.mx[i] * self.mx[i] + self.my[i] * self.my[i])

    def getNumOfMeas(self):
        return self.numOfMeasurements

    def getNumOfSteps(self):
        return self.numOfSteps

    def getSeed(self):
        return self.seed

    def calcADC(self):
        """ADC from ln|M| against b with running mean over repeats (:54-77)."""
        self.points += 1
        b = [f.getB() for f in self.gradientFunctors]
        ln = [math.log(math.sqrt(self.mx[i] * self.mx[i] + self.my[i] * self.my[i]))
              for i in range(self.numOfMeasurements)]
        adc = -1.0 * linear_regression(ln, b)
        if self.points == 1:
            self.ADC = adc
            self.ADCmeansquare = adc * adc
        else:
            p = self.points
            self.ADC = (self.ADC * (p - 1) + adc) / p
            self.ADCmeansquare = (self.ADCmeansquare * (p - 1) + adc * adc) / p

    def getADC(self):
        return self.ADC

    def getADCMeanSquare(self):
        return self.ADCmeansquare

    def getPoints(self):
        return self.points

    def getADCError(self):
        return math.sqrt(max(self.ADCmeansquare - self.ADC * self.ADC, 0.0))


class phaseAcquisitionStream:
    """phaseAcquisitionStream<FieldType> (phaseAcquisitionStream.cuh:4-642)."""

    def __init__(self, num: int, device: Device = None):
        self.number_of_particles = int(num)
        self.acqSet: List[phaseAcquisition] = []
        self.device = device

    def addAcquisition(self, acq: phaseAcquisition):
        self.acqSet.append(acq)

    def getAcquisition(self, num: int) -> phaseAcquisition:
        return self.acqSet[num]

    def _store(self, acq, res: RunResult):
        acq.mx = list(res.mx)
        acq.my = list(res.my)
        acq.last = res

    def runAcquisitionLattice(self, num, basis, lat, timestep, blocks=None, threads=None,
                              numOfSM=None, *, specular=True, relaxation=False, permeable=False,
                              init_mode=0, init_arg=0):
        acq = self.acqSet[num]
        nb = lat.getBasisSize() if lat.getBasisSize() else len(basis)
        res = run_lattice(lat, list(basis)[:nb], acq.gradientFunctors, self.number_of_particles,
                          acq.numOfSteps, timestep, acq.seed, specular=specular,
                          relaxation=relaxation, permeable=permeable, init_mode=init_mode,
                          init_arg=init_arg, device=self.device)
        self._store(acq, res)

    def runAcquisition(self, num, basis, timestep, blocks=None, threads=None, numOfSM=None, *,
                       specular=True):
        acq = self.acqSet[num]
        res = run_single(basis, acq.gradientFunctors, self.number_of_particles, acq.numOfSteps,
                         timestep, acq.seed, specular=specular, device=self.device)
        self._store(acq, res)

    def runAcquisitionWC(self, num, basis, timestep, blocks=None, threads=None):
        """runAcquisitionWC (phaseAcquisitionStream.cuh:193-252): per
        measurement the WCDMC walker (axx_run_wc) with the functor's G(j dt)
        table.  The host-side draws (per-walker xorshift states and
        start points in the pore) come from a generator seeded with the
        acquisition's seed instead of srand/rand."""
        acq = self.acqSet[num]
        n, steps = self.number_of_particles, acq.numOfSteps
        for i, g in enumerate(acq.gradientFunctors):
            grad = np.array([tuple(g(j * timestep)) for j in range(steps)], dtype=np.float64)
            state, start = wc_start(basis, n, acq.seed)
            r = run_wc(basis, state, start, grad, timestep, device=self.device)
            acq.mx[i], acq.my[i] = r[1], r[2]

    def runAcquisitionStreamLattice(self, basis, lat, timestep, blocks=None, threads=None,
                                    numOfDevices=1, plan=None, numOfSMPerDevice=None, **kw):
        for i in range(len(self.acqSet)):
            self.runAcquisitionLattice(i, basis, lat, timestep, **kw)

    def runAcquisitionStream(self, basis, timestep, blocks=None, threads=None, numOfDevices=1,
                             plan=None, numOfSMPerDevice=None, **kw):
        for i in range(len(self.acqSet)):
            self.runAcquisition(i, basis, timestep, **kw)

    def addMagnetizationSet(self, host_mx, host_my):
        """Stores per-acquisition sums (phaseAcquisitionStream.cuh:615-621)."""
        for i, a in enumerate(self.acqSet):
            a.mx = [float(v) for v in host_mx[i]]
            a.my = [float(v) for v in host_my[i]]

    def changeSeeds(self, seed):
        for i, a in enumerate(self.acqSet):
            a.seed = int(seed) * (i + 1)

    def calcEveryADC(self):
        for a in self.acqSet:
            a.calcADC()

    def flushADC(self):
        for a in self.acqSet:
            a.ADC = 0.0
            a.ADCmeansquare = 0.0
            a.points = 0
