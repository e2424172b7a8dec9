"""Substrate builders: gamma-radius random packings (native) and the
hexagonal four-cylinder cell of the reference's hexPhase example."""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _native as N
from .acquisition import Cylinder_XY, Lattice


def rps_gamma_pack(seed: int, n: int, shape: float, mean: float, fraction: float, *,
                   rmin: float = None, rmax: float = None, D_in: float, T2_in: float,
                   D_ex: float, T2_ex: float, permeability: float = 0.0):
    """n cylinders with gamma(shape, mean/shape) radii at area fraction
    `fraction` in a periodic square cell (axx_substrate_rps_gamma).
    Returns (Lattice, [Cylinder_XY...], achieved_fraction); the list holds the
    originals then the periodic images of edge-crossing cylinders."""
    rmin = mean * 0.05 if rmin is None else rmin
    rmax = mean * 4.0 if rmax is None else rmax
    cap = n * 9
    out = (N.Basis * cap)()
    nout, side, ach = C.c_int(), C.c_double(), C.c_double()
    N.check(N.lib().axx_substrate_rps_gamma(seed, n, shape, mean, rmin, rmax, fraction, D_in,
                                            T2_in, permeability, cap, out, C.byref(nout),
                                            C.byref(side), C.byref(ach)))
    return _packing(out, nout, side, ach, T2_ex, D_ex)


def rps_gamma_pack_gpu(seed: int, n: int, specs, *, T2_ex: float, D_ex: float, device=None):
    """Many gamma packings at once on the GPU (axx_substrate_rps_gamma_gpu).
    specs: one dict per packing with shape, mean, fraction, D_in, T2_in and
    optionally permeability, rmin, rmax (defaults as rps_gamma_pack).
    Returns [(Lattice, [Cylinder_XY...], achieved_fraction), ...]."""
    from .acquisition import default_device
    dev = device or default_device()
    npack = len(specs)
    arr = (N.PackSpec * npack)()
    for i, s in enumerate(specs):
        mean = s["mean"]
        arr[i] = N.PackSpec(s["shape"], mean, s.get("rmin", mean * 0.05), s.get("rmax", mean * 4.0),
                            s["fraction"], s["D_in"], s["T2_in"], s.get("permeability", 0.0))
    cap = n * 4
    out = (N.Basis * (cap * npack))()
    nout = (C.c_int * npack)()
    side = (C.c_double * npack)()
    ach = (C.c_double * npack)()
    N.check(N.lib().axx_substrate_rps_gamma_gpu(dev.h, seed, n, npack, arr, cap, out, nout, side,
                                                ach), dev.h)
    res = []
    base = C.addressof(out)
    for p in range(npack):
        view = (N.Basis * cap).from_address(base + p * cap * C.sizeof(N.Basis))
        res.append(_packing(view, C.c_int(nout[p]), C.c_double(side[p]), C.c_double(ach[p]),
                            T2_ex, D_ex))
    return res


def pack_radii(seed: int, radii, fraction: float, *, D_in: float, T2_in: float, D_ex: float,
               T2_ex: float, permeability: float = 0.0):
    """The placement step of rps_gamma_pack for given radii
    (axx_substrate_pack).  Same return value."""
    r = np.ascontiguousarray(radii, dtype=np.float64)
    cap = len(r) * 9
    out = (N.Basis * cap)()
    nout, side, ach = C.c_int(), C.c_double(), C.c_double()
    N.check(N.lib().axx_substrate_pack(seed, len(r), r.ctypes.data_as(C.POINTER(C.c_double)),
                                       fraction, D_in, T2_in, permeability, cap, out,
                                       C.byref(nout), C.byref(side), C.byref(ach)))
    return _packing(out, nout, side, ach, T2_ex, D_ex)


def gamma_quantile_radii(n: int, shape: float, mean: float) -> np.ndarray:
    """n radii at the mid-quantiles (i + 1/2)/n of gamma(shape, mean/shape):
    a packing whose radius distribution is the gamma law itself rather than a
    random sample of it."""
    from scipy.special import gammaincinv
    q = (np.arange(n) + 0.5) / n
    return gammaincinv(shape, q) * (mean / shape)


def _packing(out, nout, side, ach, T2_ex, D_ex):
    L = side.value
    cyl = []
    for i in range(nout.value):
        b = out[i]
        cyl.append(Cylinder_XY(b.cx, b.cy, b.radius, b.T2, b.T1, b.D, b.region, b.permeability,
                               b.eps))
    lat = Lattice(L, L, L, T2_ex, 0.0, D_ex, len(cyl))
    return lat, cyl, ach.value


def hex_cell(radius: float, fraction: float, *, D_in, T2_in, D_ex, T2_ex, permeability=0.0):
    """Hexagonal packing as a periodic d x 2h cell holding four cylinders
    (examples/hexPhase.cu:110-124): d = sqrt(2 pi r^2 / (sqrt(3) f))."""
    d = math.sqrt(2.0 * math.pi * radius * radius / (math.sqrt(3.0) * fraction))
    h = d * 0.86602540378443864676372317075294
    cyl = [Cylinder_XY(d / 2.0, 0.0, radius, T2_in, 0.0, D_in, 1, permeability),
           Cylinder_XY(0.0, h, radius, T2_in, 0.0, D_in, 2, permeability),
           Cylinder_XY(d / 2.0, 2.0 * h, radius, T2_in, 0.0, D_in, 3, permeability),
           Cylinder_XY(d, h, radius, T2_in, 0.0, D_in, 4, permeability)]
    return Lattice(d, 2.0 * h, d, T2_ex, 0.0, D_ex, 4), cyl


def volume_fraction(lattice, basis, points: int = 1 << 22, seed: int = 1234, device=None):
    """Monte Carlo intracellular volume fraction of a lattice substrate
    (axx_volume_fraction; the reference's calcf, src/util/calcf.cuh).
    Returns (fraction, count)."""
    from .acquisition import default_device
    dev = device or default_device()
    b = N.array_of(N.Basis, [x.record() for x in basis])
    f, n = C.c_double(), C.c_int64()
    N.check(N.lib().axx_volume_fraction(dev.h, C.byref(lattice.record()), b, len(basis),
                                        int(points), int(seed), C.byref(f), C.byref(n)), dev.h)
    return f.value, n.value
