"""ctypes binding of the CPU oracle (liboracle.so) and of the reference's own
walker compiled for the host (_ref/libaxxref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline arm of bench.py, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REFLIB = os.path.join(HERE, "_ref", "libaxxref.so")
REFLIB_ACQ = os.path.join(HERE, "_ref", "libaxxref_acq.so")
# The reference's source tree (for building its walker for the host): the
# AXX_REFERENCE_SRC environment variable, or the path given to build().
REF_SRC = os.environ.get("AXX_REFERENCE_SRC", "")
REF_SRC_RECORD = os.path.join(HERE, "_ref", "ref_src.txt")

REF64, KERN64, KERN32 = 0, 1, 2
REF_VARIANTS = ("spec_imp", "spec_imp_t2", "spec_perm", "spec_perm_t2", "rej", "rej_t2",
                "pick_spec", "pick_rej")
FLAG_LATTICE_PICKING = 32


class Basis(C.Structure):
    _fields_ = [("type", C.c_int32), ("region", C.c_int32), ("cx", C.c_double),
                ("cy", C.c_double), ("cz", C.c_double), ("radius", C.c_double),
                ("D", C.c_double), ("T2", C.c_double), ("T1", C.c_double),
                ("permeability", C.c_double), ("eps", C.c_double),
                ("nx", C.c_double), ("ny", C.c_double), ("nz", C.c_double)]


class Lattice(C.Structure):
    _fields_ = [("a", C.c_double), ("b", C.c_double), ("c", C.c_double),
                ("T2", C.c_double), ("T1", C.c_double), ("D", C.c_double)]


class Sequence(C.Structure):
    _fields_ = [("kind", C.c_int32), ("num_periods", C.c_int32), ("G", C.c_double),
                ("duration", C.c_double), ("spacing", C.c_double), ("gx", C.c_double),
                ("gy", C.c_double), ("gz", C.c_double)]


class Params(C.Structure):
    _fields_ = [("num_walkers", C.c_int64), ("steps", C.c_int32), ("init_mode", C.c_int32),
                ("init_arg", C.c_int32), ("flags", C.c_uint32), ("seed", C.c_uint64),
                ("timestep", C.c_double), ("gamma", C.c_double), ("walker_offset", C.c_int64)]


class Trace(C.Structure):
    _fields_ = [("ntrace", C.c_int32), ("init_pos", C.POINTER(C.c_double)),
                ("pos", C.POINTER(C.c_double)), ("region", C.POINTER(C.c_int32)),
                ("hits", C.POINTER(C.c_int32)), ("words", C.POINTER(C.c_int32))]


def build(ref: bool = True, ref_src: str = None) -> None:
    """Builds liboracle.so, and _ref/libaxxref.so + _ref/libaxxref_acq.so when
    the reference tree (`ref_src`, else AXX_REFERENCE_SRC) exists."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    src = ref_src or REF_SRC
    if ref and src and os.path.isdir(os.path.join(src, "src")):
        subprocess.run(["make", "-s", "-j8", "-C", HERE, "ref", "REF=" + src], check=True)
        with open(REF_SRC_RECORD, "w") as f:
            f.write(os.path.abspath(src))


def reference_src():
    """The reference source tree _ref/ was built from, or None."""
    if REF_SRC and os.path.isdir(os.path.join(REF_SRC, "src")):
        return REF_SRC
    try:
        with open(REF_SRC_RECORD) as f:
            p = f.read().strip()
    except OSError:
        return None
    return p if os.path.isdir(os.path.join(p, "src")) else None


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build(ref=False)
        _lib = C.CDLL(LIB)
        _lib.orc_walk.restype = C.c_int
        _lib.orc_step.restype = C.c_int
        _lib.orc_bvalue.restype = C.c_double
    return _lib


def reflib():
    """The reference's walker, or None when it was not built here."""
    global _ref
    if _ref is None and os.path.exists(REFLIB):
        _ref = C.CDLL(REFLIB)
    return _ref


_ref_acq = None


def reflib_acq():
    """The reference's acquisition post-processing (linear_regression,
    phaseAcquisition::calcADC), or None when it was not built here."""
    global _ref_acq
    if _ref_acq is None and os.path.exists(REFLIB_ACQ):
        L = C.CDLL(REFLIB_ACQ)
        L.ref_linear_regression.restype = C.c_double
        L.ref_linear_regression.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int]
        L.ref_calc_adc.restype = C.c_int
        _ref_acq = L
    return _ref_acq


def _arr(seq, cls):
    seq = list(seq)
    a = (cls * max(len(seq), 1))()
    for i, s in enumerate(seq):
        a[i] = s
    return a


def make_trace(ntrace: int, steps: int):
    n = ntrace * max(steps - 1, 0)
    bufs = dict(init_pos=np.zeros(ntrace * 3), pos=np.zeros(n * 3),
                region=np.zeros(n, np.int32), hits=np.zeros(n, np.int32),
                words=np.zeros(n, np.int32))
    t = Trace(ntrace,
              bufs["init_pos"].ctypes.data_as(C.POINTER(C.c_double)),
              bufs["pos"].ctypes.data_as(C.POINTER(C.c_double)),
              bufs["region"].ctypes.data_as(C.POINTER(C.c_int32)),
              bufs["hits"].ctypes.data_as(C.POINTER(C.c_int32)),
              bufs["words"].ctypes.data_as(C.POINTER(C.c_int32)))
    return t, bufs


def _shape_trace(bufs, ntrace, steps):
    return dict(init_pos=bufs["init_pos"].reshape(ntrace, 3),
                pos=bufs["pos"].reshape(ntrace, steps - 1, 3),
                region=bufs["region"].reshape(ntrace, steps - 1),
                hits=bufs["hits"].reshape(ntrace, steps - 1),
                words=bufs["words"].reshape(ntrace, steps - 1))


def walk(lat, bases, seqs, params, mode=REF64, nthreads=1, ntrace=0):
    """Runs the oracle.  lat None = single pore.  Returns (sums[M,5], trace|None, caps);
    with flag 64 (compartment sums) on a lattice, sums[2M,5]: rows M.. sum the
    walkers that start inside a basis."""
    L = lib()
    b = _arr(bases, Basis)
    s = _arr(seqs, Sequence)
    rows = 2 * len(seqs) if (lat is not None and params.flags & 64) else len(seqs)
    sums = np.zeros(max(rows, 1) * 5)
    tr, bufs = (make_trace(ntrace, params.steps) if ntrace else (None, None))
    caps = C.c_int64(0)
    rc = L.orc_walk(C.byref(lat) if lat is not None else None, b, len(bases), s, len(seqs),
                    C.byref(params), mode, nthreads,
                    sums.ctypes.data_as(C.POINTER(C.c_double)),
                    C.byref(tr) if tr is not None else None, C.byref(caps))
    if rc != 0:
        raise ValueError("orc_walk failed: %d" % rc)
    return (sums[: rows * 5].reshape(rows, 5),
            _shape_trace(bufs, ntrace, params.steps) if ntrace else None, caps.value)


def mesh_walk(vertices, triangles, D, seqs, params, mode=KERN32, nthreads=1, ntrace=0):
    """The mesh-pore walk (GPU formulation, FP64 or FP32).  Returns
    (sums[M,5], trace|None, escaped)."""
    L = lib()
    v = np.ascontiguousarray(vertices, np.float64)
    t = np.ascontiguousarray(triangles, np.int32)
    s = _arr(seqs, Sequence)
    sums = np.zeros(max(len(seqs), 1) * 5)
    tr, bufs = (make_trace(ntrace, params.steps) if ntrace else (None, None))
    esc = C.c_int64(0)
    rc = L.orc_mesh_walk(v.ctypes.data_as(C.POINTER(C.c_double)), len(v),
                         t.ctypes.data_as(C.POINTER(C.c_int32)), len(t), C.c_double(D), s, len(seqs),
                         C.byref(params), mode, nthreads,
                         sums.ctypes.data_as(C.POINTER(C.c_double)),
                         C.byref(tr) if tr is not None else None, C.byref(esc))
    if rc != 0:
        raise ValueError("orc_mesh_walk failed: %d" % rc)
    return (sums[: len(seqs) * 5].reshape(len(seqs), 5),
            _shape_trace(bufs, ntrace, params.steps) if ntrace else None, esc.value)


def ref_walk(variant, lat, bases, seqs, params, nthreads=1, ntrace=0):
    """Runs the reference's own walker (compiled here); None if unavailable."""
    R = reflib()
    if R is None:
        return None
    fn = getattr(R, "ref_walk_" + variant)
    b = _arr(bases, Basis)
    s = _arr(seqs, Sequence)
    sums = np.zeros(max(len(seqs), 1) * 5)
    tr, bufs = (make_trace(ntrace, params.steps) if ntrace else (None, None))
    rc = fn(C.byref(lat) if lat is not None else None, b, len(bases), s, len(seqs),
            C.byref(params), nthreads, sums.ctypes.data_as(C.POINTER(C.c_double)),
            C.byref(tr) if tr is not None else None)
    if rc != 0:
        raise ValueError("ref_walk_%s failed: %d" % (variant, rc))
    return (sums[: len(seqs) * 5].reshape(len(seqs), 5),
            _shape_trace(bufs, ntrace, params.steps) if ntrace else None)


def variant_for(flags: int) -> str:
    spec = not (flags & 4)
    if flags & FLAG_LATTICE_PICKING:
        return "pick_spec" if spec else "pick_rej"
    t2 = bool(flags & 1)
    perm = bool(flags & 2)
    if spec:
        return ("spec_perm" if perm else "spec_imp") + ("_t2" if t2 else "")
    return "rej_t2" if t2 else "rej"


def stream_words(seed: int, walker: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.uint32)
    lib().orc_stream_words(C.c_uint64(seed), C.c_uint64(walker), n,
                           out.ctypes.data_as(C.POINTER(C.c_uint32)))
    return out


def philox(ctr, key) -> np.ndarray:
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, o)
    return np.array(list(o), np.uint32)


def sincos_2pi_f32(u: float):
    s, c = C.c_float(), C.c_float()
    lib().orc_sincos_2pi_f32(C.c_float(u), C.byref(s), C.byref(c))
    return s.value, c.value


def step(lat, bases, params, mode, walker, i, r_in, word):
    b = _arr(bases, Basis)
    rin = (C.c_double * 3)(*r_in)
    rout = (C.c_double * 3)()
    reg, hits, wout = C.c_int32(), C.c_int32(), C.c_int32()
    rc = lib().orc_step(C.byref(lat), b, len(bases), C.byref(params), mode, C.c_int64(walker), i,
                        rin, C.c_int32(word), rout, C.byref(reg), C.byref(hits), C.byref(wout))
    if rc != 0:
        raise ValueError("orc_step failed")
    return np.array(list(rout)), reg.value, hits.value, wout.value


def bvalue(seq, gamma=0.0) -> float:
    return lib().orc_bvalue(C.byref(seq), C.c_double(gamma))


def gradient(seq, t: float):
    out = (C.c_double * 3)()
    lib().orc_gradient(C.byref(seq), C.c_double(t), out)
    return np.array(list(out))


# ---- magnetisation (Bloch) path --------------------------------------------
MAG_VARIANTS = ("mag_rot_spec", "mag_rot_rej", "mag_rk4_spec", "mag_ms_spec")
ROTATE, RK4, MULTISTEP, DORP = 0, 1, 2, 3


class Field(C.Structure):
    _fields_ = [("kind", C.c_int32), ("num_periods", C.c_int32), ("B0", C.c_double),
                ("G", C.c_double), ("gx", C.c_double), ("gy", C.c_double), ("gz", C.c_double),
                ("duration", C.c_double), ("spacing", C.c_double), ("period", C.c_double),
                ("ramp", C.c_double), ("rf_duration", C.c_double), ("dtmin", C.c_double),
                ("dtmax", C.c_double), ("TE", C.c_double)]


class MagParams(C.Structure):
    _fields_ = [("num_walkers", C.c_int64), ("steps", C.c_int32), ("integrator", C.c_int32),
                ("flags", C.c_uint32), ("dorp_levels", C.c_uint32), ("seed", C.c_uint64),
                ("timestep", C.c_double), ("gamma", C.c_double), ("m0", C.c_double * 3),
                ("walker_offset", C.c_int64), ("dorp_tol", C.c_double)]


def mag_params(n, steps, seed, dt, integrator=ROTATE, reject=False, gamma=267500.0,
               m0=(1.0, 0.0, 0.0), offset=0, dorp_levels=0, dorp_tol=0.0):
    return MagParams(n, steps, integrator, 4 if reject else 0, dorp_levels, seed, dt, gamma,
                     (C.c_double * 3)(*m0), offset, dorp_tol)


def mag_variant(integrator: int, reject: bool) -> str:
    """The reference build of an integrator, or None (no reference build:
    rejection walks other than the rotation, and Dormand-Prince)."""
    if reject:
        return "mag_rot_rej" if integrator == ROTATE else None
    if integrator == DORP:
        return None
    return ("mag_rot_spec", "mag_rk4_spec", "mag_ms_spec")[integrator]


def _mag_out(sums, mw, bufs, nf, ntrace, steps):
    return (sums.reshape(nf, 3), mw.reshape(ntrace, nf, 3) if ntrace else None,
            _shape_trace(bufs, ntrace, steps) if ntrace else None)


def mag_walk(pore, fields, params, nthreads=1, ntrace=0):
    """updateWalkersMag restated (FP64, reference order).  Returns
    (sums[nf,3], final M of the first ntrace walkers [ntrace,nf,3] | None,
    their traces | None)."""
    L = lib()
    nf = len(fields)
    f = _arr(fields, Field)
    sums = np.zeros(nf * 3)
    mw = np.zeros(max(ntrace, 1) * nf * 3)
    tr, bufs = (make_trace(ntrace, params.steps) if ntrace else (None, None))
    rc = L.orc_mag_walk(C.byref(pore), f, nf, C.byref(params), nthreads,
                        sums.ctypes.data_as(C.POINTER(C.c_double)),
                        mw.ctypes.data_as(C.POINTER(C.c_double)) if ntrace else None,
                        C.byref(tr) if tr is not None else None)
    if rc != 0:
        raise ValueError("orc_mag_walk failed: %d" % rc)
    return _mag_out(sums, mw, bufs, nf, ntrace, params.steps)


def ref_mag(variant, pore, fields, params, ntrace=0):
    """The reference's updateWalkersMag compiled here; None if unavailable."""
    R = reflib()
    if R is None:
        return None
    fn = getattr(R, "ref_mag_" + variant)
    nf = len(fields)
    f = _arr(fields, Field)
    sums = np.zeros(nf * 3)
    mw = np.zeros(max(ntrace, 1) * nf * 3)
    tr, bufs = (make_trace(ntrace, params.steps) if ntrace else (None, None))
    rc = fn(C.byref(pore), f, nf, C.byref(params), sums.ctypes.data_as(C.POINTER(C.c_double)),
            mw.ctypes.data_as(C.POINTER(C.c_double)) if ntrace else None,
            C.byref(tr) if tr is not None else None)
    if rc != 0:
        raise ValueError("ref_mag_%s failed: %d" % (variant, rc))
    return _mag_out(sums, mw, bufs, nf, ntrace, params.steps)


def mag_along(fields, params, pos) -> np.ndarray:
    """Final M [nf,3] of one walker along the trajectory pos[steps,3] (FP64)."""
    nf = len(fields)
    f = _arr(fields, Field)
    p = np.ascontiguousarray(pos, dtype=np.float64)
    out = np.zeros(nf * 3)
    lib().orc_mag_along(f, nf, C.byref(params), p.ctypes.data_as(C.POINTER(C.c_double)),
                        out.ctypes.data_as(C.POINTER(C.c_double)))
    return out.reshape(nf, 3)


def bfield(field, gamma, r, t) -> np.ndarray:
    out = (C.c_double * 3)()
    lib().orc_bfield(C.byref(field), C.c_double(gamma), (C.c_double * 3)(*r), C.c_double(t), out)
    return np.array(list(out))


def volume_fraction(lat, bases, points, seed, mode=REF64, nthreads=1) -> int:
    """Count of the calcf points inside a basis of region > 0."""
    b = _arr(bases, Basis)
    n = C.c_int64()
    rc = lib().orc_volume_fraction(C.byref(lat), b, len(bases), C.c_int64(points),
                                   C.c_uint64(seed), mode, nthreads, C.byref(n))
    if rc != 0:
        raise ValueError("orc_volume_fraction failed")
    return n.value


def wc(pore, rng_state, start, grad, timestep, gamma=267500.0):
    """kernelWC restated (FP64).  Returns (phase[n], sum_cos, sum_sin)."""
    st = np.ascontiguousarray(rng_state, np.uint32)
    p0 = np.ascontiguousarray(start, np.float64)
    g = np.ascontiguousarray(grad, np.float64)
    n, steps = len(st), len(g)
    ph = np.zeros(n)
    sc, ss = C.c_double(), C.c_double()
    rc = lib().orc_wc(C.byref(pore), C.c_int64(n), steps, C.c_double(timestep),
                      C.c_double(gamma), st.ctypes.data_as(C.POINTER(C.c_uint32)),
                      p0.ctypes.data_as(C.POINTER(C.c_double)),
                      g.ctypes.data_as(C.POINTER(C.c_double)),
                      ph.ctypes.data_as(C.POINTER(C.c_double)), C.byref(sc), C.byref(ss))
    if rc != 0:
        raise ValueError("orc_wc failed")
    return ph, sc.value, ss.value
