"""ctypes binding of libaxx.so (the C ABI of include/axx.h).

The library is built in-tree by ``axonexa_gb300.build``; importing this module
never falls back to anything else: a missing or unloadable library raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libaxx.so")

AXX_OK = 0
AXX_ERR_REFLECTION_CAP = 3
STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "reflection cap hit",
          4: "timeout", 5: "no CUDA device", 6: "out of device memory", 7: "aborted",
          8: "unsupported", 9: "non-finite value"}

PRIM_CYLINDER_Z, PRIM_SPHERE, PRIM_PLANE, PRIM_CYLINDER = 0, 1, 2, 3
SEQ_PGSE, SEQ_COS, SEQ_SIN, SEQ_APODCOS, SEQ_SQUARE = 0, 1, 2, 3, 4
FLAG_RELAXATION, FLAG_PERMEABLE, FLAG_SIMPLE_REJECTION = 1, 2, 4
FLAG_KEEP_INIT_QUIRK, FLAG_FIX_INIT_QUIRK = 8, 16
FLAG_LATTICE_PICKING = 32
FLAG_COMPARTMENTS = 64
INIT_UNIFORM, INIT_IN_REGION, INIT_IN_BASIS = 0, 1, 2


class AxxError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__("%s (%d): %s" % (STATUS.get(status, "?"), status, msg))
        self.status = status


class ReflectionCapError(AxxError):
    """Some moves needed more than 1024 boundary hits; results were still written."""


class Basis(C.Structure):
    _fields_ = [("type", C.c_int32), ("region", C.c_int32), ("cx", C.c_double),
                ("cy", C.c_double), ("cz", C.c_double), ("radius", C.c_double),
                ("D", C.c_double), ("T2", C.c_double), ("T1", C.c_double),
                ("permeability", C.c_double), ("eps", C.c_double),
                ("nx", C.c_double), ("ny", C.c_double), ("nz", C.c_double)]


class LatticeRec(C.Structure):
    _fields_ = [("a", C.c_double), ("b", C.c_double), ("c", C.c_double),
                ("T2", C.c_double), ("T1", C.c_double), ("D", C.c_double)]


class SequenceRec(C.Structure):
    _fields_ = [("kind", C.c_int32), ("num_periods", C.c_int32), ("G", C.c_double),
                ("duration", C.c_double), ("spacing", C.c_double), ("gx", C.c_double),
                ("gy", C.c_double), ("gz", C.c_double)]


class RunParams(C.Structure):
    _fields_ = [("num_walkers", C.c_int64), ("steps", C.c_int32), ("init_mode", C.c_int32),
                ("init_arg", C.c_int32), ("flags", C.c_uint32), ("seed", C.c_uint64),
                ("timestep", C.c_double), ("gamma", C.c_double), ("walker_offset", C.c_int64)]


class Stats(C.Structure):
    _fields_ = [("sxx", C.POINTER(C.c_double)), ("syy", C.POINTER(C.c_double)),
                ("sxy", C.POINTER(C.c_double)), ("reflection_cap_hits", C.c_int64),
                ("walker_steps", C.c_int64), ("boundary_hits", C.c_int64),
                ("mx_in", C.POINTER(C.c_double)), ("my_in", C.POINTER(C.c_double)),
                ("walkers_in", C.c_int64)]


class PackSpec(C.Structure):
    _fields_ = [("shape", C.c_double), ("mean", C.c_double), ("rmin", C.c_double),
                ("rmax", C.c_double), ("fraction", C.c_double), ("D", C.c_double),
                ("T2", C.c_double), ("permeability", C.c_double)]


class MeshRec(C.Structure):
    _fields_ = [("vertices", C.POINTER(C.c_double)), ("nvert", C.c_int32),
                ("triangles", C.POINTER(C.c_int32)), ("ntri", C.c_int32), ("D", C.c_double)]


class Job(C.Structure):
    _fields_ = [("mode", C.c_int32), ("lattice", LatticeRec), ("basis", C.POINTER(Basis)),
                ("nbasis", C.c_int32), ("seqs", C.POINTER(SequenceRec)), ("nseq", C.c_int32),
                ("params", RunParams)]


class BatchOptions(C.Structure):
    _fields_ = [("tile", C.c_int32), ("blocks_per_sm", C.c_int32), ("use_graph", C.c_int32)]


# exported symbols and their argument types
class Field(C.Structure):
    """axx_field"""
    _fields_ = [("kind", C.c_int32), ("num_periods", C.c_int32), ("B0", C.c_double),
                ("G", C.c_double), ("gx", C.c_double), ("gy", C.c_double), ("gz", C.c_double),
                ("duration", C.c_double), ("spacing", C.c_double), ("period", C.c_double),
                ("ramp", C.c_double), ("rf_duration", C.c_double), ("dtmin", C.c_double),
                ("dtmax", C.c_double), ("TE", C.c_double)]


class MagParams(C.Structure):
    """axx_mag_params"""
    _fields_ = [("num_walkers", C.c_int64), ("steps", C.c_int32), ("integrator", C.c_int32),
                ("flags", C.c_uint32), ("dorp_levels", C.c_uint32), ("seed", C.c_uint64),
                ("timestep", C.c_double), ("gamma", C.c_double), ("m0", C.c_double * 3),
                ("walker_offset", C.c_int64), ("dorp_tol", C.c_double)]


_SIGS = {
    "axx_abi_version": ([], C.c_int),
    "axx_status_string": ([C.c_int], C.c_char_p),
    "axx_create": ([C.POINTER(C.c_void_p), C.c_int], C.c_int),
    "axx_destroy": ([C.c_void_p], C.c_int),
    "axx_last_error": ([C.c_void_p], C.c_char_p),
    "axx_device_info": ([C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                         C.POINTER(C.c_size_t)], C.c_int),
    "axx_abort": ([C.c_void_p], C.c_int),
    "axx_run_lattice": ([C.c_void_p, C.POINTER(LatticeRec), C.POINTER(Basis), C.c_int,
                         C.POINTER(SequenceRec), C.c_int, C.POINTER(RunParams),
                         C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(Stats)], C.c_int),
    "axx_run_single": ([C.c_void_p, C.POINTER(Basis), C.POINTER(SequenceRec), C.c_int,
                        C.POINTER(RunParams), C.POINTER(C.c_double), C.POINTER(C.c_double),
                        C.POINTER(Stats)], C.c_int),
    "axx_run_lattice_noalloc": ([C.c_void_p, C.POINTER(LatticeRec), C.POINTER(Basis), C.c_int,
                                 C.POINTER(SequenceRec), C.c_int, C.POINTER(RunParams),
                                 C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(Stats)],
                                C.c_int),
    "axx_plan_lattice": ([C.c_void_p, C.POINTER(LatticeRec), C.POINTER(Basis), C.c_int,
                          C.POINTER(SequenceRec), C.c_int, C.POINTER(RunParams),
                          C.POINTER(C.c_void_p)], C.c_int),
    "axx_plan_single": ([C.c_void_p, C.POINTER(Basis), C.POINTER(SequenceRec), C.c_int,
                         C.POINTER(RunParams), C.POINTER(C.c_void_p)], C.c_int),
    "axx_plan_launch": ([C.c_void_p], C.c_int),
    "axx_plan_read": ([C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                       C.POINTER(Stats)], C.c_int),
    "axx_plan_info": ([C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                       C.POINTER(C.c_int64)], C.c_int),
    "axx_plan_candidates": ([C.c_void_p, C.POINTER(C.c_double)], C.c_int),
    "axx_plan_destroy": ([C.c_void_p], C.c_int),
    "axx_transfer_bytes": ([C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)], C.c_int),
    "axx_event_record": ([C.c_void_p, C.c_int], C.c_int),
    "axx_event_elapsed": ([C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_float)], C.c_int),
    "axx_sync": ([C.c_void_p], C.c_int),
    "axx_fp32_fma_peak": ([C.c_void_p, C.POINTER(C.c_double)], C.c_int),
    "axx_batch_create": ([C.c_void_p, C.POINTER(Job), C.c_int, C.POINTER(BatchOptions),
                          C.POINTER(C.c_void_p)], C.c_int),
    "axx_batch_launch": ([C.c_void_p], C.c_int),
    "axx_batch_read": ([C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                        C.POINTER(Stats)], C.c_int),
    "axx_batch_info": ([C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                        C.POINTER(C.c_int), C.POINTER(C.c_int64)], C.c_int),
    "axx_batch_destroy": ([C.c_void_p], C.c_int),
    "axx_run_batch": ([C.c_void_p, C.POINTER(Job), C.c_int, C.POINTER(BatchOptions),
                       C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(Stats)], C.c_int),
    "axx_autotune_batch": ([C.c_void_p, C.POINTER(Job), C.c_int, C.c_int,
                            C.POINTER(BatchOptions), C.POINTER(C.c_double)], C.c_int),
    "axx_mlp_create": ([C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_uint64,
                        C.POINTER(C.c_void_p)], C.c_int),
    "axx_mlp_destroy": ([C.c_void_p], C.c_int),
    "axx_mlp_num_params": ([C.c_void_p, C.POINTER(C.c_int64)], C.c_int),
    "axx_mlp_get_params": ([C.c_void_p, C.POINTER(C.c_float)], C.c_int),
    "axx_mlp_set_params": ([C.c_void_p, C.POINTER(C.c_float)], C.c_int),
    "axx_mlp_gradients": ([C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int,
                           C.POINTER(C.c_float), C.POINTER(C.c_float)], C.c_int),
    "axx_mlp_train": ([C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int, C.c_int,
                       C.c_int, C.c_float, C.c_uint64, C.POINTER(C.c_float)], C.c_int),
    "axx_mlp_predict": ([C.c_void_p, C.POINTER(C.c_float), C.c_int, C.POINTER(C.c_float)],
                        C.c_int),
    "axx_mlp_predict_device": ([C.c_void_p, C.c_void_p, C.c_int, C.c_void_p], C.c_int),
    "axx_mlp_flops_per_row": ([C.c_void_p, C.POINTER(C.c_double)], C.c_int),
    "axx_bvalue": ([C.POINTER(SequenceRec), C.c_double, C.POINTER(C.c_double)], C.c_int),
    "axx_gradient_eval": ([C.POINTER(SequenceRec), C.POINTER(C.c_double), C.c_int,
                           C.POINTER(C.c_double)], C.c_int),
    "axx_philox_words": ([C.c_void_p, C.c_uint64, C.c_uint64, C.c_int, C.POINTER(C.c_uint32)],
                         C.c_int),
    "axx_trace_lattice": ([C.c_void_p, C.POINTER(LatticeRec), C.POINTER(Basis), C.c_int,
                           C.POINTER(RunParams), C.c_int, C.POINTER(C.c_float),
                           C.POINTER(C.c_float), C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                           C.POINTER(C.c_int32)], C.c_int),
    "axx_trace_single": ([C.c_void_p, C.POINTER(Basis), C.POINTER(RunParams), C.c_int,
                          C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_int32),
                          C.POINTER(C.c_int32), C.POINTER(C.c_int32)], C.c_int),
    "axx_substrate_rps_gamma": ([C.c_uint64, C.c_int, C.c_double, C.c_double, C.c_double,
                                 C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                 C.c_int, C.POINTER(Basis), C.POINTER(C.c_int),
                                 C.POINTER(C.c_double), C.POINTER(C.c_double)], C.c_int),
    "axx_substrate_pack": ([C.c_uint64, C.c_int, C.POINTER(C.c_double), C.c_double, C.c_double,
                            C.c_double, C.c_double, C.c_int, C.POINTER(Basis),
                            C.POINTER(C.c_int), C.POINTER(C.c_double),
                            C.POINTER(C.c_double)], C.c_int),
    "axx_substrate_rps_gamma_gpu": ([C.c_void_p, C.c_uint64, C.c_int, C.c_int,
                                     C.POINTER(PackSpec), C.c_int, C.POINTER(Basis),
                                     C.POINTER(C.c_int), C.POINTER(C.c_double),
                                     C.POINTER(C.c_double)], C.c_int),
    "axx_volume_fraction": ([C.c_void_p, C.POINTER(LatticeRec), C.POINTER(Basis), C.c_int,
                             C.c_int64, C.c_uint64, C.POINTER(C.c_double),
                             C.POINTER(C.c_int64)], C.c_int),
    "axx_run_wc": ([C.c_void_p, C.POINTER(Basis), C.c_int64, C.c_int32, C.c_double, C.c_double,
                    C.POINTER(C.c_uint32), C.POINTER(C.c_double), C.POINTER(C.c_double),
                    C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)],
                   C.c_int),
    "axx_run_mag": ([C.c_void_p, C.POINTER(Basis), C.POINTER(Field), C.c_int,
                     C.POINTER(MagParams), C.POINTER(C.c_double), C.POINTER(C.c_double),
                     C.POINTER(C.c_double)], C.c_int),
    "axx_trace_mag": ([C.c_void_p, C.POINTER(Basis), C.POINTER(Field), C.c_int,
                       C.POINTER(MagParams), C.c_int, C.POINTER(C.c_float),
                       C.POINTER(C.c_float), C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                       C.POINTER(C.c_float)], C.c_int),
    "axx_run_mesh": ([C.c_void_p, C.POINTER(MeshRec), C.POINTER(SequenceRec), C.c_int,
                      C.POINTER(RunParams), C.POINTER(C.c_double), C.POINTER(C.c_double),
                      C.POINTER(Stats), C.POINTER(C.c_int64)], C.c_int),
    "axx_trace_mesh": ([C.c_void_p, C.POINTER(MeshRec), C.POINTER(RunParams), C.c_int,
                        C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_int32),
                        C.POINTER(C.c_int32), C.POINTER(C.c_int64)], C.c_int),
}

_lib = None


def lib():
    """The loaded libaxx.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libaxx.so is not built: run axonexa_gb300.build.build() "
                              "(python -c 'import __graft_entry__ as g; g.build()')")
        L = C.CDLL(LIB_PATH)
        for name, (args, res) in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def exported_symbols():
    return sorted(_SIGS)


def check(status: int, ctx=None) -> None:
    if status == AXX_OK:
        return
    msg = ""
    if ctx is not None:
        raw = lib().axx_last_error(ctx)
        msg = raw.decode() if raw else ""
    if status == AXX_ERR_REFLECTION_CAP:
        raise ReflectionCapError(status, msg)
    raise AxxError(status, msg)


def array_of(cls, items):
    items = list(items)
    a = (cls * max(len(items), 1))()
    for i, it in enumerate(items):
        a[i] = it
    return a
