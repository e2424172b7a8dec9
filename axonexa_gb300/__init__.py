"""GB300-native random-walker phase path of the axonexa diffusion-MRI simulator.

The compute runs in hand-written sm_103a CUDA kernels behind the C ABI of
include/axx.h (libaxx.so, built in-tree by ``axonexa_gb300.build``).  This
package is the host-side mirror of the reference's acquisition API.
"""
from .acquisition import (GAMMA, PI, ApodCosGFunc, CosGFunc, Cylinder, Cylinder_XY, Device,
                          Lattice, Plane, RectGrad, RunResult, SinGFunc, Sphere, SWOGSEFunc, Vector3,
                          default_device, linear_regression, phaseAcquisition,
                          phaseAcquisitionStream, philox_words, run_lattice, run_single,
                          trace_lattice, trace_single)
from .substrate import gamma_quantile_radii, hex_cell, pack_radii, rps_gamma_pack, volume_fraction
from .batch import Batch, Job, autotune, run_batch
from .magnetization import (COS_GRE, QSC_COS_GRE, QSC_GRE, QSC_GRE_TRAP, QSC_PGSE, RECT_GRE,
                            SIN_GRE, UCN_lowfield, magAcquisition, magAcquisitionStream,
                            run_mag, trace_mag)
from .acquisition import run_wc, wc_start
from .mesh import Mesh, Triangle, cube, icosphere, prism, run_mesh, trace_mesh

__all__ = [n for n in dir() if not n.startswith("_")]
