"""Generates tests/golden/ref_walks.npz from the reference's own walker.

Runs the reference's updateWalkersLatticePhase / updateWalkersPhase compiled
for the host (oracle/_ref/libaxxref.so, built from the reference source tree
by oracle/Makefile) on small seeded cases and stores the signal sums and the
traces of the first walkers.  The fixtures pin the CPU oracle where the
reference tree is absent.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402
import cases  # noqa: E402

NTRACE = 4       # walkers whose traces are stored
TRACE_MOVES = 400  # first moves of each stored trace


def golden_cases():
    """(name, variant, lattice|None, bases, seqs, params)"""
    out = []
    seqs = [s for s in cases.seq_mix() if s.kind != 4]
    lat, cyl = cases.one_cylinder()
    out.append(("cyl_imp", "spec_imp", lat, cyl, seqs, cases.params(96, 1500, 11)))
    out.append(("cyl_imp_t2", "spec_imp_t2", lat, cyl, seqs, cases.params(96, 1500, 12, flags=1)))
    latp, cylp = cases.one_cylinder(D_in=1.7e-6, kappa=5e-5)
    out.append(("cyl_perm_t2", "spec_perm_t2", latp, cylp, seqs,
                cases.params(96, 1500, 13, flags=3)))
    out.append(("cyl_rej_t2", "rej_t2", lat, cyl, seqs, cases.params(96, 1500, 14, flags=5)))
    lath, hexc = cases.hex_cylinders()
    out.append(("hex_imp_t2", "spec_imp_t2", lath, hexc, seqs, cases.params(96, 1500, 15, flags=1)))
    lats, sph = cases.sphere_lattice()
    out.append(("sph_imp_t2", "spec_imp_t2", lats, sph, seqs, cases.params(96, 1200, 16, flags=1)))
    out.append(("free_box", "spec_imp", cases.lattice_box(), [], seqs,
                cases.params(96, 1500, 1234, dt=0.005)))
    b0 = O.Basis(1, 1, 0.0, 0.0, 0.0, 4 * cases.UM, cases.D2, 0, 0, 0, 1e-14)
    out.append(("single_sph", "spec_imp", None, [b0], seqs, cases.params(96, 1500, 17)))
    b1 = O.Basis(0, 1, 0.001, -0.002, 0.0, 4 * cases.UM, cases.D2, 0, 0, 0, 1e-14)
    out.append(("single_cyl", "spec_imp", None, [b1], seqs, cases.params(96, 1500, 18)))
    # Plane bases (plane.cuh): parallel plates as in the planePhase example
    latq, plates = cases.parallel_plates()
    out.append(("plates_imp_t2", "spec_imp_t2", latq, plates, seqs,
                cases.params(96, 1500, 21, flags=1)))
    out.append(("plates_perm", "spec_perm", latq, plates, seqs, cases.params(96, 1500, 22, flags=2)))
    # LATTICE_PICKING moves (kernelPhase.cuh:31-35)
    out.append(("single_cyl_pick", "pick_spec", None, [b1], seqs,
                cases.params(96, 1500, 19, flags=32)))
    out.append(("single_sph_pick", "pick_spec", None, [b0], seqs,
                cases.params(96, 1500, 20, flags=32)))
    return out


def mag_golden_cases():
    """(name, variant, pore, fields, params) of the magnetisation walker."""
    MP = O.mag_params
    fa, fm = cases.mag_fields(), cases.mag_multistep_fields()
    cyl, sph = cases.mag_pore(False), cases.mag_pore(True)
    return [
        ("mag_rot_cyl", "mag_rot_spec", cyl, fa, MP(48, 800, 21, 0.002)),
        ("mag_rot_sph", "mag_rot_spec", sph, fa, MP(48, 800, 22, 0.002)),
        ("mag_rej_cyl", "mag_rot_rej", cyl, fa, MP(48, 800, 23, 0.002, reject=True)),
        ("mag_rk4_cyl", "mag_rk4_spec", cyl, fa, MP(48, 800, 24, 0.002, integrator=O.RK4)),
        ("mag_ms_cyl", "mag_ms_spec", cyl, fm, MP(48, 800, 25, 0.002, integrator=O.MULTISTEP,
                                                  m0=(0.0, 0.0, 1.0))),
        ("mag_ms_sph", "mag_ms_spec", sph, fm, MP(48, 800, 26, 0.002, integrator=O.MULTISTEP)),
    ]


def main():
    if O.reflib() is None:
        O.build(ref=True)
    if O.reflib() is None:
        raise SystemExit("the reference walker (oracle/_ref) could not be built")
    data = {}
    for name, var, lat, bases, seqs, p in golden_cases():
        sums, tr = O.ref_walk(var, lat, bases, seqs, p, nthreads=1, ntrace=NTRACE)
        data[name + "/sums"] = sums
        for k, v in tr.items():
            data[name + "/" + k] = v if k == "init_pos" else v[:, :TRACE_MOVES]
    np.savez_compressed(os.path.join(HERE, "ref_walks.npz"), **data)
    print("wrote", len(data), "arrays")
    mag = {}
    for name, var, pore, fields, p in mag_golden_cases():
        sums, mw, tr = O.ref_mag(var, pore, fields, p, ntrace=NTRACE)
        mag[name + "/sums"] = sums
        mag[name + "/m_walk"] = mw
        if tr is not None and "rej" not in var:  # boundaryNormal is hooked in specular builds
            for k, v in tr.items():
                mag[name + "/" + k] = v if k == "init_pos" else v[:, :TRACE_MOVES]
    np.savez_compressed(os.path.join(HERE, "ref_mag.npz"), **mag)
    print("wrote", len(mag), "arrays")


if __name__ == "__main__":
    main()
