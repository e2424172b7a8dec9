"""Seeded synthetic workloads with the shapes of the benchmark configurations.

Units are the reference's (mm, ms, T/mm).  No dataset is read: every input is
drawn from a seeded generator.

* free_box()          -- free diffusion in an empty periodic 50 um box, 65,536
                         walkers, dt 5 us, 6,000 steps, PGSE delta 5 / Delta
                         20 ms, 16 G values 0-300 mT/m along x.
* one_cylinder()      -- one impermeable cylinder r 5 um in a 12 um cell,
                         1,048,576 walkers, dt 2 us, T2 80/60 ms; PGSE delta
                         10 / Delta 40 ms (25,000 steps), 32 G 0-200 mT/m, and
                         cosine OGSE at 50/100/200 Hz (delta 20, Delta 40 ms).
* gamma_pack()        -- 400 cylinders, gamma radii (k 5, mean 2.5 um) at area
                         fraction 0.6, permeable kappa 0.02 um/ms, D 1.7/2.0,
                         T2 80/60, dt 1 us, 64 sequences (PGSE, cosine and
                         square-wave OGSE, G <= 300 mT/m, directions uniform on
                         the sphere).
* batch_256()         -- 256 substrates from a seed: single cylinder (r 1-8 um),
                         single sphere (r 2-10 um) or hexagonal pack (f 0.4-0.7,
                         kappa 0-0.05 um/ms); walkers log-uniform 1e4-1e6;
                         8-64 sequences (PGSE, cosine and square-wave OGSE).
"""
from __future__ import annotations

import math

import numpy as np

from .acquisition import CosGFunc, Cylinder_XY, Lattice, RectGrad, Sphere, SWOGSEFunc
from .batch import Job
from .substrate import hex_cell, rps_gamma_pack

UM = 1e-3      # mm per um
D1 = 1e-6      # mm^2/ms per um^2/ms
MTM = 1e-6     # T/mm per mT/m
KAPPA = 1e-3   # mm/ms per um/ms


def free_box():
    s = 50 * UM
    lat = Lattice(s, s, s, 0.0, 0.0, 2.0 * D1, 0)
    seqs = [RectGrad(g * MTM, 5.0, 15.0) for g in np.linspace(0, 300, 16)]
    return dict(lattice=lat, basis=[], seqs=seqs, num_walkers=65536, steps=6000,
                timestep=0.005, seed=1234)


def one_cylinder():
    c, r = 12 * UM, 5 * UM
    lat = Lattice(c, c, c, 60.0, 0.0, 2.0 * D1, 1)
    cyl = [Cylinder_XY(c / 2, c / 2, r, 80.0, 0.0, 2.0 * D1, 1, 0.0)]
    pgse = [RectGrad(g * MTM, 10.0, 30.0) for g in np.linspace(0, 200, 32)]
    ogse = [CosGFunc(100 * MTM, 20.0, 20.0, n) for n in (1, 2, 4)]
    return dict(lattice=lat, basis=cyl, acquisitions=[(pgse, 25000), (ogse, 30000)],
                num_walkers=1 << 20, timestep=0.002, seed=1234)


def random_directions(n, rng):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def gamma_pack(seed=7, n_cyl=400, walkers=1 << 22):
    lat, cyl, f = rps_gamma_pack(seed, n_cyl, 5.0, 2.5 * UM, 0.6, D_in=1.7 * D1, T2_in=80.0,
                                 D_ex=2.0 * D1, T2_ex=60.0, permeability=0.02 * KAPPA)
    rng = np.random.default_rng(seed)
    # four waveforms, sixteen (G, direction) pairs each
    waves = [("pgse", 10.0, 30.0, 0), ("cos", 20.0, 5.0, 2), ("cos", 20.0, 5.0, 4),
             ("sw", 20.0, 5.0, 2)]
    seqs = []
    for kind, d, sp, n in waves:
        for g, u in zip(rng.uniform(0, 300, 16), random_directions(16, rng)):
            if kind == "pgse":
                q = RectGrad(g * MTM, d, sp)
                q.ghat = tuple(u)
            elif kind == "cos":
                q = CosGFunc(g * MTM, d, sp, n, tuple(u))
            else:
                q = SWOGSEFunc(g * MTM, d, sp, n, tuple(u))
            seqs.append(q)
    te = max(2 * d + sp for _, d, sp, _ in waves)
    return dict(lattice=lat, basis=cyl, seqs=seqs, num_walkers=walkers,
                steps=int(round(te / 0.001)), timestep=0.001, seed=seed, fraction=f)


def batch_256(seed=2026, n_sub=256, timestep=0.005, walker_scale=1.0, max_steps=None):
    """Jobs of the uneven 256-substrate batch."""
    rng = np.random.default_rng(seed)
    menu = [("pgse", 5.0, 15.0, 0), ("pgse", 10.0, 20.0, 0), ("cos", 20.0, 5.0, 1),
            ("cos", 20.0, 5.0, 2), ("cos", 20.0, 5.0, 4), ("sw", 20.0, 5.0, 2)]
    jobs = []
    for s in range(n_sub):
        kind = int(rng.integers(3))
        nw = int(round(10 ** rng.uniform(4, 6) * walker_scale))
        nseq = int(rng.integers(8, 65))
        picks = rng.integers(len(menu), size=nseq)
        G = rng.uniform(0, 300, size=nseq)
        seqs = []
        for k, g in zip(picks, G):
            w, d, sp, n = menu[int(k)]
            if w == "pgse":
                seqs.append(RectGrad(g * MTM, d, sp))
            elif w == "cos":
                seqs.append(CosGFunc(g * MTM, d, sp, n))
            else:
                seqs.append(SWOGSEFunc(g * MTM, d, sp, n))
        te = max(2 * menu[int(k)][1] + menu[int(k)][2] for k in picks)
        steps = int(round(te / timestep))
        if max_steps:
            steps = min(steps, max_steps)
        if kind == 0:
            r = rng.uniform(1, 8) * UM
            job = Job([Cylinder_XY(0.0, 0.0, r, 0.0, 0.0, 2.0 * D1, 1, 0.0)], seqs, nw, steps,
                      timestep, seed * 1000 + s)
        elif kind == 1:
            r = rng.uniform(2, 10) * UM
            job = Job([Sphere(0.0, 0.0, 0.0, r, 0.0, 0.0, 2.0 * D1, 1, 0.0)], seqs, nw, steps,
                      timestep, seed * 1000 + s)
        else:
            f = rng.uniform(0.4, 0.7)
            kappa = rng.uniform(0.0, 0.05) * KAPPA
            r = rng.uniform(1.5, 4.0) * UM
            lat, cyl = hex_cell(r, f, D_in=1.7 * D1, T2_in=80.0, D_ex=2.0 * D1, T2_ex=60.0,
                                permeability=kappa)
            job = Job(cyl, seqs, nw, steps, timestep, seed * 1000 + s, lattice=lat,
                      relaxation=True, permeable=kappa > 0)
        jobs.append(job)
    return jobs


def _plan(dev, lattice, basis, seqs, n, steps, timestep, seed, flags):
    import ctypes as C

    from . import _native as N
    from .acquisition import _params
    L = N.lib()
    p = _params(n, steps, seed, timestep, flags)
    b = N.array_of(N.Basis, [x.record() for x in basis])
    s = N.array_of(N.SequenceRec, [q.record() for q in seqs])
    h = C.c_void_p()
    N.check(L.axx_plan_lattice(dev.h, C.byref(lattice.record()), b, len(basis), s, len(seqs),
                               C.byref(p), C.byref(h)), dev.h)
    return h


def measure(name: str, steps: int = 0, walkers: int = 0, reps: int = 3, device=None) -> dict:
    """Walker-steps/s of one workload's walks with its tables resident on the
    GPU (CUDA events on the library stream, best of `reps` after one warm-up).
    `steps` / `walkers` > 0 shorten the walk / change the walker count."""
    import ctypes as C

    from . import _native as N
    from .acquisition import default_device, run_flags
    dev = device or default_device()
    L = N.lib()
    if name == "free_box":
        w = free_box()
        acqs = [(w["seqs"], w["steps"])]
        flags = run_flags()
    elif name == "one_cylinder":
        w = one_cylinder()
        acqs = w["acquisitions"]
        flags = run_flags(relaxation=True)
    elif name == "gamma_pack":
        w = gamma_pack()
        acqs = [(w["seqs"], w["steps"])]
        flags = run_flags(relaxation=True, permeable=True)
    else:
        raise ValueError("unknown workload " + name)
    n = walkers or w["num_walkers"]
    acqs = [(q, min(st, steps) if steps else st) for q, st in acqs]
    plans = [(_plan(dev, w["lattice"], w["basis"], q, n, st, w["timestep"], w["seed"], flags),
              len(q), st) for q, st in acqs]
    ws = sum(n * (st - 1) for _, _, st in plans)

    def launch():
        for h, _, _ in plans:
            N.check(L.axx_plan_launch(h), dev.h)

    launch()
    N.check(L.axx_sync(dev.h), dev.h)
    best = None
    for _ in range(reps):
        N.check(L.axx_event_record(dev.h, 0), dev.h)
        launch()
        N.check(L.axx_event_record(dev.h, 1), dev.h)
        ms = C.c_float()
        N.check(L.axx_event_elapsed(dev.h, 0, 1, C.byref(ms)), dev.h)
        best = ms.value if best is None else min(best, ms.value)
    out = {"workload": name, "walkers": n, "steps": [st for _, _, st in plans],
           "sequences": [m for _, m, _ in plans], "walker_steps": ws, "ms": best,
           "walker_steps_per_s": ws / (best * 1e-3),
           "signals_per_s": sum(m for _, m, _ in plans) / (best * 1e-3)}
    hits = caps = 0
    sig = []
    for h, m, _ in plans:
        mx, my = (C.c_double * m)(), (C.c_double * m)()
        st = N.Stats(None, None, None, 0, 0, 0)
        rc = L.axx_plan_read(h, mx, my, C.byref(st))
        if rc != N.AXX_ERR_REFLECTION_CAP:
            N.check(rc, dev.h)
        hits += st.boundary_hits
        caps += st.reflection_cap_hits
        sig += [math.hypot(mx[i], my[i]) / n for i in range(m)]
        L.axx_plan_destroy(h)
    out.update(boundary_hits_per_move=hits / ws, reflection_cap_hits=caps,
               signal_min=min(sig), signal_max=max(sig))
    if name == "free_box" and not steps:
        D = w["lattice"].D
        ref = [math.exp(-q.getB() * D) for q in acqs[0][0]]
        out["max_abs_vs_exp_bD"] = max(abs(a - b) for a, b in zip(sig, ref))
        out["standard_error_scale"] = 1.0 / math.sqrt(2.0 * n)
    if "fraction" in w:
        out["fraction"] = w["fraction"]
    return out


def main(argv=None):
    import argparse
    import json
    ap = argparse.ArgumentParser(description="time one seeded workload on the GPU")
    ap.add_argument("workload", choices=["free_box", "one_cylinder", "gamma_pack", "mag_lowfield",
                                         "wc_sphere", "mesh_sphere", "batch_256"])
    ap.add_argument("--steps", type=int, default=0, help="cut every walk to this many steps")
    ap.add_argument("--walkers", type=int, default=0)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--walker-scale", type=float, default=1.0,
                    help="batch_256: scale of every job's walker count")
    a = ap.parse_args(argv)
    if a.workload == "mag_lowfield":
        print(json.dumps(measure_mag(a.walkers, a.steps, a.reps)))
    elif a.workload == "wc_sphere":
        print(json.dumps(measure_wc(a.walkers or 32768, a.steps or 22000, a.reps)))
    elif a.workload == "mesh_sphere":
        print(json.dumps(measure_mesh(a.walkers or (1 << 20), a.steps or 6001, a.reps)))
    elif a.workload == "batch_256":
        print(json.dumps(measure_batch(a.walker_scale, a.steps or None, a.reps)))
    else:
        print(json.dumps(measure(a.workload, a.steps, a.walkers, a.reps)))



def mag_lowfield(n_fields=16, walkers=57344, gd=1.0, gs=1.0):
    """The low-field helium-3 cell of the reference's magLF example, in its
    units: cylinder radius 24.2, D 20, dt 0.001, GAMMA -203789, B0 6e-4,
    QSC_GRE gradient-echo fields with G = i * 6e-6 / n_fields, duration and
    spacing gd, gs; one walk, n_fields field functors."""
    from .acquisition import Cylinder_XY
    from .magnetization import QSC_GRE
    pore = Cylinder_XY(0.0, 0.0, 24.2, 0.0, 0.0, 20.0, 0, 0.0)
    fields = [QSC_GRE(6e-4, i * 6e-6 / n_fields, gd, gs) for i in range(n_fields)]
    te = 2.0 * gd + gs
    return dict(pore=pore, fields=fields, num_walkers=walkers, steps=int(te / 0.001),
                timestep=0.001, gamma=-203789.0, seed=1234)


def measure_mag(walkers: int = 0, steps: int = 0, reps: int = 3, device=None) -> dict:
    """Walker-steps/s of the magnetisation walk (axx_run_mag, host records in,
    host sums out, best of reps after one warm-up)."""
    import time

    from .magnetization import run_mag
    w = mag_lowfield()
    n = walkers or w["num_walkers"]
    st = steps or w["steps"]
    kw = dict(gamma=w["gamma"], device=device)
    run_mag(w["pore"], w["fields"], n, st, w["timestep"], w["seed"], **kw)
    best, r = None, None
    for _ in range(reps):
        t0 = time.perf_counter()
        r = run_mag(w["pore"], w["fields"], n, st, w["timestep"], w["seed"], **kw)
        dtw = time.perf_counter() - t0
        best = dtw if best is None else min(best, dtw)
    ws = n * (st - 1)
    out = {"workload": "mag_lowfield", "walkers": n, "steps": st, "fields": len(w["fields"]),
           "seconds": best, "walker_steps_per_s": ws / best,
           "field_updates_per_s": n * st * len(w["fields"]) / best,
           "signal": [float(x) for x in r.signal]}
    return out



def measure_wc(walkers: int = 32768, steps: int = 22000, reps: int = 3, device=None) -> dict:
    """The WCDMC walker (axx_run_wc) against the main single-pore walker
    (axx_run_single, specular) on WCcompare's sphere: radius 2.5 um, D
    2.5 um^2/ms, dt 1 us, a cosine OGSE gradient (delta 10, spacing 2 ms)."""
    import time

    from .acquisition import CosGFunc, Sphere, run_single, run_wc, wc_start
    pore = Sphere(0.0, 0.0, 0.0, 2.5 * UM, 0.0, 0.0, 2.5 * D1, 1, 0.0)
    seq = CosGFunc(50 * MTM, 10.0, 2.0, 5)
    dt = 0.001
    grad = np.array([tuple(seq(j * dt)) for j in range(steps)], dtype=np.float64)
    state, start = wc_start(pore, walkers, 7)
    run_wc(pore, state, start, grad, dt, device=device)
    t_wc = min(_timed(lambda: run_wc(pore, state, start, grad, dt, device=device))
               for _ in range(reps))
    run_single(pore, [seq], walkers, steps, dt, 7, device=device)
    t_sp = min(_timed(lambda: run_single(pore, [seq], walkers, steps, dt, 7, device=device))
               for _ in range(reps))
    return {"workload": "wc_sphere", "walkers": walkers, "steps": steps,
            "wc_walker_steps_per_s": walkers * steps / t_wc, "wc_seconds": t_wc,
            "specular_walker_steps_per_s": walkers * (steps - 1) / t_sp, "specular_seconds": t_sp}


def measure_mesh(walkers: int = 1 << 20, steps: int = 6001, reps: int = 3, device=None) -> dict:
    """A 5 um sphere as a 5,120-triangle icosphere mesh (axx_run_mesh) against
    the analytic sphere pore (axx_run_single): D 2 um^2/ms, dt 2 us, PGSE 16
    G values (delta 2, Delta 10 ms)."""
    from .acquisition import RectGrad, Sphere, run_single
    from .mesh import icosphere, run_mesh
    mesh = icosphere(5 * UM, 4, 2 * D1)
    seqs = [RectGrad(g * MTM, 2.0, 8.0) for g in np.linspace(0, 300, 16)]
    run_mesh(mesh, seqs, walkers, steps, 0.002, 7, device=device)
    t_m = min(_timed(lambda: run_mesh(mesh, seqs, walkers, steps, 0.002, 7, device=device))
              for _ in range(reps))
    r = run_mesh(mesh, seqs, walkers, steps, 0.002, 7, device=device)
    pore = Sphere(0.0, 0.0, 0.0, 5 * UM, 0.0, 0.0, 2 * D1, 1, 0.0)
    run_single(pore, seqs, walkers, steps, 0.002, 7, device=device)
    t_s = min(_timed(lambda: run_single(pore, seqs, walkers, steps, 0.002, 7, device=device))
              for _ in range(reps))
    return {"workload": "mesh_sphere", "triangles": len(mesh.triangles), "walkers": walkers,
            "steps": steps, "mesh_walker_steps_per_s": walkers * (steps - 1) / t_m,
            "mesh_seconds": t_m, "escaped": r.escaped,
            "hits_per_move": r.hits / r.walker_steps,
            "sphere_walker_steps_per_s": walkers * (steps - 1) / t_s}


def measure_batch(walker_scale: float = 1.0, max_steps: int = None, reps: int = 3,
                  device=None) -> dict:
    """The uneven 256-substrate batch as one persistent launch replayed from a
    CUDA graph (the autotuned tile): walker-steps/s and signals/s."""
    from .acquisition import default_device
    from .batch import Batch
    dev = device or default_device()
    jobs = batch_256(walker_scale=walker_scale, max_steps=max_steps)
    b = Batch(jobs, device=dev)
    b.launch()
    b.read()
    t = min(_timed(lambda: (b.launch(), b.read())) for _ in range(reps))
    info = b.info()
    b.close()
    ws = sum(j.num_walkers * (j.steps - 1) for j in jobs)
    return {"workload": "batch_256", "jobs": len(jobs), "walker_scale": walker_scale,
            "max_steps": max_steps, "walker_steps": ws, "seconds": t,
            "walker_steps_per_s": ws / t, "signals_per_s": sum(len(j.seqs) for j in jobs) / t,
            "info": {k: v for k, v in info.items() if isinstance(v, (int, float, str))}}


def _timed(fn):
    import time
    t0 = time.perf_counter()
    fn()
    return time.perf_counter() - t0


if __name__ == "__main__":
    main()
