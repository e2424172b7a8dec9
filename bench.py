"""Throughput of the GB300 walker on the 400-cylinder permeable gamma packing.

Headline workload (one bench step = the whole job): 400 cylinders per
periodic cell with gamma-distributed radii (shape 5, mean 2.5 um) packed to an
intra-axonal area fraction of 0.6 (435 bases with their periodic images);
permeable membranes, kappa = 0.02 um/ms; D_in = 1.7, D_ex = 2.0 um^2/ms;
T2 80/60 ms; 4,194,304 walkers uniform in the cell, FP32 with Kahan-compensated
phase and an FP64 signal reduction; dt = 1 us over TE = 50 ms (50,000 steps);
64 sequences (16 each of PGSE delta 10 / Delta 40 ms, cosine OGSE with 2 and
4 periods and square-wave OGSE with 2 periods over delta 20 ms), G uniform in
0-300 mT/m, gradient directions uniform on the sphere.  Inputs are seeded
synthetic substrates and sequences (packing seed 7); nothing is read from a
dataset.

Lines printed (rank 0):
  default arm       -- walker-steps/s of the headline job with the plan resident
                       on the GPU (value) and through the one-shot C-ABI call
                       with host records in and host sums out (e2e); roofline of
                       the walk kernel against the measured FP32 FMA peak; the
                       CPU oracle on a bounded walker sample of the same job
                       (cpu_baseline) and every signal of that sample against
                       the FP64 oracle of the same streams (fp64_check).
                       Sections: "restricted_cylinder" (one impermeable
                       cylinder, 1,048,576 walkers, 35 sequences), "free_box"
                       (free diffusion, 16 PGSE), "batch" (the uneven
                       256-substrate batch in one persistent graph launch),
                       "mag" (Bloch walk), "wc" (WCDMC walker), "mesh"
                       (triangle-mesh pore), "surrogate" (tcgen05 inference).
  --impl reference  -- the reference's walker loop on the host cores: the CPU
                       restatement of updateWalkersLatticePhase (oracle, FP64,
                       reference operation order) over all host threads, on a
                       walker sample of the headline job.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "walker-steps/s on 1 GB300; surrogate signals/s at |dS|<=2e-3 vs plain MC"
UNIT = "walker-steps/s"
WORKLOAD = "gamma_pack_400_cylinders_permeable_64seq"

# restricted-cylinder section (reference units: mm, ms, T)
CELL, RADIUS = 0.012, 0.005
D, T2_IN, T2_EX = 2.0e-6, 80.0, 60.0
DT2 = 0.002
N2 = 1 << 20
SEED2 = 1234
PGSE_STEPS, OGSE_STEPS = 25000, 30000

# DRAM bytes read + written per walker by the headline walk launch (ncu
# capture at 262,144 walkers, 2,000 steps: block partials and tables only,
# walker state never leaves registers), scaled by walkers
WALK_DRAM_BYTES_PER_WALKER = (158464.0 + 139520.0) / 262144
WALK_ISSUE_ACTIVE_NCU = 0.658


def headline_workload():
    from axonexa_gb300 import workloads as W
    return W.gamma_pack()


def restricted_records(A):
    import numpy as np
    lat = A.Lattice(CELL, CELL, CELL, T2_EX, 0.0, D, 1)
    cyl = [A.Cylinder_XY(CELL / 2, CELL / 2, RADIUS, T2_IN, 0.0, D, 1, 0.0)]
    pgse = [A.RectGrad(g * 1e-6, 10.0, 30.0) for g in np.linspace(0.0, 200.0, 32)]
    ogse = [A.CosGFunc(100e-6, 20.0, 20.0, n) for n in (1, 2, 4)]
    return lat, cyl, [(pgse, PGSE_STEPS), (ogse, OGSE_STEPS)]


class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thr = threading.Thread(target=self._read, daemon=True)
            self.thr.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for k, name in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower().startswith("active"):
                    reasons.add(name)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def flush_l2(buf):
    """Writes a 512 MiB buffer (L2 is 129 MB) between timed iterations."""
    if buf is not None:
        buf.zero_()


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if os.environ.get("AXX_BENCH_BACKEND", "gloo") == "nccl" else "gloo"
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def oracle_records(w):
    """The headline job's records for the CPU oracle."""
    from oracle import oracle as O
    lat = w["lattice"]
    L = O.Lattice(lat.a, lat.b, lat.c, lat.T2, lat.T1, lat.D)
    B = [O.Basis(0, c.region, c.centerX, c.centerY, 0.0, c.radius, c.D, c.T2, c.T1,
                 c.permeability, c.eps) for c in w["basis"]]
    Q = [O.Sequence(q.kind, q.num_periods, q.G, q.duration, q.spacing, q.ghat[0], q.ghat[1],
                    q.ghat[2]) for q in w["seqs"]]
    return L, B, Q


def cpu_sample(w, n_walkers: int, threads: int, steps: int = None):
    """The oracle's FP64 reference-order walk (updateWalkersLatticePhase
    restated, permeable, with relaxation) over the first `n_walkers` walkers
    of the headline job (their own Philox streams), full walks unless `steps`."""
    from oracle import oracle as O
    O.lib()
    L, B, Q = oracle_records(w)
    st = w["steps"] if steps is None else steps
    p = O.Params(n_walkers, st, 0, 0, 1 | 2, w["seed"], w["timestep"], 0.0, 0)
    t0 = time.perf_counter()
    sums, _, _ = O.walk(L, B, Q, p, O.REF64, nthreads=threads)
    dt = time.perf_counter() - t0
    ws = n_walkers * (st - 1)
    return ws / dt, dt, ws, sums


def fp64_check(A, dev, w, n_walkers: int, ref_sums) -> dict:
    """The GPU walk of the same first walkers (the same Philox streams)
    against the oracle's FP64 reference-order sums: |dS| per sequence and its
    ratio to the walk's standard error, over every sequence."""
    import numpy as np
    r = A.run_lattice(w["lattice"], w["basis"], w["seqs"], n_walkers, w["steps"],
                      w["timestep"], w["seed"], relaxation=True, permeable=True, device=dev)
    s_ref = np.hypot(ref_sums[:, 0], ref_sums[:, 1]) / n_walkers
    d = np.abs(r.signal - s_ref)
    return {"walkers": n_walkers, "sequences": len(w["seqs"]),
            "max_abs_dS": float(d.max()), "mean_abs_dS": float(d.mean()),
            "max_dS_over_se": float((d / np.maximum(r.stderr, 1e-12)).max()),
            "oracle": "FP64 reference-order restatement, the same streams"}


def time_launches(N, L, dev, launch, reps, flush=None):
    """CUDA-event milliseconds of `launch` on the library stream, one event
    pair per repetition, the L2 flushed between repetitions."""
    import ctypes as C

    import torch
    out = []
    for _ in range(reps):
        if flush is not None:
            flush_l2(flush)
            torch.cuda.synchronize()
        N.check(L.axx_event_record(dev.h, 0), dev.h)
        launch()
        N.check(L.axx_event_record(dev.h, 1), dev.h)
        ms = C.c_float()
        N.check(L.axx_event_elapsed(dev.h, 0, 1, C.byref(ms)), dev.h)
        out.append(ms.value)
    return out


def make_plan(A, N, L, dev, lat, basis, seqs, nw, steps, dt, seed, flags, offset=0):
    import ctypes as C
    p = A.acquisition._params(nw, steps, seed, dt, flags, offset=offset)
    h = C.c_void_p()
    N.check(L.axx_plan_lattice(dev.h, C.byref(lat.record()),
                               N.array_of(N.Basis, [c.record() for c in basis]), len(basis),
                               N.array_of(N.SequenceRec, [q.record() for q in seqs]),
                               len(seqs), C.byref(p), C.byref(h)), dev.h)
    return h


def plan_facts(N, L, dev, h, M):
    """Channels, candidates per move and boundary hits per move of the plan's
    last launch."""
    import ctypes as C
    ch = C.c_int()
    N.check(L.axx_plan_info(h, C.byref(ch), None, None, None), dev.h)
    cand = C.c_double()
    N.check(L.axx_plan_candidates(h, C.byref(cand)), dev.h)
    mx, my = (C.c_double * M)(), (C.c_double * M)()
    st = N.Stats(None, None, None, 0, 0, 0, None, None, 0)
    N.check(L.axx_plan_read(h, mx, my, C.byref(st)), dev.h)
    return ch.value, cand.value, st.boundary_hits / max(st.walker_steps, 1)


def ops_per_move(channels, cand, hits):
    """Algorithmic FP32 ops per move (one FMA = one op): 18 direction and move,
    6 periodic wrap, 7 per phase channel, 1 T2, 23 per candidate cylinder test,
    20 per boundary hit."""
    return 18 + 6 + 7 * channels + 1 + 23 * cand + 20 * hits


def transfer_bytes(N, L, dev):
    import ctypes as C
    a, b = C.c_int64(), C.c_int64()
    N.check(L.axx_transfer_bytes(dev.h, C.byref(a), C.byref(b)), dev.h)
    return a.value, b.value


def restricted_section(A, N, L, dev, reps=3):
    """The single impermeable cylinder (r 5 um, 12 um cell, 1,048,576 walkers,
    dt 2 us; PGSE 32 G over 25,000 steps + cosine OGSE 3 over 30,000): device
    resident plans timed with CUDA events, the one-shot C-ABI call timed on the
    host, and the roofline of its walk."""
    lat, cyl, acqs = restricted_records(A)
    flags = A.acquisition.run_flags(relaxation=True)
    plans = [(make_plan(A, N, L, dev, lat, cyl, seqs, N2, steps, DT2, SEED2, flags), len(seqs),
              steps) for seqs, steps in acqs]

    def launch():
        for h, _, _ in plans:
            N.check(L.axx_plan_launch(h), dev.h)

    launch()
    ms = min(time_launches(N, L, dev, launch, reps))
    ws = N2 * sum(s - 1 for _, s in acqs)
    facts = [plan_facts(N, L, dev, h, M) for h, M, _ in plans]
    ops = N2 * sum(ops_per_move(*f) * (s - 1) for f, (_, _, s) in zip(facts, plans))
    for h, _, _ in plans:
        L.axx_plan_destroy(h)
    t0 = time.perf_counter()
    for seqs, steps in acqs:
        A.run_lattice(lat, cyl, seqs, N2, steps, DT2, SEED2, relaxation=True, device=dev)
    e2e_s = time.perf_counter() - t0
    peak = fma_peak(N, L, dev)
    return {"workload": "restricted_cylinder_pgse32_ogse3", "walkers": N2,
            "moves": [PGSE_STEPS - 1, OGSE_STEPS - 1], "ms": ms,
            "walker_steps_per_s": ws / (ms * 1e-3), "e2e_walker_steps_per_s": ws / e2e_s,
            "roofline": {"bound": "simt", "achieved": ops / (ms * 1e-3) / 1e12,
                         "peak": peak / 1e12, "unit": "TFLOP/s",
                         "frac": ops / (ms * 1e-3) / peak,
                         "ops_per_move": [round(ops_per_move(*f), 2) for f in facts]}}


def free_box_section(A, dev, reps=3):
    """Free diffusion in the empty 50 um box: 65,536 walkers, 6,000 steps,
    16 PGSE G (one-shot calls, host timed), against exp(-bD)."""
    import numpy as np
    from axonexa_gb300 import workloads as W
    w = W.free_box()
    best = None
    for _ in range(reps):
        t0 = time.perf_counter()
        r = A.run_lattice(w["lattice"], w["basis"], w["seqs"], w["num_walkers"], w["steps"],
                          w["timestep"], w["seed"], device=dev)
        t = time.perf_counter() - t0
        best = t if best is None else min(best, t)
    b = np.array([q.getB() for q in w["seqs"]])
    ana = np.exp(-b * w["lattice"].D)
    return {"workload": "free_box_pgse16", "walkers": w["num_walkers"], "steps": w["steps"],
            "e2e_walker_steps_per_s": w["num_walkers"] * (w["steps"] - 1) / best,
            "max_abs_dS_vs_exp_bD": float(np.abs(r.signal - ana).max()),
            "max_se": float(r.stderr.max())}


def fma_peak(N, L, dev):
    import ctypes as C
    peak = C.c_double()
    N.check(L.axx_fp32_fma_peak(dev.h, C.byref(peak)), dev.h)
    return peak.value


def surrogate_section(A, N, L, dev, queries=1000000, reps=10, plain_subs=2):
    """Learned surrogate: the trained network of the 400-cylinder
    configuration (axonexa_gb300/data) against its held-out pairs' plain
    Monte Carlo truth (|dS|), tcgen05 inference of `queries` rows resident on
    the GPU (CUDA events on the library stream), the same through the host API
    (host rows in, host signals out), and the plain walk's signals/s on the
    surrogate's own data-generation jobs (400-cylinder gamma packings, 262,144
    walkers, 64 sequences each, dt 1 us, read at 55 ms)."""
    import numpy as np
    import torch

    from axonexa_gb300 import surrogate as S
    out = {}
    if os.path.exists(S.WEIGHTS):
        m, held, meta = S.load(device=dev)
        pred = m.predict(S.normalise(held["P"]))
        err = np.abs(pred - held["truth"])
        out.update({"weights": os.path.relpath(S.WEIGHTS, ROOT), "trained_on": meta,
                    "heldout_pairs": int(len(err)),
                    "heldout_truth_se_mean": float(np.mean(held["truth_se"])),
                    "heldout_abs_dS_mean": float(err.mean()),
                    "heldout_abs_dS_p95": float(np.quantile(err, 0.95)),
                    "heldout_abs_dS_max": float(err.max()),
                    "heldout_frac_within_2e-3": float(np.mean(err <= 2e-3))})
    else:
        m = S.MLP(seed=0, device=dev)
        out["weights"] = "untrained (no saved weights): throughput only"
    g = torch.Generator(device="cuda")
    g.manual_seed(SEED2)
    X = torch.rand(queries, 10, device="cuda", generator=g) * 2 - 1
    y = torch.empty(queries, device="cuda")
    torch.cuda.synchronize()
    for _ in range(3):
        m.predict_device(X.data_ptr(), queries, y.data_ptr())
    N.check(L.axx_sync(dev.h), dev.h)
    times = time_launches(N, L, dev, lambda: m.predict_device(X.data_ptr(), queries,
                                                             y.data_ptr()), reps)
    ms = float(np.median(times))
    flops = m.flops_per_row() * queries
    # end to end: queries in and outputs out through pinned host memory
    Xp = torch.empty((queries, 10), dtype=torch.float32, pin_memory=True)
    Xp.copy_(X)
    yp = torch.empty(queries, dtype=torch.float32, pin_memory=True)
    Xh, yh = Xp.numpy(), yp.numpy()
    m.predict(Xh[:4096])
    e2e = []
    for _ in range(5):
        t0 = time.perf_counter()
        m.predict(Xh, out=yh)
        e2e.append(time.perf_counter() - t0)
    e2e_s = float(np.median(e2e))
    assert np.array_equal(yh, y.cpu().numpy()), "host and device inference disagree"
    peaks = measured_peaks()
    pk = peaks.get("bf16_tflops")
    out.update({"queries": queries, "signals_per_s": queries / (ms * 1e-3), "ms": ms,
                "e2e_signals_per_s": queries / e2e_s, "h2d_bytes": int(Xh.nbytes),
                "d2h_bytes": int(4 * queries), "kernel_launches_per_call": 1,
                "e2e_path": "axx_mlp_predict from pinned host memory (median of 5 calls): "
                            "up to 4 chunks of whole kernel waves, each chunk's copy in "
                            "overlapping the previous chunk's kernel",
                "roofline": {"bound": "tensor", "achieved": flops / (ms * 1e-3) / 1e12,
                             "peak": pk, "unit": "TFLOP/s",
                             "frac": (flops / (ms * 1e-3) / 1e12 / pk) if pk else None,
                             "peak_source": "measured bf16 GEMM burst" if pk else None,
                             "flops_per_row": m.flops_per_row()}})
    m.close()
    if plain_subs > 0:
        rng = np.random.default_rng(SEED2)
        subs = S.draw_substrates(plain_subs, rng)
        jobs, P = S.make_jobs(subs, rng, 262144, 0.001, 400)
        t0 = time.perf_counter()
        sig = S.simulate(jobs, device=dev)
        t_mc = time.perf_counter() - t0
        out["plain_signals_per_s"] = len(sig) / t_mc
        out["plain_job"] = ("%d 400-cylinder gamma packings x 64 sequences x 262,144 walkers, "
                            "dt 1 us, 55,001 steps" % plain_subs)
        out["speedup_vs_plain"] = out["signals_per_s"] / out["plain_signals_per_s"]
    return out


def batch_section(A, N, L, dev, reps=2, walker_scale=1.0, max_steps=None):
    """The uneven 256-substrate batch as configured: single cylinders (r 1-8
    um), single spheres (r 2-10 um) and hexagonal packs (f 0.4-0.7, kappa
    0-0.05 um/ms); walkers log-uniform over 1e4-1e6; 8-64 PGSE, cosine and
    square-wave OGSE sequences each; full-length walks (TE 45-50 ms at dt
    5 us).  One launch of the job-class kernels replayed from a CUDA graph with
    the autotuned tile (best of `reps` after one warm-up), against the same
    jobs as device-resident plans launched one after another (one pass), and
    the roofline of the persistent launch (per job the op count of its plan:
    channels, candidates per move, hits per move)."""
    import ctypes as C

    from axonexa_gb300 import workloads as W
    from axonexa_gb300.acquisition import _params, run_flags
    from axonexa_gb300.batch import Batch
    jobs = W.batch_256(walker_scale=walker_scale, max_steps=max_steps)

    b = Batch(jobs, device=dev)
    info = b.info()
    b.launch()
    N.check(L.axx_sync(dev.h), dev.h)
    ms_batch = min(time_launches(N, L, dev, b.launch, reps))
    b.read()
    b.close()
    plans, keep = [], []
    for j in jobs:
        seqs = N.array_of(N.SequenceRec, [q.record() for q in j.seqs])
        basis = N.array_of(N.Basis, [x.record() for x in j.basis])
        h = C.c_void_p()
        if j.lattice is not None:
            p = _params(j.num_walkers, j.steps, j.seed, j.timestep,
                        run_flags(True, j.relaxation, j.permeable))
            N.check(L.axx_plan_lattice(dev.h, C.byref(j.lattice.record()), basis, len(j.basis),
                                       seqs, len(j.seqs), C.byref(p), C.byref(h)), dev.h)
        else:
            p = _params(j.num_walkers, j.steps, j.seed, j.timestep, run_flags(True))
            N.check(L.axx_plan_single(dev.h, basis, seqs, len(j.seqs), C.byref(p), C.byref(h)),
                    dev.h)
        plans.append((h, len(j.seqs), j.num_walkers * (j.steps - 1),
                      j.lattice is not None))
        keep += [seqs, basis, p]

    def launch_plans():
        for h, _, _, _ in plans:
            N.check(L.axx_plan_launch(h), dev.h)

    ms_plans = time_launches(N, L, dev, launch_plans, 1)[0]
    ops = 0.0
    for h, M, ws_j, lat in plans:
        ch, cand, hits = plan_facts(N, L, dev, h, M)
        # single pores walk no periodic wrap
        ops += ws_j * (ops_per_move(ch, cand, hits) - (0 if lat else 6))
        L.axx_plan_destroy(h)
    ws = info["walker_steps"]
    peak = fma_peak(N, L, dev)
    return {"workload": "batch_256 (256 substrates, walkers log-uniform 1e4-1e6, "
                        "full-length walks)" if walker_scale == 1.0 and not max_steps else
                        "batch_256 (walkers x%.2f, walks cut to %s steps)" % (walker_scale,
                                                                              max_steps),
            "jobs": len(jobs), "signals": int(sum(len(j.seqs) for j in jobs)),
            "walker_steps": ws, "persistent_graph_ms": ms_batch,
            "persistent_walker_steps_per_s": ws / (ms_batch * 1e-3),
            "signals_per_s": int(sum(len(j.seqs) for j in jobs)) / (ms_batch * 1e-3),
            "per_job_launches_ms": ms_plans, "per_job_walker_steps_per_s": ws / (ms_plans * 1e-3),
            "speedup": ms_plans / ms_batch, "tile": info["tile"],
            "blocks_per_sm": info["blocks_per_sm"], "work_items": info["items"],
            "kernel_launches_per_batch": info["kernel_launches"],
            "roofline": {"bound": "simt", "achieved": ops / (ms_batch * 1e-3) / 1e12,
                         "peak": peak / 1e12, "unit": "TFLOP/s",
                         "frac": ops / (ms_batch * 1e-3) / peak,
                         "ops_per_move": ops / ws}}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def workload_config(w, nw):
    return {"workload": WORKLOAD, "cylinders": 400, "bases_with_images": len(w["basis"]),
            "area_fraction": round(float(w["fraction"]), 4), "gamma_shape": 5.0,
            "mean_radius_um": 2.5, "kappa_um_per_ms": 0.02, "D_in_ex": [1.7, 2.0],
            "T2_in_ex_ms": [80.0, 60.0], "walkers": nw, "dt_us": 1.0, "steps": w["steps"],
            "moves": w["steps"] - 1, "sequences": len(w["seqs"]), "seed": w["seed"]}


def run_reference(args, world, rank):
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    w = headline_workload()
    # bounded sample: the first n walkers of the job, full walks, per step
    n = int(os.environ.get("AXX_REF_SAMPLE", "32"))
    for _ in range(args.warmup):
        cpu_sample(w, min(n, threads), threads, steps=500)
    total_t, total_ws = 0.0, 0
    for _ in range(args.steps):
        _, t, ws, _ = cpu_sample(w, n, threads)
        total_t += t
        total_ws += ws
    value = total_ws / total_t
    cfg = workload_config(w, w["num_walkers"])
    cfg.update({"sample_walkers_per_step": n, "parallelism": "host threads"})
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total_t / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": cfg,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "%d walkers x full 50,000-step walks per step, FP64 "
                                   "reference-order restatement of "
                                   "updateWalkersLatticePhase (permeable, relaxation)" % n},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the one-shot C-ABI timing")
    ap.add_argument("--e2e-steps", type=int, default=3,
                    help="one-shot C-ABI calls timed for e2e (at most --steps)")
    ap.add_argument("--walkers", type=int, default=None,
                    help="walkers of the headline job (smaller cases for profiling)")
    ap.add_argument("--job-steps", type=int, default=None,
                    help="steps of the headline job (smaller cases for profiling)")
    ap.add_argument("--no-sections", action="store_true",
                    help="print the headline fields only")
    ap.add_argument("--no-surrogate", action="store_true", help="skip the surrogate section")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-launch section")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the magnetisation, WCDMC and mesh sections")
    ap.add_argument("--surrogate-only", action="store_true",
                    help="print only the surrogate section (profiling the inference kernel)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_init()
    if args.impl == "reference":
        return run_reference(args, world, rank)

    import ctypes as C

    import torch

    import axonexa_gb300 as A
    from axonexa_gb300 import _native as N

    torch.cuda.set_device(local)
    dev = A.Device(local)
    L = N.lib()
    if args.surrogate_only:
        if rank == 0:
            print(json.dumps({"surrogate": surrogate_section(A, N, L, dev, plain_subs=0)}))
        return 0
    w = headline_workload()
    nw = args.walkers or w["num_walkers"]
    steps = args.job_steps or w["steps"]
    w["steps"] = steps
    dt, seed = w["timestep"], w["seed"]
    flags = A.acquisition.run_flags(relaxation=True, permeable=True)
    offset = rank * nw  # each rank walks its own walker ids (weak scaling)
    h = make_plan(A, N, L, dev, w["lattice"], w["basis"], w["seqs"], nw, steps, dt, seed, flags,
                  offset)
    M = len(w["seqs"])
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    ws = nw * (steps - 1)

    def launch():
        N.check(L.axx_plan_launch(h), dev.h)

    # ---- warm-up
    for _ in range(args.warmup):
        launch()
    N.check(L.axx_sync(dev.h), dev.h)
    torch.cuda.synchronize()

    # ---- timed region: the device-resident plan, one event pair per step,
    # L2 flushed between steps (outside the events)
    clocks = Clocks(local)
    clocks.start()
    barrier(world)
    torch.cuda.synchronize()
    walk_ms = time_launches(N, L, dev, launch, args.steps, flush)
    N.check(L.axx_sync(dev.h), dev.h)
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    t_step = max_over_ranks(sum(walk_ms) / args.steps, world)
    value = world * ws / (t_step * 1e-3)
    channels, cand, hits = plan_facts(N, L, dev, h, M)
    kl = C.c_int()
    N.check(L.axx_plan_info(h, None, None, C.byref(kl), None), dev.h)
    L.axx_plan_destroy(h)

    # ---- e2e: the one-shot C-ABI call (axx_run_lattice) with host records in
    # and host sums out; the bytes it moves are counted by the library
    barrier(world)
    e2e_steps = 0 if args.no_e2e else max(1, min(args.e2e_steps, args.steps))
    h2d0, d2h0 = transfer_bytes(N, L, dev)
    e2e_s = 0.0
    for _ in range(e2e_steps):
        flush_l2(flush)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        A.run_lattice(w["lattice"], w["basis"], w["seqs"], nw, steps, dt, seed,
                      relaxation=True, permeable=True, walker_offset=offset, device=dev)
        e2e_s += time.perf_counter() - t0
    h2d1, d2h1 = transfer_bytes(N, L, dev)
    e2e_step = max_over_ranks(e2e_s / e2e_steps, world) if e2e_steps else float("nan")
    e2e_value = world * ws / e2e_step if e2e_steps else None

    if rank != 0:
        return 0
    peak = fma_peak(N, L, dev)
    F = ops_per_move(channels, cand, hits)
    achieved = nw * (steps - 1) * F / (t_step * 1e-3)
    roof = {"bound": "simt", "achieved": achieved / 1e12, "peak": peak / 1e12,
            "unit": "TFLOP/s", "frac": achieved / peak,
            "traffic": WALK_DRAM_BYTES_PER_WALKER * nw,
            "traffic_source": "ncu dram__bytes_read+write of the walk launch at 262,144 "
                              "walkers x 2,000 steps, scaled by walkers (bytes per launch)",
            "issue_active_ncu": WALK_ISSUE_ACTIVE_NCU,
            "peak_source": "measured: axx_fp32_fma_peak (register FMA chains on all SMs)",
            "ops_per_move": round(F, 2), "channels": channels,
            "candidates_per_move": round(cand, 3), "hits_per_move": round(hits, 5)}
    cfg = workload_config(w, nw)
    cfg.update({"parallelism": "replicas (walker ranges)" if world > 1 else "single GPU",
                "l2": "flushed between steps (512 MiB write)"})
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": cfg,
        "e2e": {"value": e2e_value, "unit": UNIT, "steps": e2e_steps,
                "h2d_bytes_per_step": (h2d1 - h2d0) // max(e2e_steps, 1),
                "d2h_bytes_per_step": (d2h1 - d2h0) // max(e2e_steps, 1),
                "bytes_source": "counted by the library (axx_transfer_bytes)"},
        "gpu_launches": args.steps * kl.value,
        "roofline": roof,
        "clocks": clk,
    }
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        n = int(os.environ.get("AXX_CPU_SAMPLE", "640"))
        v, t, _, ref_sums = cpu_sample(w, n, threads)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": "the first %d walkers x full %d-step walks (%.1f s), "
                                          "FP64 reference-order oracle" % (n, steps, t)}
        # every signal of that sample against the FP64 walk of the same streams
        line["fp64_check"] = fp64_check(A, dev, w, n, ref_sums)
    if not args.no_sections:
        line["restricted_cylinder"] = restricted_section(A, N, L, dev)
        line["free_box"] = free_box_section(A, dev)
        if not args.no_batch:
            line["batch"] = batch_section(A, N, L, dev)
        if not args.no_extra:
            from axonexa_gb300 import workloads as W
            # host-timed calls through the C ABI (tables uploaded per call)
            line["mag"] = W.measure_mag(reps=3, device=dev)
            line["wc"] = W.measure_wc(reps=3, device=dev)
            line["mesh"] = W.measure_mesh(reps=3, device=dev)
        if not args.no_surrogate:
            line["surrogate"] = surrogate_section(A, N, L, dev)
    print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
