"""Throughput of the GB300 walker on the restricted-cylinder workload.

Workload (one bench step): a single impermeable cylinder of radius 5 um, axis
z, centred in a 12 um periodic square cell; 1,048,576 walkers uniform in the
cell (intra/extra split by volume); D_in = D_ex = 2.0 um^2/ms, T2 80/60 ms;
dt = 2 us.  Two acquisitions, each one walk of every walker:
  * PGSE delta 10 ms, Delta 40 ms (25,000 steps), 32 G values 0-200 mT/m along x;
  * cosine OGSE at 50/100/200 Hz: delta 20 ms, Delta 40 ms (N = 1, 2, 4
    periods, 30,000 steps), 100 mT/m along x.
Inputs are seeded synthetic parameters (Philox seed 1234); nothing is read
from a dataset.

Lines printed (rank 0):
  default arm       -- walker-steps/s with the plans resident on the GPU
                       (value), and through the one-shot C-ABI call with host
                       records in and host sums out (e2e); roofline of the walk
                       kernel against the measured FP32 FMA peak; the CPU oracle
                       on a bounded sample of the same workload (cpu_baseline);
                       "mag": the Bloch walk on the magLF low-field cell;
                       "wc": the WCDMC walker beside the specular one;
                       "batch": the uneven 256-substrate batch in one
                       persistent graph launch against per-job launches;
                       "surrogate": tcgen05 inference signals/s on 1e6 queries
                       (tensor roofline against the measured bf16 peak) beside
                       the plain walk's signals/s on the surrogate's own
                       data-generation jobs.
  --impl reference  -- the reference's walker loop on the host cores: the CPU
                       restatement of updateWalkersLatticePhase (oracle, FP64,
                       reference operation order) over all host threads.
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

# workload (reference units: mm, ms, T)
CELL, RADIUS = 0.012, 0.005
D, T2_IN, T2_EX = 2.0e-6, 80.0, 60.0
DT = 0.002
N_WALKERS = 1 << 20
SEED = 1234
PGSE_STEPS, OGSE_STEPS = 25000, 30000
# from one ncu --set full capture of the PGSE walk launch (262,144 walkers):
# DRAM bytes read + written per walker, and smsp__issue_active
WALK_DRAM_BYTES_PER_WALKER = 159488.0 / 262144
WALK_ISSUE_ACTIVE_NCU = 0.776


def workload_records(A):
    import numpy as np
    lat = A.Lattice(CELL, CELL, CELL, T2_EX, 0.0, D, 1)
    cyl = [A.Cylinder_XY(CELL / 2, CELL / 2, RADIUS, T2_IN, 0.0, D, 1, 0.0)]
    pgse = [A.RectGrad(g * 1e-6, 10.0, 30.0) for g in np.linspace(0.0, 200.0, 32)]
    ogse = [A.CosGFunc(100e-6, 20.0, 20.0, n) for n in (1, 2, 4)]
    return lat, cyl, [(pgse, PGSE_STEPS), (ogse, OGSE_STEPS)]


def walker_steps_per_bench_step(n=N_WALKERS):
    return n * ((PGSE_STEPS - 1) + (OGSE_STEPS - 1))


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


def cpu_sample_baseline(n_walkers: int, threads: int, steps_frac: float = 1.0):
    """The oracle's FP64 reference-order walk (updateWalkersLatticePhase
    restated) over a bounded walker sample of the same workload."""
    from oracle import oracle as O
    O.lib()
    import numpy as np
    lat = O.Lattice(CELL, CELL, CELL, T2_EX, 0.0, D)
    cyl = [O.Basis(0, 1, CELL / 2, CELL / 2, 0.0, RADIUS, D, T2_IN, 0.0, 0.0, 1e-14)]
    pg = [O.Sequence(0, 0, g * 1e-6, 10.0, 30.0, 1, 0, 0) for g in np.linspace(0, 200, 32)]
    og = [O.Sequence(1, n, 100e-6, 20.0, 20.0, 1, 0, 0) for n in (1, 2, 4)]
    total_ws, t0 = 0, time.perf_counter()
    sums = []
    for seqs, steps in ((pg, PGSE_STEPS), (og, OGSE_STEPS)):
        st = max(2, int(steps * steps_frac))
        p = O.Params(n_walkers, st, 0, 0, 1, SEED, DT, 0.0, 0)
        s, _, _ = O.walk(lat, cyl, seqs, p, O.REF64, nthreads=threads)
        sums.append(s)
        total_ws += n_walkers * (st - 1)
    dt = time.perf_counter() - t0
    return total_ws / dt, dt, total_ws, sums


def fp64_check(A, dev, n_walkers: int, ref_sums) -> dict:
    """The GPU walk of the same first walkers (the same Philox streams)
    against the oracle's FP64 reference-order sums: |dS| per sequence and its
    ratio to the walk's standard error."""
    import numpy as np
    lat, cyl, acqs = workload_records(A)
    worst_d, worst_r = 0.0, 0.0
    for (seqs, steps), ref in zip(acqs, ref_sums):
        r = A.run_lattice(lat, cyl, seqs, n_walkers, steps, DT, SEED, relaxation=True,
                          device=dev)
        s_ref = np.hypot(ref[:, 0], ref[:, 1]) / n_walkers
        d = np.abs(r.signal - s_ref)
        worst_d = max(worst_d, float(d.max()))
        worst_r = max(worst_r, float((d / np.maximum(r.stderr, 1e-12)).max()))
    return {"walkers": n_walkers, "sequences": sum(len(q) for q, _ in acqs),
            "max_abs_dS": worst_d, "max_dS_over_se": worst_r,
            "oracle": "FP64 reference-order restatement, the same streams"}


def surrogate_section(A, N, L, dev, queries=1000000, reps=10, plain_subs=2):
    """Learned-surrogate throughput: tcgen05 inference of `queries` rows
    resident on the GPU (CUDA events on the library stream), the same through
    the host API (host rows in, host signals out), and the plain walk's
    signals/s on the surrogate's data-generation jobs (100-cylinder gamma
    packings, 262,144 walkers, 64 sequences each, dt 5 us)."""
    import ctypes as C

    import numpy as np
    import torch

    from axonexa_gb300 import surrogate as S
    m = S.MLP(seed=0, device=dev)
    g = torch.Generator(device="cuda")
    g.manual_seed(SEED)
    X = torch.rand(queries, 10, device="cuda", generator=g) * 2 - 1
    y = torch.empty(queries, device="cuda")
    torch.cuda.synchronize()
    for _ in range(3):
        m.predict_device(X.data_ptr(), queries, y.data_ptr())
    N.check(L.axx_sync(dev.h), dev.h)
    times = []
    for _ in range(reps):
        N.check(L.axx_event_record(dev.h, 0), dev.h)
        m.predict_device(X.data_ptr(), queries, y.data_ptr())
        N.check(L.axx_event_record(dev.h, 1), dev.h)
        ms = C.c_float()
        N.check(L.axx_event_elapsed(dev.h, 0, 1, C.byref(ms)), dev.h)
        times.append(ms.value)
    ms = float(np.median(times))
    flops = m.flops_per_row() * queries
    Xh = X.cpu().numpy()
    m.predict(Xh[:4096])
    t0 = time.perf_counter()
    yh = m.predict(Xh)
    e2e_s = time.perf_counter() - t0
    assert np.array_equal(yh, y.cpu().numpy()), "host and device inference disagree"
    peaks = measured_peaks()
    pk = peaks.get("bf16_tflops")
    out = {"queries": queries, "signals_per_s": queries / (ms * 1e-3), "ms": ms,
           "e2e_signals_per_s": queries / e2e_s, "h2d_bytes": int(Xh.nbytes),
           "d2h_bytes": int(4 * queries), "kernel_launches_per_call": 1,
           "roofline": {"bound": "tensor", "achieved": flops / (ms * 1e-3) / 1e12,
                        "peak": pk, "unit": "TFLOP/s",
                        "frac": (flops / (ms * 1e-3) / 1e12 / pk) if pk else None,
                        "peak_source": "measured bf16 GEMM burst" if pk else None,
                        "flops_per_row": m.flops_per_row()}}
    m.close()
    if plain_subs > 0:
        rng = np.random.default_rng(SEED)
        subs = S.draw_substrates(plain_subs, rng)
        jobs, P = S.make_jobs(subs, rng, 262144, 0.005, 100)
        S.simulate(jobs, device=dev)  # same batch shape: tunes (cached) and warms up
        t0 = time.perf_counter()
        sig = S.simulate(jobs, device=dev)
        t_mc = time.perf_counter() - t0
        out["plain_signals_per_s"] = len(sig) / t_mc
        out["plain_job"] = "%d gamma packings x 64 sequences x 262,144 walkers, dt 5 us" % plain_subs
        out["speedup_vs_plain"] = out["signals_per_s"] / out["plain_signals_per_s"]
    return out


def batch_section(A, N, L, dev, reps=3, walker_scale=0.25, max_steps=3000):
    """The uneven 256-substrate batch (single cylinders, single spheres and
    hexagonal packs; walkers log-uniform over 1e4-1e6 scaled by
    `walker_scale`; 8-64 sequences each; walks cut to `max_steps`) as one
    persistent launch replayed from a CUDA graph with the autotuned tile,
    against the same jobs as device-resident plans launched one after another."""
    import ctypes as C

    from axonexa_gb300 import workloads as W
    from axonexa_gb300.acquisition import _params, run_flags
    from axonexa_gb300.batch import Batch
    jobs = W.batch_256(walker_scale=walker_scale, max_steps=max_steps)

    def timed(launch):
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
        return best

    b = Batch(jobs, device=dev)
    info = b.info()
    ms_batch = timed(b.launch)
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
        plans.append(h)
        keep += [seqs, basis, p]

    def launch_plans():
        for h in plans:
            N.check(L.axx_plan_launch(h), dev.h)

    ms_plans = timed(launch_plans)
    for h in plans:
        L.axx_plan_destroy(h)
    ws = info["walker_steps"]
    return {"workload": "batch_256 (walkers x%.2f, walks cut to %d steps)" % (walker_scale,
                                                                                max_steps),
            "jobs": len(jobs), "signals": int(sum(len(j.seqs) for j in jobs)),
            "walker_steps": ws, "persistent_graph_ms": ms_batch,
            "persistent_walker_steps_per_s": ws / (ms_batch * 1e-3),
            "per_job_launches_ms": ms_plans, "per_job_walker_steps_per_s": ws / (ms_plans * 1e-3),
            "speedup": ms_plans / ms_batch, "tile": info["tile"],
            "blocks_per_sm": info["blocks_per_sm"], "work_items": info["items"],
            "kernel_launches_per_batch": info["kernel_launches"]}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def run_reference(args, world, rank):
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    # bounded sample: 2,048 walkers of the full workload per step
    n = int(os.environ.get("AXX_REF_SAMPLE", "2048"))
    for _ in range(args.warmup):
        cpu_sample_baseline(max(threads, 64), threads, 0.01)
    vals, total_t, total_ws = [], 0.0, 0
    for _ in range(args.steps):
        v, t, ws, _ = cpu_sample_baseline(n, threads)
        vals.append(v)
        total_t += t
        total_ws += ws
    value = total_ws / total_t
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total_t / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "restricted_cylinder_pgse32_ogse3", "walkers": N_WALKERS,
                   "sample_walkers_per_step": n, "moves": [PGSE_STEPS - 1, OGSE_STEPS - 1],
                   "dt_ms": DT, "parallelism": "host threads"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "%d walkers x full 25,000 + 30,000-step walks per step, "
                                   "FP64 reference-order restatement of "
                                   "updateWalkersLatticePhase" % n},
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
    ap.add_argument("--walkers", type=int, default=N_WALKERS,
                    help="walkers per acquisition (smaller cases for profiling)")
    ap.add_argument("--no-surrogate", action="store_true", help="skip the surrogate section")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-launch section")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the magnetisation and WCDMC walker sections")
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
    lat, cyl, acqs = workload_records(A)
    nw = args.walkers
    offset = rank * nw  # each rank walks its own walker ids (weak scaling)
    plans = []
    for seqs, steps in acqs:
        p = A.acquisition._params(nw, steps, SEED, DT, A.acquisition.run_flags(
            relaxation=True), offset=offset)
        h = C.c_void_p()
        N.check(L.axx_plan_lattice(dev.h, C.byref(lat.record()),
                                   N.array_of(N.Basis, [c.record() for c in cyl]), 1,
                                   N.array_of(N.SequenceRec, [q.record() for q in seqs]),
                                   len(seqs), C.byref(p), C.byref(h)), dev.h)
        plans.append((h, len(seqs), steps, p))
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    ws = walker_steps_per_bench_step(nw)

    def step_resident():
        for h, _, _, _ in plans:
            N.check(L.axx_plan_launch(h), dev.h)

    # ---- warm-up
    for _ in range(args.warmup):
        step_resident()
    N.check(L.axx_sync(dev.h), dev.h)
    torch.cuda.synchronize()

    # ---- timed region: device-resident plans, one event pair per step,
    # L2 flushed between steps (outside the events)
    clocks = Clocks(local)
    clocks.start()
    barrier(world)
    torch.cuda.synchronize()
    walk_ms, total_ms = [], 0.0
    for _ in range(args.steps):
        flush_l2(flush)
        torch.cuda.synchronize()
        N.check(L.axx_event_record(dev.h, 0), dev.h)
        for h, _, _, _ in plans:
            N.check(L.axx_plan_launch(h), dev.h)
        N.check(L.axx_event_record(dev.h, 1), dev.h)
        ms = C.c_float()
        N.check(L.axx_event_elapsed(dev.h, 0, 1, C.byref(ms)), dev.h)
        total_ms += ms.value
        walk_ms.append(ms.value)
    N.check(L.axx_sync(dev.h), dev.h)
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    t_step = max_over_ranks(total_ms / args.steps, world)
    value = world * ws / (t_step * 1e-3)

    # results of the last launch (and hit statistics for the roofline)
    hits_per_move = []
    for h, M, steps, _ in plans:
        mx, my = (C.c_double * M)(), (C.c_double * M)()
        st = N.Stats(None, None, None, 0, 0, 0)
        N.check(L.axx_plan_read(h, mx, my, C.byref(st)), dev.h)
        hits_per_move.append(st.boundary_hits / max(st.walker_steps, 1))

    # ---- e2e: the one-shot C-ABI call with host records in and host sums out
    barrier(world)
    e2e_ms = 0.0
    h2d = d2h = 0
    for _ in range(0 if args.no_e2e else args.steps):
        flush_l2(flush)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for seqs, steps in acqs:
            r = A.run_lattice(lat, cyl, seqs, nw, steps, DT, SEED, relaxation=True,
                              walker_offset=offset, device=dev)
        e2e_ms += (time.perf_counter() - t0) * 1e3
    e2e_step = max_over_ranks(e2e_ms / args.steps, world) if not args.no_e2e else float("nan")
    for seqs, steps in acqs:
        # tables uploaded per call: instances, cell lists, slots, waveforms, coefficients
        h2d += 32 * 2 + 8 + 2 + 16 * 2 + 4 * 2 + 4 * steps * (1 if len(seqs) > 3 else 3) + \
            8 * len(seqs) * (1 if len(seqs) > 3 else 3)
        d2h += 8 * 5 * len(seqs) + 8 * 4
    e2e_value = world * ws / (e2e_step * 1e-3)

    if rank != 0:
        return 0
    # ---- roofline: algorithmic FP32 ops per move (one FMA = one op):
    # 18 direction + move, 6 periodic wrap, 7 per phase channel, 1 T2,
    # 23 per candidate cylinder test, 20 per boundary hit
    F = []
    for (h, M, steps, _), hp in zip(plans, hits_per_move):
        ch = C.c_int()
        N.check(L.axx_plan_info(h, C.byref(ch), None, None, None), dev.h)
        F.append(18 + 6 + 7 * ch.value + 1 + 23 * 1 + 20 * hp)
    moves = [PGSE_STEPS - 1, OGSE_STEPS - 1]
    ops = nw * sum(f * m for f, m in zip(F, moves))
    peak = C.c_double()
    N.check(L.axx_fp32_fma_peak(dev.h, C.byref(peak)), dev.h)
    achieved = ops / (t_step * 1e-3)
    roof = {"bound": "simt", "achieved": achieved / 1e12, "peak": peak.value / 1e12,
            "unit": "TFLOP/s", "frac": achieved / peak.value,
            "traffic": WALK_DRAM_BYTES_PER_WALKER * nw,
            "traffic_source": "ncu dram__bytes_read+write of the PGSE walk launch at 262,144 "
                              "walkers, scaled by walkers (bytes per launch)",
            "issue_active_ncu": WALK_ISSUE_ACTIVE_NCU,
            "peak_source": "measured: axx_fp32_fma_peak (register FMA chains on all SMs)",
            "ops_per_move": [round(f, 2) for f in F],
            "hits_per_move": [round(x, 4) for x in hits_per_move]}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "restricted_cylinder_pgse32_ogse3", "walkers": nw,
                   "cell_um": 12.0, "radius_um": 5.0, "dt_us": 2.0,
                   "moves": moves, "sequences": [32, 3], "seed": SEED,
                   "parallelism": "replicas (walker ranges)" if world > 1 else "single GPU",
                   "l2": "flushed between steps (512 MiB write)"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": args.steps * 2 * len(plans),
        "roofline": roof,
        "clocks": clk,
    }
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
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        n = int(os.environ.get("AXX_CPU_SAMPLE", "4096"))
        v, t, wsamp, ref_sums = cpu_sample_baseline(n, threads)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": "%d walkers x full walks (%.1f s), FP64 reference-"
                                          "order oracle" % (n, t)}
        # every signal of that sample against the FP64 walk of the same streams
        line["fp64_check"] = fp64_check(A, dev, n, ref_sums)
    for h, _, _, _ in plans:
        L.axx_plan_destroy(h)
    print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
