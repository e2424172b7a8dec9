"""Full-scale surrogate workflow: data generation on the walk, training on the
tensor cores, held-out evaluation against plain Monte Carlo, inference
throughput.

    python -m axonexa_gb300.surrogate_run --out result.json \
        --save-weights axonexa_gb300/data/surrogate_400cyl.npz

Defaults follow the surrogate configuration: 200,000 (parameters, signal)
pairs from 400-cylinder gamma packings (the permeable benchmark substrate's
style: dt 1 us, parameters uniform over the training ranges) with 262,144
walkers each; Adam with batches of 4,096; |dS| against plain Monte Carlo on
2,048 held-out pairs from unseen seeds, whose truth is walked with 4,194,304
walkers (standard error near 3e-4, well below the 2e-3 bar); a second packing
of the first held-out substrates (another placement of the same radii)
measures how much of |dS| the packing realisation alone explains; 1e6
inference queries.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import time

import numpy as np


def _stats(err, pref):
    err = np.asarray(err)
    return {pref + "mean": float(err.mean()), pref + "p95": float(np.quantile(err, 0.95)),
            pref + "max": float(err.max()), pref + "frac_within_2e-3": float(np.mean(err <= 2e-3))}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--pairs", type=int, default=200000)
    ap.add_argument("--walkers", type=int, default=262144)
    ap.add_argument("--timestep", type=float, default=0.001)
    ap.add_argument("--cylinders", type=int, default=400)
    ap.add_argument("--steps", type=int, default=60000, help="Adam steps of 4,096 pairs")
    ap.add_argument("--lr", type=float, default=2e-3, help="initial learning rate")
    ap.add_argument("--heldout", type=int, default=2048)
    ap.add_argument("--heldout-walkers", type=int, default=1 << 22)
    ap.add_argument("--realizations", type=int, default=4,
                    help="held-out substrates walked again on a second packing")
    ap.add_argument("--queries", type=int, default=1000000)
    ap.add_argument("--out", default="")
    ap.add_argument("--data", default="", help="pairs file (.npz): read if present, else written")
    ap.add_argument("--save-weights", default="")
    a = ap.parse_args(argv)
    import torch

    import axonexa_gb300.surrogate as S
    from axonexa_gb300 import _native as N
    dev = S.default_device()
    n_sub = (a.pairs + 63) // 64
    rec = {"pairs": n_sub * 64, "substrates": n_sub, "walkers": a.walkers,
           "timestep_ms": a.timestep, "cylinders_per_cell": a.cylinders}
    if a.data and os.path.exists(a.data):
        z = np.load(a.data)
        P, Y, Ph, Yh, SEh = z["P"], z["Y"], z["Ph"], z["Yh"], z["SEh"]
        rec["data_loaded"] = a.data
    else:
        counts = {}
        t0 = time.perf_counter()
        P, Y = S.generate(n_sub, seed=12345, walkers=a.walkers, timestep=a.timestep,
                          n_cyl=a.cylinders, device=dev, counts=counts)
        rec["generation_s"] = time.perf_counter() - t0
        rec["mc_signals_per_s"] = len(Y) / rec["generation_s"]
        rec["walker_steps"] = counts.get("walker_steps", 0)
        rec["reflection_cap_hits"] = counts.get("cap_hits", 0)
        se = []
        t0 = time.perf_counter()
        Ph, Yh = S.generate((a.heldout + 63) // 64, seed=987654, walkers=a.heldout_walkers,
                            timestep=a.timestep, n_cyl=a.cylinders, device=dev, stderr=se)
        SEh = np.concatenate(se)
        rec["heldout_generation_s"] = time.perf_counter() - t0
        if a.data:
            np.savez_compressed(a.data, P=P, Y=Y, Ph=Ph, Yh=Yh, SEh=SEh)
    rec["heldout_pairs"] = int(len(Yh))
    rec["heldout_walkers"] = a.heldout_walkers
    rec["heldout_truth_se_mean"] = float(np.mean(SEh))
    rec["heldout_truth_se_max"] = float(np.max(SEh))
    # the packing realisation: the first held-out substrates on another
    # placement of the same radii (same parameter rows, same sequences)
    if a.realizations > 0:
        rng = np.random.default_rng(987654)
        subs = S.draw_substrates((a.heldout + 63) // 64, rng)[:a.realizations]
        jobs, P2 = S.make_jobs(subs, np.random.default_rng(55555), a.heldout_walkers,
                               a.timestep, a.cylinders)
        # same sequences as the held-out rows: rebuild them from those rows
        for k, j in enumerate(jobs):
            rows = Ph[k * 64:(k + 1) * 64]
            j.seqs = [S._sequence(r[6], r[7], r[8], r[9]) for r in rows]
        Y2 = S.simulate(jobs, device=dev)
        d2 = np.abs(Y2 - Yh[:len(Y2)])
        rec.update(_stats(d2, "second_packing_abs_dS_"))
    t0 = time.perf_counter()
    sur = S.Surrogate.fit(P, Y, steps=a.steps, batch=4096, lr=a.lr, seed=0, device=dev)
    rec["train_steps"] = a.steps
    rec["train_lr"] = a.lr
    rec["train_s"] = time.perf_counter() - t0
    rec["final_loss"] = float(np.mean(sur.loss[-100:]))
    pred, fb = sur.predict(Ph)
    err = np.abs(pred - Yh)
    rec.update(_stats(err, "heldout_abs_dS_"))
    rec["heldout_fallback_rows"] = int(fb.sum())
    if a.save_weights:
        os.makedirs(os.path.dirname(os.path.abspath(a.save_weights)), exist_ok=True)
        meta = {k: rec[k] for k in ("pairs", "walkers", "timestep_ms", "cylinders_per_cell",
                                    "train_steps", "train_lr", "heldout_walkers") if k in rec}
        S.save(sur.mlp, a.save_weights, heldout={"P": Ph, "truth": Yh, "truth_se": SEh},
               meta=meta)
    # inference throughput with device-resident queries (tensor cores)
    Q = np.tile(S.normalise(Ph), (a.queries // len(Ph) + 1, 1))[:a.queries].astype(np.float32)
    dX = torch.from_numpy(Q).cuda()
    dy = torch.empty(a.queries, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    L = N.lib()
    for _ in range(3):
        sur.mlp.predict_device(dX.data_ptr(), a.queries, dy.data_ptr())
    N.check(L.axx_sync(dev.h), dev.h)
    times = []
    for _ in range(10):
        N.check(L.axx_event_record(dev.h, 0), dev.h)
        sur.mlp.predict_device(dX.data_ptr(), a.queries, dy.data_ptr())
        N.check(L.axx_event_record(dev.h, 1), dev.h)
        ms_ = C.c_float()
        N.check(L.axx_event_elapsed(dev.h, 0, 1, C.byref(ms_)), dev.h)
        times.append(ms_.value)
    ms = float(np.median(times))
    y_dev = dy.cpu().numpy()[:len(Ph)]
    assert np.allclose(y_dev, pred[:len(Ph)], atol=1e-6), "device and host inference disagree"
    flops = sur.mlp.flops_per_row() * a.queries
    rec.update({"inference_queries": a.queries, "inference_ms": ms,
                "surrogate_signals_per_s": a.queries / (ms * 1e-3),
                "inference_tflops": flops / (ms * 1e-3) / 1e12})
    if "mc_signals_per_s" in rec:
        rec["speedup_vs_mc_signals_per_s"] = rec["surrogate_signals_per_s"] / rec["mc_signals_per_s"]
    print(json.dumps(rec))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(rec, f, indent=1)


if __name__ == "__main__":
    main()
