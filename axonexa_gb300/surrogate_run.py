"""Full-scale surrogate workflow (data generation on the walk, training,
held-out evaluation against plain Monte Carlo, inference throughput).

    python -m axonexa_gb300.surrogate_run --out result.json [--pairs 200000]

Defaults follow the surrogate configuration: 200,000 (parameters, signal)
pairs from gamma-radius packings with 262,144 walkers each, Adam with batches
of 4,096, 1e6 inference queries, |dS| against plain Monte Carlo on 2,048
held-out pairs from unseen seeds.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import time

import numpy as np


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--pairs", type=int, default=200000)
    ap.add_argument("--walkers", type=int, default=262144)
    ap.add_argument("--timestep", type=float, default=0.005)
    ap.add_argument("--cylinders", type=int, default=100)
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--heldout", type=int, default=2048)
    ap.add_argument("--queries", type=int, default=1000000)
    ap.add_argument("--out", default="")
    ap.add_argument("--save-data", default="", help="write the pairs (P, Y, Ph, Yh) as .npz")
    a = ap.parse_args(argv)
    import torch

    import axonexa_gb300.surrogate as S
    from axonexa_gb300 import _native as N
    dev = S.default_device()
    n_sub = (a.pairs + 63) // 64
    counts = {}
    t0 = time.perf_counter()
    P, Y = S.generate(n_sub, seed=12345, walkers=a.walkers, timestep=a.timestep,
                      n_cyl=a.cylinders, device=dev, counts=counts)
    t_gen = time.perf_counter() - t0
    Ph, Yh = S.generate((a.heldout + 63) // 64, seed=987654, walkers=a.walkers,
                        timestep=a.timestep, n_cyl=a.cylinders, device=dev)
    if a.save_data:
        np.savez_compressed(a.save_data, P=P, Y=Y, Ph=Ph, Yh=Yh)
    t0 = time.perf_counter()
    sur = S.Surrogate.fit(P, Y, steps=a.steps, batch=4096, lr=1e-3, seed=0, device=dev)
    t_train = time.perf_counter() - t0
    pred, fb = sur.predict(Ph)
    err = np.abs(pred - Yh)
    # inference throughput with device-resident queries (tensor cores)
    Q = np.tile(S.normalise(Ph), (a.queries // len(Ph) + 1, 1))[:a.queries].astype(np.float32)
    dX = torch.from_numpy(Q).cuda()
    dy = torch.empty(a.queries, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    L = N.lib()
    for _ in range(3):
        sur.mlp.predict_device(dX.data_ptr(), a.queries, dy.data_ptr())
    N.check(L.axx_sync(dev.h), dev.h)
    # events on the library's own stream, where the inference kernel runs
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
    rec = {
        "pairs": int(len(Y)), "substrates": n_sub, "walkers": a.walkers, "timestep_ms": a.timestep,
        "cylinders_per_cell": a.cylinders, "generation_s": t_gen,
        "mc_signals_per_s": len(Y) / t_gen, "walker_steps": counts.get("walker_steps", 0),
        "reflection_cap_hits": counts.get("cap_hits", 0), "train_steps": a.steps, "train_s": t_train,
        "final_loss": float(np.mean(sur.loss[-100:])), "heldout_pairs": int(len(Yh)),
        "heldout_abs_err_mean": float(err.mean()), "heldout_abs_err_p95": float(np.quantile(err, 0.95)),
        "heldout_abs_err_max": float(err.max()), "heldout_frac_within_2e-3": float(np.mean(err <= 2e-3)),
        "mc_noise_se_typical": float(1.0 / np.sqrt(a.walkers)),
        "inference_queries": a.queries, "inference_ms": ms,
        "surrogate_signals_per_s": a.queries / (ms * 1e-3),
        "inference_tflops": flops / (ms * 1e-3) / 1e12,
    }
    rec["speedup_vs_mc_signals_per_s"] = rec["surrogate_signals_per_s"] / rec["mc_signals_per_s"]
    print(json.dumps(rec))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(rec, f, indent=1)


if __name__ == "__main__":
    main()
