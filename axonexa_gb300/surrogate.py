"""Learned surrogate of the walk: an MLP from substrate and sequence
parameters to the signal, trained on signals the simulator produces.

Inputs (10): mean radius [um], gamma shape, intracellular area fraction,
kappa [um/ms], D_in, D_ex [um^2/ms], G [mT/m], Delta, delta [ms], omega [Hz]
(omega = 0: PGSE; otherwise cosine OGSE with omega*delta whole periods).
Output: the normalised signal |M|/N read at the fixed time TE_READ (55 ms,
the longest Delta + delta of the ranges) for every sequence: the walk goes on
past a sequence's own echo with its phase frozen while T2 keeps acting, so a
common readout time makes the signal a function of the ten inputs alone.

The network (MLP in -> 4 x 256 SiLU -> 1) lives in libaxx.so: BF16 tensor-core
training (tcgen05 GEMMs with TMEM accumulators, FP32 accumulate, Adam) and
tcgen05 inference.  The trained parameters of the 400-cylinder configuration,
with their held-out pairs and Monte Carlo truth, ship in data/ (load()).  Plain
Monte Carlo stays the fallback: queries outside the training ranges are
simulated, not predicted.
"""
from __future__ import annotations

import ctypes as C
import json
import math
import os
from dataclasses import dataclass
from typing import Dict, List, Optional, Tuple

import numpy as np

from . import _native as N
from .acquisition import CosGFunc, Device, RectGrad, default_device
from .batch import Job, run_batch
from .substrate import gamma_quantile_radii, pack_radii

INPUTS = ("mean_radius_um", "gamma_shape", "fraction", "kappa_um_ms", "D_in", "D_ex", "G_mTm",
          "Delta_ms", "delta_ms", "omega_hz")
# training ranges around the 400-cylinder permeable substrate (mean radius
# 2.5 um, shape 5, f 0.6, kappa 0.02, D 1.7 / 2.0) and its sequences
RANGES = np.array([[1.5, 3.5], [3.0, 8.0], [0.40, 0.65], [0.0, 0.05], [1.2, 2.2], [1.6, 2.6],
                   [0.0, 300.0], [20.0, 40.0], [5.0, 15.0], [0.0, 400.0]])
T2_IN, T2_EX = 80.0, 60.0
TE_READ = float(RANGES[7][1] + RANGES[8][1])  # ms


class MLP:
    """axx_mlp: in_dim -> depth x 256 SiLU -> 1."""

    def __init__(self, in_dim=10, width=256, depth=4, seed=0, device: Device = None):
        self.dev = device or default_device()
        h = C.c_void_p()
        N.check(N.lib().axx_mlp_create(self.dev.h, in_dim, width, depth, seed, C.byref(h)),
                self.dev.h)
        self.h = h
        self.dev.adopt(self)
        self.in_dim, self.width, self.depth = in_dim, width, depth
        n = C.c_int64()
        N.check(N.lib().axx_mlp_num_params(h, C.byref(n)))
        self.nparam = n.value

    def close(self):
        if getattr(self, "h", None):
            N.lib().axx_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _f(a):
        a = np.ascontiguousarray(a, dtype=np.float32)
        return a, a.ctypes.data_as(C.POINTER(C.c_float))

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.nparam, np.float32)
        N.check(N.lib().axx_mlp_get_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float))),
                self.dev.h)
        return p

    def set_params(self, p):
        p, ptr = self._f(p)
        N.check(N.lib().axx_mlp_set_params(self.h, ptr), self.dev.h)

    def layers(self, p=None):
        """[(W [out][in], b [out]), ...] views of a parameter vector."""
        p = self.get_params() if p is None else p
        out, o = [], 0
        for l in range(self.depth + 1):
            i = self.in_dim if l == 0 else self.width
            od = 1 if l == self.depth else self.width
            W = p[o:o + od * i].reshape(od, i)
            o += od * i
            b = p[o:o + od]
            o += od
            out.append((W, b))
        return out

    def gradients(self, X, y):
        X, px = self._f(X)
        y, py = self._f(y)
        g = np.zeros(self.nparam, np.float32)
        loss = C.c_float()
        N.check(N.lib().axx_mlp_gradients(self.h, px, py, len(y),
                                          g.ctypes.data_as(C.POINTER(C.c_float)),
                                          C.byref(loss)), self.dev.h)
        return g, loss.value

    def train(self, X, y, batch=4096, steps=1000, lr=1e-3, seed=0):
        X, px = self._f(X)
        y, py = self._f(y)
        loss = np.zeros(max(steps, 1), np.float32)
        N.check(N.lib().axx_mlp_train(self.h, px, py, len(y), batch, steps, lr, seed,
                                      loss.ctypes.data_as(C.POINTER(C.c_float))), self.dev.h)
        return loss[:steps]

    def predict(self, X, out=None) -> np.ndarray:
        """Outputs for the rows of X (host memory); out: a float32 array of
        len(X) to write them into (pinned host memory lets the chunks' copies
        overlap the kernel)."""
        X, px = self._f(X)
        if out is None:
            out = np.zeros(len(X), np.float32)
        if out.dtype != np.float32 or out.shape != (len(X),) or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous float32 array of len(X)")
        y = out
        N.check(N.lib().axx_mlp_predict(self.h, px, len(X),
                                        y.ctypes.data_as(C.POINTER(C.c_float))), self.dev.h)
        return y

    def predict_device(self, dX_ptr: int, n: int, dy_ptr: int):
        N.check(N.lib().axx_mlp_predict_device(self.h, C.c_void_p(dX_ptr), n,
                                               C.c_void_p(dy_ptr)), self.dev.h)

    def flops_per_row(self) -> float:
        f = C.c_double()
        N.check(N.lib().axx_mlp_flops_per_row(self.h, C.byref(f)))
        return f.value


def normalise(P: np.ndarray) -> np.ndarray:
    """Parameters -> [-1, 1] per input."""
    lo, hi = RANGES[:, 0], RANGES[:, 1]
    return (2.0 * (np.asarray(P, np.float64) - lo) / (hi - lo) - 1.0).astype(np.float32)


def in_range(P: np.ndarray) -> np.ndarray:
    P = np.asarray(P, np.float64)
    return np.all((P >= RANGES[:, 0] - 1e-9) & (P <= RANGES[:, 1] + 1e-9), axis=1)


def _sequence(G, Delta, delta, omega):
    """PGSE (omega 0) or cosine OGSE with round(omega*delta) periods; G mT/m."""
    if omega <= 0.0:
        return RectGrad(G * 1e-6, delta, Delta - delta)
    n = max(1, int(round(omega * delta * 1e-3)))
    return CosGFunc(G * 1e-6, delta, Delta - delta, n)


def snap_omega(omega, delta):
    """The frequency a sequence actually has (whole periods per lobe)."""
    if omega <= 0.0:
        return 0.0
    n = max(1, int(round(omega * delta * 1e-3)))
    return n / (delta * 1e-3)


@dataclass
class SubstrateDraw:
    mean_radius: float
    shape: float
    fraction: float
    kappa: float
    D_in: float
    D_ex: float


def draw_substrates(n, rng) -> List[SubstrateDraw]:
    out = []
    for _ in range(n):
        v = [rng.uniform(lo, hi) for lo, hi in RANGES[:6]]
        out.append(SubstrateDraw(*v))
    return out


def make_jobs(subs: List[SubstrateDraw], rng, walkers: int, timestep: float,
              n_cyl: int = 400, waves_per_sub: int = 8, g_per_wave: int = 8):
    """One batch job per substrate: `waves_per_sub` waveforms (Delta, delta,
    omega) x `g_per_wave` amplitudes, all read at TE_READ.  Returns (jobs,
    parameter rows)."""
    jobs, rows = [], []
    for k, s in enumerate(subs):
        # radii at the gamma quantiles: the packing's radius distribution is
        # the one its input row names, not a 100-sample draw from it
        radii = gamma_quantile_radii(n_cyl, s.shape, s.mean_radius * 1e-3)
        lat, cyl, f = pack_radii(int(rng.integers(1 << 31)), radii, s.fraction,
                                 D_in=s.D_in * 1e-6, T2_in=T2_IN, D_ex=s.D_ex * 1e-6,
                                 T2_ex=T2_EX, permeability=s.kappa * 1e-3)
        seqs = []
        for _ in range(waves_per_sub):
            Delta = rng.uniform(*RANGES[7])
            delta = min(rng.uniform(*RANGES[8]), Delta - 1.0)
            omega = 0.0 if rng.uniform() < 0.25 else snap_omega(rng.uniform(20.0, RANGES[9][1]), delta)
            if omega > RANGES[9][1]:
                omega = 0.0
            for G in rng.uniform(*RANGES[6], size=g_per_wave):
                seqs.append(_sequence(G, Delta, delta, omega))
                rows.append([s.mean_radius, s.shape, f, s.kappa, s.D_in, s.D_ex, G, Delta,
                             delta, omega])
        steps = int(math.ceil(TE_READ / timestep)) + 1
        jobs.append(Job(cyl, seqs, walkers, steps, timestep, int(rng.integers(1 << 31)),
                        lattice=lat, relaxation=True, permeable=s.kappa > 0))
    return jobs, np.array(rows)


# Dense packings hold narrow channels between neighbouring cylinders where a
# rare move reflects more than 1024 times; such moves end at their last
# reflection.  Training data accepts them up to this fraction of all moves.
MAX_CAP_FRACTION = 1e-8


def simulate(jobs: List[Job], device: Device = None, chunk: int = 64,
             counts: Optional[Dict[str, int]] = None, method: str = "auto",
             stderr: Optional[list] = None) -> np.ndarray:
    """Normalised signals |M|/N of every sequence of every job (plain MC).
    method "batch": persistent batched launches of `chunk` jobs; "plans": one
    walk per job (axx_run_lattice: the single-job kernels, faster for large
    dense packings); "auto": plans when a job holds more than 100 bases.
    `counts`, when given, accumulates walker_steps and cap_hits; `stderr`,
    when given, receives each signal's standard error."""
    from .acquisition import run_lattice
    if method == "auto":
        method = "plans" if jobs and max(len(j.basis) for j in jobs) > 100 else "batch"
    out = []

    def tally(r):
        out.append(r.signal)
        if stderr is not None:
            stderr.append(r.stderr)
        if counts is not None:
            counts["walker_steps"] = counts.get("walker_steps", 0) + int(r.walker_steps)
            counts["cap_hits"] = counts.get("cap_hits", 0) + int(r.cap_hits)

    if method == "plans":
        for j in jobs:
            r = run_lattice(j.lattice, j.basis, j.seqs, j.num_walkers, j.steps, j.timestep,
                            j.seed, relaxation=j.relaxation, permeable=j.permeable,
                            device=device, allow_cap=True)
            if r.cap_hits > MAX_CAP_FRACTION * r.walker_steps:
                raise N.ReflectionCapError(N.AXX_ERR_REFLECTION_CAP,
                                           "%d reflection-cap moves" % r.cap_hits)
            tally(r)
    else:
        for i in range(0, len(jobs), chunk):
            for r in run_batch(jobs[i:i + chunk], device=device,
                               max_cap_fraction=MAX_CAP_FRACTION):
                tally(r)
    return np.concatenate(out) if out else np.zeros(0)


def generate(n_sub: int, seed: int, walkers: int = 262144, timestep: float = 0.001,
             n_cyl: int = 400, device: Device = None, counts: Optional[Dict[str, int]] = None,
             stderr: Optional[list] = None):
    """(parameters [n][10], signals [n]) from n_sub substrates x 64 sequences:
    by default the 400-cylinder gamma packings at dt 1 us of the permeable
    benchmark substrate, 262,144 walkers per packing."""
    rng = np.random.default_rng(seed)
    subs = draw_substrates(n_sub, rng)
    jobs, P = make_jobs(subs, rng, walkers, timestep, n_cyl)
    S = simulate(jobs, device=device, counts=counts, stderr=stderr)
    return P, S


WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "surrogate_400cyl.npz")


def save(mlp: MLP, path: str, heldout: Optional[dict] = None, meta: Optional[dict] = None):
    """The trained parameters (FP32, axx_mlp layout), with the held-out pairs
    and their Monte Carlo truth when given."""
    d = {"params": mlp.get_params(), "shape": np.array([mlp.in_dim, mlp.width, mlp.depth])}
    for k, v in (heldout or {}).items():
        d["heldout_" + k] = np.asarray(v)
    if meta:
        d["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(path, **d)


def load(path: str = WEIGHTS, device: Device = None):
    """(MLP with the saved parameters, held-out dict, meta dict)."""
    z = np.load(path)
    in_dim, width, depth = (int(x) for x in z["shape"])
    mlp = MLP(in_dim, width, depth, device=device)
    mlp.set_params(z["params"])
    held = {k[len("heldout_"):]: z[k] for k in z.files if k.startswith("heldout_")}
    meta = json.loads(str(z["meta"])) if "meta" in z.files else {}
    return mlp, held, meta


class Surrogate:
    """Trained network plus the Monte Carlo fallback for out-of-range queries."""

    def __init__(self, mlp: MLP):
        self.mlp = mlp

    # learning-rate schedule: fraction of the steps and lr multiplier
    SCHEDULE = ((0.5, 1.0), (0.25, 0.3), (0.15, 0.1), (0.1, 0.03))

    @classmethod
    def fit(cls, P, S, steps=4000, batch=4096, lr=1e-3, seed=0, device=None):
        """Adam on the normalised rows, with the learning rate stepped down
        over the run (SCHEDULE); Adam's moments carry across the stages."""
        mlp = MLP(seed=seed, device=device)
        X, y = normalise(P), np.asarray(S, np.float32)
        losses, done = [], 0
        for k, (frac, mult) in enumerate(cls.SCHEDULE):
            n = steps - done if k == len(cls.SCHEDULE) - 1 else int(round(frac * steps))
            if n <= 0:
                continue
            losses.append(mlp.train(X, y, batch=batch, steps=n, lr=lr * mult, seed=seed + k))
            done += n
        s = cls(mlp)
        s.loss = np.concatenate(losses)
        return s

    def predict(self, P, fallback_walkers: int = 262144, timestep: float = 0.001,
                device: Device = None, n_cyl: int = 400) -> Tuple[np.ndarray, np.ndarray]:
        """Signals for parameter rows; rows outside the training ranges are
        simulated.  Returns (signals, used_fallback mask)."""
        P = np.asarray(P, np.float64)
        ok = in_range(P)
        out = np.zeros(len(P))
        if ok.any():
            out[ok] = self.mlp.predict(normalise(P[ok]))
        if (~ok).any():
            rng = np.random.default_rng(0)
            for i in np.nonzero(~ok)[0]:
                p = P[i]
                sub = SubstrateDraw(*p[:6])
                jobs, _ = make_jobs([sub], rng, fallback_walkers, timestep, n_cyl=n_cyl,
                                    waves_per_sub=1, g_per_wave=1)
                jobs[0].seqs = [_sequence(p[6], p[7], p[8], p[9])]
                out[i] = simulate(jobs, device=device)[0]
        return out, ~ok
