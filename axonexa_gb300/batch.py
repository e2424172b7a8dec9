"""Batched acquisitions: many substrates and sequence sets, uneven walker
counts, one persistent launch replayed from a CUDA graph (axx_batch_*)."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np

from . import _native as N
from .acquisition import Device, Lattice, RunResult, _params, default_device, run_flags


@dataclass
class Job:
    """One acquisition: a lattice substrate (lattice given) or a single pore
    (lattice None, basis = [pore])."""
    basis: Sequence
    seqs: Sequence
    num_walkers: int
    steps: int
    timestep: float
    seed: int
    lattice: Optional[Lattice] = None
    relaxation: bool = False
    permeable: bool = False
    walker_offset: int = 0


class _Records:
    """Keeps the ctypes arrays of a job list alive while the library uses them."""

    def __init__(self, jobs: List[Job]):
        self.keep = []
        arr = (N.Job * len(jobs))()
        for i, j in enumerate(jobs):
            b = N.array_of(N.Basis, [x.record() for x in j.basis])
            s = N.array_of(N.SequenceRec, [q.record() for q in j.seqs])
            self.keep += [b, s]
            mode = 0 if j.lattice is not None else 1
            lat = j.lattice.record() if j.lattice is not None else N.LatticeRec(1, 1, 1, 0, 0, 0)
            flags = run_flags(True, j.relaxation, j.permeable)
            p = _params(j.num_walkers, j.steps, j.seed, j.timestep, flags, offset=j.walker_offset)
            arr[i] = N.Job(mode, lat, C.cast(b, C.POINTER(N.Basis)), len(j.basis),
                           C.cast(s, C.POINTER(N.SequenceRec)), len(j.seqs), p)
        self.arr = arr
        self.n = len(jobs)
        self.nseq = [len(j.seqs) for j in jobs]
        self.nw = [int(j.num_walkers) for j in jobs]


class Batch:
    """A planned batch (axx_batch_create): launch() enqueues one execution,
    read() returns one RunResult per job."""

    def __init__(self, jobs: List[Job], tile: int = 0, blocks_per_sm: int = 0,
                 use_graph: bool = True, device: Device = None):
        self.dev = device or default_device()
        self.rec = _Records(jobs)
        h = C.c_void_p()
        opt = N.BatchOptions(int(tile), int(blocks_per_sm), 1 if use_graph else 0)
        N.check(N.lib().axx_batch_create(self.dev.h, self.rec.arr, self.rec.n, C.byref(opt),
                                         C.byref(h)), self.dev.h)
        self.h = h
        self.dev.adopt(self)

    def launch(self):
        N.check(N.lib().axx_batch_launch(self.h), self.dev.h)

    def info(self):
        it, tile, bps, kl = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        ws = C.c_int64()
        N.check(N.lib().axx_batch_info(self.h, C.byref(it), C.byref(tile), C.byref(bps),
                                       C.byref(kl), C.byref(ws)))
        return dict(items=it.value, tile=tile.value, blocks_per_sm=bps.value,
                    kernel_launches=kl.value, walker_steps=ws.value)

    def read(self, max_cap_fraction: float = 0.0) -> List[RunResult]:
        """Signals of every job.  Moves that hit the reflection cap raise
        ReflectionCapError unless they are at most `max_cap_fraction` of the
        batch's walker-steps (each result's `cap_hits` holds its count)."""
        tot = sum(self.rec.nseq)
        mx, my = np.zeros(max(tot, 1)), np.zeros(max(tot, 1))
        bufs = [[np.zeros(max(m, 1)) for _ in range(3)] for m in self.rec.nseq]
        st = (N.Stats * self.rec.n)()
        for j, b in enumerate(bufs):
            p = [x.ctypes.data_as(C.POINTER(C.c_double)) for x in b]
            st[j] = N.Stats(p[0], p[1], p[2], 0, 0, 0)
        status = N.lib().axx_batch_read(self.h, mx.ctypes.data_as(C.POINTER(C.c_double)),
                                        my.ctypes.data_as(C.POINTER(C.c_double)), st)
        if status == N.AXX_ERR_REFLECTION_CAP and max_cap_fraction > 0.0:
            caps = sum(st[j].reflection_cap_hits for j in range(self.rec.n))
            steps = sum(st[j].walker_steps for j in range(self.rec.n))
            if caps <= max_cap_fraction * steps:
                status = 0
        N.check(status, self.dev.h)
        out, o = [], 0
        for j, m in enumerate(self.rec.nseq):
            b = bufs[j]
            out.append(RunResult(mx[o:o + m].copy(), my[o:o + m].copy(), b[0][:m], b[1][:m],
                                 b[2][:m], st[j].reflection_cap_hits, st[j].walker_steps,
                                 self.rec.nw[j], st[j].boundary_hits))
            o += m
        return out

    def close(self):
        if getattr(self, "h", None):
            N.lib().axx_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_batch(jobs: List[Job], max_cap_fraction: float = 0.0, **kw) -> List[RunResult]:
    b = Batch(jobs, **kw)
    try:
        b.launch()
        return b.read(max_cap_fraction)
    finally:
        b.close()


def autotune(jobs: List[Job], probe_steps: int = 300, device: Device = None):
    """The project's autotuner (axx_autotune_batch): best (tile, blocks per SM)."""
    dev = device or default_device()
    rec = _Records(jobs)
    best = N.BatchOptions(0, 0, 0)
    ms = C.c_double()
    N.check(N.lib().axx_autotune_batch(dev.h, rec.arr, rec.n, probe_steps, C.byref(best),
                                       C.byref(ms)), dev.h)
    return dict(tile=best.tile, blocks_per_sm=best.blocks_per_sm, ms=ms.value)
