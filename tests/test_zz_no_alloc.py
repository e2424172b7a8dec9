"""axx_run_lattice_noalloc: the lattice walk for callers that cannot allocate
GPU memory.

Callers that cannot call cudaMalloc when they run a walk -- code whose GPU
memory is owned by a pool or a fixed budget, frameworks that forbid device
allocation after start-up, threads that must not trigger the device-wide
synchronisation cudaMalloc/cudaFree can cause -- use this entry point.  It
runs the same kernels as axx_run_lattice but keeps every device-side buffer in
a static array compiled into the library, so it must give the same signals as
the allocating call, call after call (the array is reused and keeps the
previous call's contents), and it must refuse walks that do not fit.

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _records():
    import axonexa_gb300 as A
    from axonexa_gb300 import _native as N
    c, r = 0.012, 0.005
    lat = A.Lattice(c, c, c, 60.0, 0.0, 2e-6, 1).record()
    basis = N.array_of(N.Basis, [A.Cylinder_XY(c / 2, c / 2, r, 80.0, 0.0, 2e-6, 1, 0.0).record()])
    seqs = [A.RectGrad(g * 1e-6, 10.0, 30.0) for g in (0.0, 80.0, 160.0)] + \
        [A.CosGFunc(100e-6, 10.0, 10.0, 2, (0.6, 0.8, 0.0))]
    srec = N.array_of(N.SequenceRec, [q.record() for q in seqs])
    return lat, basis, srec, len(seqs)


def _call(fn, ctx, lat, basis, srec, m, params):
    from axonexa_gb300 import _native as N
    out = [np.zeros(m) for _ in range(5)]
    ptr = [o.ctypes.data_as(C.POINTER(C.c_double)) for o in out]
    st = N.Stats(ptr[2], ptr[3], ptr[4], 0, 0, 0)
    rc = fn(ctx, C.byref(lat), basis, 1, srec, m, C.byref(params), ptr[0], ptr[1], C.byref(st))
    N.check(rc, ctx)
    return out, st


def test_noalloc_matches_allocating_call_twice_in_a_row():
    import axonexa_gb300 as A
    from axonexa_gb300 import _native as N
    dev = A.default_device()
    L = N.lib()
    lat, basis, srec, m = _records()
    n = 20000
    params = N.RunParams(n, 3000, 0, 0, N.FLAG_RELAXATION, 4242, 0.002, 0.0, 0)
    want, st_w = _call(L.axx_run_lattice, dev.h, lat, basis, srec, m, params)
    for _ in range(2):
        got, st_g = _call(L.axx_run_lattice_noalloc, dev.h, lat, basis, srec, m, params)
        # the same kernels on the same grid: the same bits
        for a, b in zip(got, want):
            np.testing.assert_array_equal(a, b)
        assert st_g.walker_steps == st_w.walker_steps
        assert st_g.boundary_hits == st_w.boundary_hits
        assert st_g.reflection_cap_hits == 0


def _seqs_along(waves, dirs):
    """One sequence per (waveform, direction): len(waves) x 3 phase channels
    when the directions span space."""
    import axonexa_gb300 as A
    out = []
    for k, (d, sp, n) in enumerate(waves):
        for j, u in enumerate(dirs):
            g = (40.0 + 10 * j) * 1e-6
            out.append(A.CosGFunc(g, d, sp, n, tuple(u)) if n else A.RectGrad(g, d, sp, None))
            if not n:
                out[-1].ghat = A.acquisition.Vector3(*u)
    return out


@pytest.mark.parametrize("nwaves", [3, 5])
def test_noalloc_many_channels_match_allocating_call(nwaves):
    """9 and 15 phase channels (the 12- and 16-channel kernels), twice in a
    row, bit for bit."""
    import axonexa_gb300 as A
    from axonexa_gb300 import _native as N
    dev = A.default_device()
    L = N.lib()
    lat, basis, _, _ = _records()
    rng = np.random.default_rng(nwaves)
    dirs = rng.normal(size=(4, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    waves = [(10.0, 2.0, 0), (6.0, 2.0, 1), (6.0, 2.0, 2), (6.0, 2.0, 3), (4.0, 4.0, 2)][:nwaves]
    seqs = _seqs_along(waves, dirs)
    srec = N.array_of(N.SequenceRec, [q.record() for q in seqs])
    m = len(seqs)
    n = 12000
    params = N.RunParams(n, 1500, 0, 0, N.FLAG_RELAXATION, 99, 0.002, 0.0, 0)
    want, _ = _call(L.axx_run_lattice, dev.h, lat, basis, srec, m, params)
    for _ in range(2):
        got, _ = _call(L.axx_run_lattice_noalloc, dev.h, lat, basis, srec, m, params)
        for a, b in zip(got, want):
            np.testing.assert_array_equal(a, b)


def test_noalloc_shrunk_grid_matches_allocating_call():
    """256 sequences of 8 waveforms over 60,000 steps and 120,000 walkers: the
    waveform tables (1.9 MB) leave the array room for the FP64 partials of
    about 640 blocks of 256 sequences, fewer than the full grid's 760, so the
    grid shrinks; the sums then differ from the allocating call's only by the
    grouping of the per-block partials."""
    import axonexa_gb300 as A
    from axonexa_gb300 import _native as N
    dev = A.default_device()
    L = N.lib()
    lat, basis, _, _ = _records()
    seqs = [A.RectGrad(g * 1e-6, 4.0 + k, 20.0) for k in range(8)
            for g in np.linspace(0.0, 200.0, 32)]
    srec = N.array_of(N.SequenceRec, [q.record() for q in seqs])
    m = len(seqs)
    n = 120000
    params = N.RunParams(n, 60000, 0, 0, N.FLAG_RELAXATION, 5, 0.002, 0.0, 0)
    want, _ = _call(L.axx_run_lattice, dev.h, lat, basis, srec, m, params)
    for _ in range(2):
        got, _ = _call(L.axx_run_lattice_noalloc, dev.h, lat, basis, srec, m, params)
        for a, b in zip(got, want):
            np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-9)


def test_noalloc_refuses_walks_that_do_not_fit():
    import axonexa_gb300 as A
    from axonexa_gb300 import _native as N
    dev = A.default_device()
    lat, basis, _, _ = _records()
    # 16 distinct waveforms x 140,000 steps of FP32 tables exceed the 8 MiB array
    seqs = [A.RectGrad(1e-4, 1.0 + k, 5.0) for k in range(16)]
    srec = N.array_of(N.SequenceRec, [q.record() for q in seqs])
    params = N.RunParams(64, 140000, 0, 0, 0, 1, 0.002, 0.0, 0)
    with pytest.raises(N.AxxError) as e:
        _call(N.lib().axx_run_lattice_noalloc, dev.h, lat, basis, srec, len(seqs), params)
    assert e.value.status == 1
    assert "no-allocation scratch" in str(e.value)


def test_noalloc_compartment_sums_match_allocating_call():
    import axonexa_gb300 as A
    from axonexa_gb300 import _native as N
    dev = A.default_device()
    L = N.lib()
    lat, basis, srec, m = _records()
    n = 20000
    params = N.RunParams(n, 2000, 0, 0, N.FLAG_RELAXATION | N.FLAG_COMPARTMENTS, 77, 0.002, 0.0,
                         0)
    res = []
    for fn in (L.axx_run_lattice, L.axx_run_lattice_noalloc):
        out = [np.zeros(m) for _ in range(4)]
        ptr = [o.ctypes.data_as(C.POINTER(C.c_double)) for o in out]
        st = N.Stats(None, None, None, 0, 0, 0, ptr[2], ptr[3], 0)
        N.check(fn(dev.h, C.byref(lat), basis, 1, srec, m, C.byref(params), ptr[0], ptr[1],
                   C.byref(st)), dev.h)
        res.append((out, st.walkers_in))
    (a, na), (b, nb) = res
    assert na == nb and 0 < na < n
    for x, y in zip(a, b):
        np.testing.assert_allclose(x, y, rtol=0, atol=1e-9 * n)
