"""The C ABI library loads, exports every declared entry point, and validates
its inputs without a GPU."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(axx_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from axonexa_gb300 import _native as N
    return N.lib()


def test_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s


def test_binding_covers_header():
    from axonexa_gb300 import _native as N
    assert set(declared_symbols()) <= set(N.exported_symbols())


def test_abi_version(lib):
    assert lib.axx_abi_version() == 1


def test_status_strings(lib):
    assert lib.axx_status_string(0) == b"ok"
    assert lib.axx_status_string(3) == b"reflection cap hit"


def test_create_rejects_null_and_reports_no_device(lib):
    assert lib.axx_create(None, 0) == 1
    h = C.c_void_p()
    rc = lib.axx_create(C.byref(h), 0)
    assert rc in (0, 5)
    if rc == 0:
        lib.axx_destroy(h)


def test_sequence_helpers_match_oracle(orc):
    import cases
    import axonexa_gb300 as A
    from axonexa_gb300 import _native as N
    for q in cases.seq_mix() + [cases.cos_ogse(70, 3, kind=4), cases.pgse(55, 7.0, 19.0)]:
        rec = N.SequenceRec(q.kind, q.num_periods, q.G, q.duration, q.spacing, q.gx, q.gy, q.gz)
        b = C.c_double()
        assert N.lib().axx_bvalue(C.byref(rec), 0.0, C.byref(b)) == 0
        assert b.value == orc.bvalue(q)
        ts = [0.0, 1.3, 9.99, 10.0, 25.0, 40.0, 45.5, 49.999, 50.0, 61.0]
        t = (C.c_double * len(ts))(*ts)
        out = (C.c_double * (3 * len(ts)))()
        assert N.lib().axx_gradient_eval(C.byref(rec), t, len(ts), out) == 0
        for i, tt in enumerate(ts):
            want = orc.gradient(q, tt)
            got = list(out[3 * i:3 * i + 3])
            for a, w in zip(got, want):
                assert abs(a - w) <= 1e-15 * max(1.0, abs(w)) + 1e-30, (q.kind, tt, got, want)


def test_bvalue_closed_forms():
    import axonexa_gb300 as A
    g, d, sp = 2e-7, 10.0, 30.0
    # PGSE: b = gamma^2 G^2 delta^2 (Delta - delta/3)
    assert abs(A.RectGrad(g, d, sp).getB() - A.GAMMA ** 2 * g * g * d * d * (d + sp - d / 3)) < 1e-9
    # cosine OGSE: b = gamma^2 G^2 delta^3 / (4 pi^2 N^2)
    n = 2
    want = A.GAMMA ** 2 * g * g * d ** 3 / (4 * A.PI ** 2 * n * n)
    assert abs(A.CosGFunc(g, d, sp, n).getB() - want) < 1e-9 * want


def test_gamma_packing_statistics():
    """Packing: achieved fraction, periodic minimum gap, radius distribution,
    images of edge-crossing cylinders (RPSLatticeInitializer semantics)."""
    import numpy as np
    import axonexa_gb300 as A
    lat, cyl, f = A.rps_gamma_pack(3, 400, 5.0, 2.5e-3, 0.6, D_in=1.7e-6, T2_in=80,
                                   D_ex=2e-6, T2_ex=60, permeability=2e-5)
    L = lat.a
    orig = {}
    for c in cyl:
        orig.setdefault(c.region, c)
    assert len(orig) == 400
    # the reference's initializer default-constructs its cylinders: cylEPS 1e-14
    assert all(c.eps == 1e-14 for c in cyl)
    r = np.array([orig[k].radius for k in sorted(orig)])
    x = np.array([orig[k].centerX for k in sorted(orig)])
    y = np.array([orig[k].centerY for k in sorted(orig)])
    assert abs(np.pi * (r ** 2).sum() / L ** 2 - 0.6) < 1e-9 and abs(f - 0.6) < 1e-9
    # gamma(k=5, mean 2.5 um): mean and coefficient of variation 1/sqrt(5)
    assert abs(r.mean() - 2.5e-3) < 0.15e-3
    assert abs(r.std() / r.mean() - 1 / np.sqrt(5)) < 0.06
    dx = x[:, None] - x[None, :]
    dy = y[:, None] - y[None, :]
    dx -= L * np.round(dx / L)
    dy -= L * np.round(dy / L)
    d = np.hypot(dx, dy) + np.eye(400) * 1e9
    assert np.all(d >= (r[:, None] + r[None, :]) * 1.0099)
    # every extra record is a periodic image of its original
    for c in cyl[400:]:
        o = orig[c.region]
        sx, sy = (c.centerX - o.centerX) / L, (c.centerY - o.centerY) / L
        assert abs(sx - round(sx)) < 1e-9 and abs(sy - round(sy)) < 1e-9 and (sx, sy) != (0, 0)


def test_pack_given_radii():
    """axx_substrate_pack: caller's radii (gamma mid-quantiles), sorted into
    regions 1..n, exact area fraction, periodic gap kept."""
    import numpy as np
    import axonexa_gb300 as A
    r = A.gamma_quantile_radii(100, 4.0, 2.0e-3)
    assert abs(r.mean() - 2.0e-3) < 0.02e-3  # quantile mean -> the law's mean
    assert np.all(np.diff(r) > 0)
    lat, cyl, f = A.pack_radii(7, r[::-1], 0.62, D_in=1.7e-6, T2_in=80, D_ex=2e-6, T2_ex=60)
    L = lat.a
    orig = {}
    for c in cyl:
        orig.setdefault(c.region, c)
    got = np.array([orig[k].radius for k in range(1, 101)])
    assert np.array_equal(got, r)
    assert abs(np.pi * (r ** 2).sum() / L ** 2 - 0.62) < 1e-12 and abs(f - 0.62) < 1e-12
    x = np.array([orig[k].centerX for k in range(1, 101)])
    y = np.array([orig[k].centerY for k in range(1, 101)])
    dx = x[:, None] - x[None, :]
    dy = y[:, None] - y[None, :]
    dx -= L * np.round(dx / L)
    dy -= L * np.round(dy / L)
    d = np.hypot(dx, dy) + np.eye(100) * 1e9
    assert np.all(d >= (r[:, None] + r[None, :]) * 1.0099)
    with pytest.raises(A._native.AxxError):
        A.pack_radii(7, np.array([1e-3, -1e-3]), 0.5, D_in=1e-6, T2_in=1, D_ex=1e-6, T2_ex=1)
