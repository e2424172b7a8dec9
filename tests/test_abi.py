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
