"""The acquisition post-processing and the C++ adapter against the reference.

* linear_regression and phaseAcquisition::calcADC / getSignal
  (src/util/misc.cuh:41-59, src/acquisition/phaseAcquisition.cuh:46-77),
  compiled from the reference's own headers (oracle/_ref/libaxxref_acq.so),
  against this repository's Python mirror (axonexa_gb300/acquisition.py) and
  C++ adapter (include/axx_acquisition.hpp), bit for bit.
* tests/cpp/drive.hpp, a reference-style main, compiles against the
  reference's own headers (nvcc, compile only) and against the adapter (g++).
The adapter's GPU run is in test_gpu_adapter.py.
"""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

import axonexa_gb300 as A
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CPP = os.path.join(ROOT, "tests", "cpp")
INC = os.path.join(ROOT, "include")
LIBDIR = os.path.join(ROOT, "axonexa_gb300")


def _ref():
    L = O.reflib_acq()
    if L is None:
        pytest.skip("the reference was not built here (oracle/_ref)")
    return L


def _dp(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(C.POINTER(C.c_double))


def _cases():
    rng = np.random.default_rng(11)
    out = []
    for kind, d, sp, per in ((0, 10.0, 30.0, 0), (1, 20.0, 5.0, 2), (2, 20.0, 5.0, 4)):
        n, points = 9, 3
        G = np.linspace(0.0, 2e-4, n)
        q = {0: A.RectGrad(1.0, d, sp), 1: A.CosGFunc(1.0, d, sp, per),
             2: A.SinGFunc(1.0, d, sp, per)}[kind]
        b = []
        for g in G:
            q.G = float(g)
            b.append(q.getB())
        b = np.array(b)
        # sums of N walkers with a decay near exp(-b D) and some noise
        N = 65536.0
        s = np.exp(-b * 1.7e-6)[None, :] * (1 + 1e-3 * rng.standard_normal((points, n)))
        ph = rng.uniform(-0.05, 0.05, (points, n))
        mx, my = N * s * np.cos(ph), N * s * np.sin(ph)
        out.append((kind, d, sp, per, G, mx, my))
    return out


def test_linear_regression_matches_reference():
    L = _ref()
    rng = np.random.default_rng(3)
    for n in (2, 5, 33):
        x, y = rng.uniform(0, 3e3, n), rng.normal(size=n)
        ref = L.ref_linear_regression(_dp(y), _dp(x), n)
        assert A.acquisition.linear_regression(list(y), list(x)) == ref


@pytest.mark.parametrize("case", range(3))
def test_calc_adc_matches_reference(case):
    L = _ref()
    kind, d, sp, per, G, mx, my = _cases()[case]
    n, points = len(G), mx.shape[0]
    adc, adcms, sig = np.zeros(points), np.zeros(points), np.zeros(n)
    assert L.ref_calc_adc(kind, n, _dp(G), C.c_double(d), C.c_double(sp), per, points, _dp(mx),
                          _dp(my), _dp(adc), _dp(adcms), _dp(sig)) == 0
    ctor = {0: lambda g: A.RectGrad(g, d, sp), 1: lambda g: A.CosGFunc(g, d, sp, per),
            2: lambda g: A.SinGFunc(g, d, sp, per)}[kind]
    pa = A.phaseAcquisition(n, 10, 1, 0)
    for g in G:
        pa.addMeasurement(ctor(float(g)))
    for p in range(points):
        pa.mx, pa.my = list(mx[p]), list(my[p])
        pa.calcADC()
        assert pa.getADC() == adc[p] and pa.getADCMeanSquare() == adcms[p]
    assert [pa.getSignal(i) for i in range(n)] == list(sig)
    # the C++ adapter on the same sums
    exe = _adapter_adc()
    inp = "%d %d %d %r %r %d\n" % (kind, n, points, d, sp, per)
    inp += " ".join(repr(float(v)) for v in G) + "\n"
    inp += " ".join(repr(float(v)) for v in mx.ravel()) + "\n"
    inp += " ".join(repr(float(v)) for v in my.ravel()) + "\n"
    r = subprocess.run([exe], input=inp, capture_output=True, text=True, check=True)
    vals = [float(v) for v in r.stdout.split()]
    got = np.array(vals[:2 * points]).reshape(points, 2)
    assert np.array_equal(got[:, 0], adc) and np.array_equal(got[:, 1], adcms)
    assert np.array_equal(np.array(vals[2 * points:]), sig)


_built = {}


def _gxx():
    g = shutil.which("g++")
    if not g:
        pytest.skip("g++ not found")
    return g


def _adapter_adc():
    if "adc" not in _built:
        out = os.path.join(LIBDIR, "_build", "adapter_adc")
        os.makedirs(os.path.dirname(out), exist_ok=True)
        # no contraction into fused multiply-adds (aarch64 GCC fuses by
        # default): the reference's code is built the same way
        subprocess.run([_gxx(), "-std=c++17", "-O2", "-ffp-contract=off", "-I", INC,
                        os.path.join(CPP, "adapter_adc.cpp"), "-L", LIBDIR, "-laxx",
                        "-Wl,-rpath," + LIBDIR, "-o", out], check=True)
        _built["adc"] = out
    return _built["adc"]


def build_adapter_main():
    """tests/cpp/adapter_main.cpp compiled against the adapter and libaxx.so."""
    out = os.path.join(LIBDIR, "_build", "adapter_main")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    subprocess.run([_gxx(), "-std=c++17", "-O2", "-ffp-contract=off", "-Wall", "-Werror",
                    "-I", INC, "-I", CPP,
                    os.path.join(CPP, "adapter_main.cpp"), "-L", LIBDIR, "-laxx",
                    "-Wl,-rpath," + LIBDIR, "-o", out], check=True)
    return out


def test_reference_style_main_builds_against_the_adapter():
    assert os.path.exists(build_adapter_main())


def test_reference_style_main_compiles_against_the_reference():
    src = O.reference_src()
    if src is None:
        pytest.skip("no reference source tree here")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    inc = []
    for d in ("util", "params", "substrate", "primitives", "kernels", "functors", "bloch",
              "acquisition"):
        inc += ["-I", os.path.join(src, "src", d)]
    out = os.path.join(LIBDIR, "_build", "reference_api_check.o")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    r = subprocess.run([nvcc, "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a"] + inc +
                       ["-I", CPP, "-c", os.path.join(CPP, "reference_api_check.cu"), "-o", out],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
