"""The C++ adapter (include/axx_acquisition.hpp) on the GPU: the reference-
style main of tests/cpp/drive.hpp, built against the adapter, gives the same
signals as axx_run_lattice on the same inputs, bit for bit, and the ADC of
phaseAcquisition::calcADC over them."""
import subprocess

import numpy as np
import pytest

import axonexa_gb300 as A
from test_acquisition_adapter import build_adapter_main

pytestmark = pytest.mark.gpu


def test_adapter_main_matches_run_lattice():
    exe = build_adapter_main()
    particles, steps, dt, seed = 65536, 5000, 0.002, 7
    r = subprocess.run([exe, str(particles), str(steps), repr(dt), str(seed)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    vals = np.array([float(v) for v in r.stdout.split()])
    sig, adc = vals[:-1], vals[-1]
    cell, radius = 0.012, 0.005
    lat = A.Lattice(cell, cell, cell, 60.0, 0.0, 2e-6, 1)
    cyl = [A.Cylinder_XY(cell / 2, cell / 2, radius, 80.0, 0.0, 2e-6, 1, 0.0)]
    seqs = [A.RectGrad(i * 25e-6, 10.0, 30.0) for i in range(8)]
    res = A.run_lattice(lat, cyl, seqs, particles, steps, dt, seed, relaxation=True)
    want = np.sqrt(res.mx * res.mx + res.my * res.my)
    assert np.array_equal(sig, want)
    pa = A.phaseAcquisition(8, steps, particles, seed)
    for q in seqs:
        pa.addMeasurement(q)
    pa.mx, pa.my = list(res.mx), list(res.my)
    pa.calcADC()
    assert adc == pa.getADC()
    # restricted diffusion: the apparent D is below the free D
    assert 0.0 < adc < 2e-6
