"""Monte Carlo intracellular volume fraction (the reference's calcf /
kernelCalcf, src/util/calcf.cuh:1-38).

The reference's own calcf does not build as written (it passes an undeclared
`maxthreads`) and divides two ints, so the oracle restates the algorithm it
describes: point i = words 1..3 of stream (seed, i) scaled by the cell
(Lattice::initializeUniformly), counted when Lattice::inRegion is > 0."""
import math

import pytest

import cases

SUBSTRATES = [
    ("hex", lambda: cases.hex_cylinders(r_um=2.5, f=0.6), 0.6),
    ("cyl", lambda: cases.one_cylinder(), math.pi * 25.0 / 144.0),
    ("spheres", lambda: cases.sphere_lattice(), 2 * (4.0 / 3.0) * math.pi * 27.0 / 1000.0),
]


@pytest.mark.parametrize("name,make,f", SUBSTRATES, ids=[s[0] for s in SUBSTRATES])
def test_oracle_fraction_against_geometry(orc, name, make, f):
    lat, bases = make()
    n = 200000
    ref = orc.volume_fraction(lat, bases, n, 7, orc.REF64, nthreads=8)
    k32 = orc.volume_fraction(lat, bases, n, 7, orc.KERN32, nthreads=8)
    sd = math.sqrt(n * f * (1 - f))
    assert abs(ref - n * f) < 4 * sd, (ref / n, f)
    # FP32 positions and the instance lookup differ from FP64 only on rounding ties
    assert abs(ref - k32) <= 2


@pytest.mark.gpu
@pytest.mark.parametrize("name,make,f", SUBSTRATES + [("gamma", cases.gamma_packing, 0.6)],
                         ids=[s[0] for s in SUBSTRATES] + ["gamma"])
def test_gpu_fraction_bit_exact(dev, orc, name, make, f):
    import axonexa_gb300 as A
    from test_gpu_parity import to_product
    lat, bases = make()
    L, B, _ = to_product(lat, bases)
    n = 1 << 20
    frac, count = A.volume_fraction(L, B, n, 11, device=dev)
    assert count == orc.volume_fraction(lat, bases, n, 11, orc.KERN32, nthreads=8)
    assert frac == count / n
    assert abs(count - n * f) < 4 * math.sqrt(n * f * (1 - f)), (frac, f)
