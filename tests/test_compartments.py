"""Start-compartment sums (AXX_FLAG_COMPARTMENTS): the signal of the walkers
that start inside a basis (Lattice::inRegion != 0), beside the whole-substrate
sums of the reference's output (phaseAcquisitionStream.cuh:185-189)."""
import math

import numpy as np
import pytest

import cases

FLAG = 64


def test_oracle_compartment_rows(orc):
    lat, cyl = cases.one_cylinder()
    seqs = [cases.pgse(0)] + cases.seq_mix()[1:4]
    n = 2000
    for mode in (orc.REF64, orc.KERN64):
        whole, _, _ = orc.walk(lat, cyl, seqs, cases.params(n, 400, 3, flags=1), mode, nthreads=4)
        both, _, _ = orc.walk(lat, cyl, seqs, cases.params(n, 400, 3, flags=1 | FLAG), mode,
                              nthreads=4)
        M = len(seqs)
        assert both.shape == (2 * M, 5)
        np.testing.assert_array_equal(both[:M], whole)
        # all walkers started in the cylinder: the rows agree with the whole
        inr, _, _ = orc.walk(lat, cyl, seqs, cases.params(n, 400, 3, flags=FLAG, init_mode=1,
                                                           init_arg=1), mode, nthreads=4)
        np.testing.assert_array_equal(inr[M:], inr[:M])
        # none did: zero rows
        out, _, _ = orc.walk(lat, cyl, seqs, cases.params(n, 400, 3, flags=FLAG, init_mode=1,
                                                           init_arg=0), mode, nthreads=4)
        assert np.all(out[M:] == 0.0)
    # G = 0 without relaxation: the x sum counts the walkers that start inside,
    # a fraction pi r^2 / c^2 of them
    s, _, _ = orc.walk(lat, cyl, [cases.pgse(0)], cases.params(20000, 3, 9, flags=FLAG),
                       orc.REF64, nthreads=4)
    f = math.pi * 25.0 / 144.0
    assert abs(s[1, 0] - 20000 * f) < 4 * math.sqrt(20000 * f * (1 - f))


@pytest.mark.gpu
def test_gpu_compartment_sums(dev, orc):
    import axonexa_gb300 as A
    from test_gpu_parity import to_product
    for lat, bases, flags in ((*cases.one_cylinder(), 1),
                              (*cases.hex_cylinders(kappa=2e-5), 3),
                              (*cases.parallel_plates(with_cylinder=True), 3)):
        seqs = [cases.pgse(0)] + cases.seq_mix()[1:4]
        L, B, S = to_product(lat, bases, seqs)
        n, steps = 4096, 1500
        kw = dict(relaxation=bool(flags & 1), permeable=bool(flags & 2), device=dev)
        r = A.run_lattice(L, B, S, n, steps, 0.002, 31, compartments=True, **kw)
        plain = A.run_lattice(L, B, S, n, steps, 0.002, 31, **kw)
        np.testing.assert_array_equal(r.mx, plain.mx)  # the whole sums are unchanged
        k32, _, _ = orc.walk(lat, bases, seqs, cases.params(n, steps, 31, flags=flags | FLAG),
                             orc.KERN32, nthreads=8)
        M = len(seqs)
        assert np.all(np.abs(r.mx_in - k32[M:, 0]) <= 2e-5 * n)
        assert np.all(np.abs(r.my_in - k32[M:, 1]) <= 2e-5 * n)
        # the walker count: the G = 0 sum of the start-inside rows without weights
        c, _, _ = orc.walk(lat, bases, [cases.pgse(0)], cases.params(n, 2, 31, flags=FLAG),
                           orc.KERN32, nthreads=8)
        assert r.n_in == int(round(c[1, 0]))
        assert 0 < r.n_in < n
