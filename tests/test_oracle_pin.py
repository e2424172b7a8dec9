"""The CPU oracle against the reference's own walker.

* golden fixtures (tests/golden/ref_walks.npz, made from the reference's
  updateWalkersLatticePhase / updateWalkersPhase compiled for the host) pin
  the oracle everywhere, bit for bit;
* when the reference tree is present, the oracle is also compared live with
  that build over more seeds and switches.
"""
import os

import numpy as np
import pytest

import cases
from golden.make_golden import NTRACE, TRACE_MOVES, golden_cases

GOLD = os.path.join(os.path.dirname(__file__), "golden", "ref_walks.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


@pytest.mark.parametrize("case", golden_cases(), ids=lambda c: c[0])
def test_oracle_matches_reference_golden(orc, gold, case):
    name, var, lat, bases, seqs, p = case
    sums, tr, caps = orc.walk(lat, bases, seqs, p, orc.REF64, nthreads=1, ntrace=NTRACE)
    assert caps == 0
    # the same walk in the same order: identical bits
    np.testing.assert_array_equal(tr["init_pos"], gold[name + "/init_pos"])
    for k in ("pos", "region", "hits", "words"):
        np.testing.assert_array_equal(tr[k][:, :TRACE_MOVES], gold[name + "/" + k], err_msg=k)
    # sums: the oracle adds walkers in the same order with one thread
    np.testing.assert_array_equal(sums, gold[name + "/sums"])


def _ref_available(orc):
    return orc.reflib() is not None


@pytest.mark.parametrize("flags", [0, 1, 2, 3, 4, 5])
@pytest.mark.parametrize("seed", [1, 99])
def test_oracle_matches_reference_live(orc, flags, seed):
    if not _ref_available(orc):
        pytest.skip("reference walker not built here (no reference source tree)")
    lat, cyl = cases.one_cylinder(D_in=1.7e-6, kappa=3e-5)
    seqs = [s for s in cases.seq_mix()]
    p = cases.params(48, 1200, seed, flags=flags)
    s_o, t_o, _ = orc.walk(lat, cyl, seqs, p, orc.REF64, ntrace=48)
    s_r, t_r = orc.ref_walk(orc.variant_for(flags), lat, cyl, seqs, p, ntrace=48)
    np.testing.assert_array_equal(s_o, s_r)
    for k in ("init_pos", "pos", "region", "hits", "words"):
        np.testing.assert_array_equal(t_o[k], t_r[k], err_msg=k)


def test_oracle_matches_reference_live_packs(orc):
    if not _ref_available(orc):
        pytest.skip("reference walker not built here (no reference source tree)")
    for lat, bases in (cases.hex_cylinders(kappa=2e-5), cases.sphere_lattice()):
        p = cases.params(32, 800, 5, flags=3 if bases[0].type == 0 else 1)
        seqs = cases.seq_mix()
        s_o, t_o, _ = orc.walk(lat, bases, seqs, p, orc.REF64, ntrace=32)
        s_r, t_r = orc.ref_walk(orc.variant_for(p.flags), lat, bases, seqs, p, ntrace=32)
        np.testing.assert_array_equal(s_o, s_r)
        for k in ("pos", "region", "hits", "words"):
            np.testing.assert_array_equal(t_o[k], t_r[k], err_msg=k)


@pytest.mark.parametrize("flags", [0, 1, 2, 3, 4, 5])
def test_oracle_matches_reference_live_plates(orc, flags):
    """Plane bases: the reference's Lattice walk over its own Plane class
    (completed with inside() = false), every switch; with simple rejection
    walkers cross the walls (a plane holds no region)."""
    if not _ref_available(orc):
        pytest.skip("reference walker not built here (no reference source tree)")
    lat, plates = cases.parallel_plates(l_um=5.0)
    seqs = [s for s in cases.seq_mix() if s.kind != 4]
    p = cases.params(48, 1500, 40 + flags, flags=flags)
    s_o, t_o, _ = orc.walk(lat, plates, seqs, p, orc.REF64, ntrace=48)
    s_r, t_r = orc.ref_walk(orc.variant_for(flags), lat, plates, seqs, p, ntrace=48)
    np.testing.assert_array_equal(s_o, s_r)
    for k in ("init_pos", "pos", "region", "hits", "words"):
        np.testing.assert_array_equal(t_o[k], t_r[k], err_msg=k)
    if not flags & 4:
        assert t_o["hits"].sum() > 0


@pytest.mark.parametrize("sph", [0, 1])
def test_oracle_matches_reference_live_lattice_picking(orc, sph):
    """LATTICE_PICKING single-pore walks, specular (trajectories and sums)
    and rejection (sums: the reference's trace hook sits in boundaryNormal)."""
    if not _ref_available(orc):
        pytest.skip("reference walker not built here (no reference source tree)")
    b = orc.Basis(sph, 1, 0.0 if sph else 0.001, 0.0 if sph else -0.002, 0.0, 0.004, cases.D2,
                  0, 0, 0, 1e-14)
    seqs = [s for s in cases.seq_mix() if s.kind != 4]
    for flags in (32, 36):
        p = cases.params(48, 1200, 3 + sph, flags=flags)
        s_o, t_o, _ = orc.walk(None, [b], seqs, p, orc.REF64, ntrace=48)
        s_r, t_r = orc.ref_walk(orc.variant_for(flags), None, [b], seqs, p, ntrace=48)
        np.testing.assert_array_equal(s_o, s_r)
        if flags == 32:
            for k in ("init_pos", "pos", "region", "hits", "words"):
                np.testing.assert_array_equal(t_o[k], t_r[k], err_msg=k)
            assert t_o["hits"].sum() > 0


def test_square_wave_is_rejected_by_reference_build(orc):
    # SWOGSEFunc::ampMod is pow(-1., 2 t nu): NaN for non-integer exponents,
    # so the reference build refuses it and the oracle uses the intended wave.
    if not _ref_available(orc):
        pytest.skip("reference walker not built here")
    lat, cyl = cases.one_cylinder()
    sw = cases.cos_ogse(50, 2, kind=4)
    with pytest.raises(ValueError):
        orc.ref_walk("spec_imp", lat, cyl, [sw], cases.params(4, 10))
