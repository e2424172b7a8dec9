"""The GPU substrate generator (axx_substrate_rps_gamma_gpu: RPSLatticeInitializer,
src/substrate/RPSinitializer.h:10-314, one block per packing) against the
host packer (axx_substrate_rps_gamma): every packing is valid (no two
cylinders closer than the 1 % gap under the minimum image, the requested area
fraction, the periodic images the edge rule gives), and the radii agree with
the host packer's in distribution."""
import numpy as np
import pytest

import axonexa_gb300 as A
from axonexa_gb300.substrate import rps_gamma_pack, rps_gamma_pack_gpu

pytestmark = pytest.mark.gpu

UM = 1e-3


def _check_packing(lat, cyl, f, n, fraction):
    L = lat.a
    assert abs(f - fraction) < 1e-12
    orig = cyl[:n]
    assert [c.region for c in orig] == list(range(1, n + 1))
    r = np.array([c.radius for c in orig])
    assert np.all(np.diff(r) >= 0)
    x = np.array([c.centerX for c in orig])
    y = np.array([c.centerY for c in orig])
    assert np.all((x >= 0) & (x < L) & (y >= 0) & (y < L))
    assert abs(np.pi * np.sum(r * r) / (L * L) - fraction) < 1e-9
    dx = x[:, None] - x[None, :]
    dy = y[:, None] - y[None, :]
    dx -= L * np.rint(dx / L)
    dy -= L * np.rint(dy / L)
    d = np.hypot(dx, dy)
    s = (r[:, None] + r[None, :]) * 1.01
    np.fill_diagonal(d, np.inf)
    assert np.all(d >= s * (1 - 1e-9)), "overlapping cylinders"
    # images: exactly the translates of edge-crossing cylinders that meet the cell
    want = []
    h = L / 2
    for i in range(n):
        if not (x[i] + r[i] > L or x[i] - r[i] < 0 or y[i] + r[i] > L or y[i] - r[i] < 0):
            continue
        for a in (-1, 0, 1):
            for b in (-1, 0, 1):
                if a == 0 and b == 0:
                    continue
                cx, cy = x[i] + L * a, y[i] + L * b
                ex, ey = abs(cx - h), abs(cy - h)
                if ex > h + r[i] or ey > h + r[i]:
                    continue
                if ex <= h or ey <= h or (ex - h) ** 2 + (ey - h) ** 2 <= r[i] ** 2:
                    want.append((i + 1, cx, cy))
    got = [(c.region, c.centerX, c.centerY) for c in cyl[n:]]
    assert len(got) == len(want)
    for (ga, gx, gy), (wa, wx, wy) in zip(got, want):
        assert ga == wa and abs(gx - wx) < 1e-12 * L and abs(gy - wy) < 1e-12 * L
    return r


@pytest.mark.parametrize("fraction,shape", [(0.45, 5.0), (0.6, 5.0), (0.65, 3.0)])
def test_gpu_packings_valid_and_match_host_in_distribution(fraction, shape):
    from scipy.stats import ks_2samp
    n, npack = 400, 24
    spec = dict(shape=shape, mean=2.5 * UM, fraction=fraction, D_in=1.7e-6, T2_in=80.0,
                permeability=2e-5)
    gpu = rps_gamma_pack_gpu(11, n, [spec] * npack, T2_ex=60.0, D_ex=2e-6)
    rg = np.concatenate([_check_packing(lat, cyl, f, n, fraction) for lat, cyl, f in gpu])
    host = [rps_gamma_pack(1000 + s, n, shape, 2.5 * UM, fraction, D_in=1.7e-6, T2_in=80.0,
                           D_ex=2e-6, T2_ex=60.0, permeability=2e-5) for s in range(npack)]
    rh = np.concatenate([_check_packing(lat, cyl, f, n, fraction) for lat, cyl, f in host])
    assert ks_2samp(rg, rh).pvalue > 1e-3
    # the truncated gamma's mean (truncation at 0.05 and 4 x the mean is negligible)
    assert abs(rg.mean() / (2.5 * UM) - 1) < 0.02
    # different seeds, different packings
    assert len({round(c[0].centerX, 12) for _, c, _ in gpu}) == npack


def test_gpu_packing_walks():
    """A walk on a GPU packing: the permeable benchmark substrate's style."""
    (lat, cyl, f), = rps_gamma_pack_gpu(3, 100, [dict(shape=5.0, mean=2.5 * UM, fraction=0.6,
                                                       D_in=1.7e-6, T2_in=80.0,
                                                       permeability=2e-5)],
                                         T2_ex=60.0, D_ex=2e-6)
    seqs = [A.RectGrad(g * 1e-6, 10.0, 20.0) for g in (0.0, 100.0)]
    r = A.run_lattice(lat, cyl, seqs, 8192, 2000, 0.001, 7, relaxation=True, permeable=True)
    assert r.hits > 0 and 0.5 < r.signal[0] <= 1.0 and r.signal[1] < r.signal[0]
