"""Shared small test substrates and sequences (reference units: mm, ms, T)."""
from oracle import oracle as O

UM = 1e-3        # mm per um
D2 = 2.0e-6      # 2 um^2/ms in mm^2/ms
MTM = 1e-6       # T/mm per mT/m


def lattice_box(side_um=50.0, D=D2, T2=60.0):
    s = side_um * UM
    return O.Lattice(s, s, s, T2, 0.0, D)


def one_cylinder(r_um=5.0, cell_um=12.0, D_in=D2, D_ex=D2, T2_in=80.0, T2_ex=60.0, kappa=0.0):
    c = cell_um * UM
    lat = O.Lattice(c, c, c, T2_ex, 0.0, D_ex)
    cyl = O.Basis(0, 1, c / 2, c / 2, 0.0, r_um * UM, D_in, T2_in, 0.0, kappa, 1e-14)
    return lat, [cyl]


def hex_cylinders(r_um=2.5, f=0.6, D_in=1.7e-6, D_ex=D2, kappa=0.0):
    import math
    r = r_um * UM
    d = math.sqrt(2.0 * math.pi * r * r / (math.sqrt(3.0) * f))
    h = d * 0.86602540378443864676372317075294
    lat = O.Lattice(d, 2 * h, d, 60.0, 0.0, D_ex)
    cs = [(d / 2, 0.0), (0.0, h), (d / 2, 2 * h), (d, h)]
    return lat, [O.Basis(0, k + 1, x, y, 0.0, r, D_in, 80.0, 0.0, kappa, 1e-14)
                 for k, (x, y) in enumerate(cs)]


def sphere_lattice(a_um=10.0, r_um=3.0):
    # body-centred cell: one sphere in the middle and the eight periodic
    # images of the corner sphere (every image that meets the cell is listed,
    # as RPSLatticeInitializer::correctEdges does)
    a = a_um * UM
    pts = [(a / 2, a / 2, a / 2)] + [(i * a, j * a, k * a) for i in (0, 1) for j in (0, 1)
                                     for k in (0, 1)]
    lat = O.Lattice(a, a, a, 60.0, 0.0, D2)
    return lat, [O.Basis(1, k + 1, x, y, z, r_um * UM, 1e-6, 70.0, 0.0, 0.0, 1e-14)
                 for k, (x, y, z) in enumerate(pts)]


def cylinder_grid(n=60, spacing_um=1.0, r_um=0.35, kappa=2e-5):
    """n x n permeable cylinders on a square grid in one periodic cell: more
    bases than the walk kernel stages in shared memory (3,600 at n = 60)."""
    s = spacing_um * UM
    lat = O.Lattice(n * s, n * s, n * s, 60.0, 0.0, D2)
    return lat, [O.Basis(0, k + 1, (k % n + 0.5) * s, (k // n + 0.5) * s, 0.0, r_um * UM, 1.5e-6,
                         80.0, 0.0, kappa, 1e-14) for k in range(n * n)]


def parallel_plates(l_um=8.0, D=D2, with_cylinder=False):
    """Walls at x = 0 and x = l of an l-wide cubic cell, normals pointing
    into the cell, as the reference's planePhase example sets them up
    (Plane(Vector3(0,0,0), Vector3(1,0,0)), Plane(Vector3(l,0,0),
    Vector3(-1,0,0))); optionally a cylinder along z between them."""
    l = l_um * UM
    lat = O.Lattice(l, l, l, 60.0, 0.0, D)
    bases = [O.Basis(2, 0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1e-14, 1.0, 0.0, 0.0),
             O.Basis(2, 0, l, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1e-14, -1.0, 0.0, 0.0)]
    if with_cylinder:
        bases.append(O.Basis(0, 1, l / 2, l / 2, 0.0, 0.3 * l, 1.2e-6, 80.0, 0.0, 3e-5, 1e-14))
    return lat, bases


def pgse(G_mTm, delta=10.0, Delta=40.0, g=(1.0, 0.0, 0.0)):
    return O.Sequence(0, 0, G_mTm * MTM, delta, Delta - delta, *g)


def cos_ogse(G_mTm, n, delta=20.0, Delta=40.0, g=(1.0, 0.0, 0.0), kind=1):
    return O.Sequence(kind, n, G_mTm * MTM, delta, Delta - delta, *g)


def seq_mix():
    return [pgse(0), pgse(100), pgse(200), cos_ogse(100, 2, g=(0.6, 0.8, 0.0)),
            cos_ogse(60, 1, kind=2, g=(0.0, 0.0, 1.0)), cos_ogse(80, 2, kind=3)]


def params(n, steps, seed=1234, dt=0.002, flags=0, init_mode=0, init_arg=0, offset=0):
    return O.Params(n, steps, init_mode, init_arg, flags, seed, dt, 0.0, offset)


def gamma_packing(n=100, seed=5, kappa=2e-5):
    """A dense periodic packing (gamma radii, area fraction 0.6, permeable)
    from the product's host packer, as oracle records: exercises cell lists
    with several candidates per move and walkers crossing cell edges."""
    import axonexa_gb300 as A
    lat, cyl, _ = A.rps_gamma_pack(seed, n, 5.0, 2.5 * UM, 0.6, D_in=1.7e-6, T2_in=80.0,
                                   D_ex=D2, T2_ex=60.0, permeability=kappa)
    L = O.Lattice(lat.a, lat.b, lat.c, lat.T2, 0.0, lat.D)
    return L, [O.Basis(0, c.region, c.centerX, c.centerY, 0.0, c.radius, c.D, c.T2, 0.0,
                       c.permeability, c.eps) for c in cyl]


# ---- magnetisation (Bloch) path: field functors and pores ------------------
def mag_fields():
    """One field functor of each kind (B in T, G in T/mm, times in ms)."""
    F = O.Field
    return [
        F(0, 0, 1e-3, 1e-3, 0, 0, 0, 0.5, 0.6, 0, 0, 0, 0, 0, 0),                # QSC_GRE
        F(1, 0, 1e-3, 1e-3, 0, 0, 0, 0.4, 0.8, 0, 0, 0.2, 0.0005, 0.002, 1.6),   # QSC_PGSE
        F(2, 2, 1e-3, 1e-3, 0, 0, 0, 0.6, 0.4, 0, 0, 0, 0, 0, 0),                # QSC_COS_GRE
        F(3, 0, 1e-3, 1e-3, 0, 0, 0, 0.3, 0.4, 0, 0.1, 0, 0, 0, 0),              # QSC_GRE_TRAP
        F(4, 0, 1e-3, 0, 1e-3, 5e-4, 0, 0.5, 0.4, 0.25, 0, 0, 0, 0, 0),          # SIN_GRE
        F(5, 2, 1e-3, 0, 0, 1e-3, 5e-4, 0.5, 0.4, 0, 0, 0, 0, 0, 0),             # COS_GRE
        F(6, 0, 1e-3, 0, 1e-3, 0, 0, 0.5, 0.4, 0, 0, 0, 0, 0, 0),                # RECT_GRE
        F(7, 0, 1e-4, 2e-4, 0, 0, 0, 0, 0, 0, 0, 0.3, 0.0005, 0.002, 0),         # UCN_lowfield
    ]


def mag_multistep_fields():
    """The functors that define getStepTimeMin (QSC_PGSE, UCN_lowfield)."""
    f = mag_fields()
    return [f[1], f[7]]


def mag_pore(sph=False):
    if sph:
        return O.Basis(1, 1, 0.0, 0.0, 0.0, 6 * UM, D2, 0.0, 0.0, 0.0, 1e-14)
    return O.Basis(0, 1, 0.0, 0.0, 0.0, 5 * UM, D2, 0.0, 0.0, 0.0, 1e-14)
