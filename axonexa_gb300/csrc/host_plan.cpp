// host_plan.cpp -- sequence and substrate planning for the walk kernels.
#include "host_plan.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <tuple>

namespace axx {

// ---- sequences -------------------------------------------------------------
// Each case restates the reference functor's operator()(time) with G = 1 and
// gHat = x (src/functors/gfunctors.cuh).

double wave_unit(const axx_sequence &q, double t) {
  const double dur = q.duration, sp = q.spacing;
  const bool lobe1 = t < dur;
  const bool lobe2 = (t >= sp + dur) && (t < 2.0 * dur + sp);
  if (!lobe1 && !lobe2) return 0.0;
  const double tt = lobe1 ? t : t - sp - dur;  // gfunctors.cuh:102-103
  const double sign = lobe1 ? 1.0 : -1.0;
  const double n = (double)q.num_periods;
  switch (q.kind) {
    case AXX_SEQ_PGSE:  // RectGrad :36-54
      return sign;
    case AXX_SEQ_COS: {  // CosGFunc :94-113, period = duration / N
      const double period = dur / n;
      return sign * std::cos(2.0 * kPi * tt / period);
    }
    case AXX_SEQ_SIN: {  // SinGFunc :148-167
      const double period = dur / n;
      return sign * std::sin(2.0 * kPi * tt / period);
    }
    case AXX_SEQ_APODCOS: {  // ApodCosGFunc :202-228
      const double period = dur / n;
      if (tt >= period / 4.0 && tt < dur - period / 4.0)
        return sign * std::cos(2.0 * kPi * tt / period);
      return sign * std::sin(4.0 * kPi * tt / period);
    }
    case AXX_SEQ_SQUARE: {  // SWOGSEFunc :265-283 with the intended (-1)^floor(2 t nu)
      const double nu = n / dur;
      const double k = std::floor(2.0 * tt * nu);
      const bool odd = std::fmod(k, 2.0) != 0.0;
      return sign * (odd ? -1.0 : 1.0);
    }
  }
  return 0.0;
}

void gradient(const axx_sequence &q, double t, double out[3]) {
  const double s = wave_unit(q, t) * q.G;
  out[0] = q.gx * s;
  out[1] = q.gy * s;
  out[2] = q.gz * s;
}

double bvalue(const axx_sequence &q, double gamma) {
  const double G = q.G, d = q.duration, sp = q.spacing, n = (double)q.num_periods;
  switch (q.kind) {
    case AXX_SEQ_PGSE:  // gfunctors.cuh:31-33
      return G * G * d * d * gamma * gamma * ((2.0 / 3.0) * d + sp);
    case AXX_SEQ_COS:  // :89-91
      return gamma * gamma * (1.0 / 4.0) * G * G * d * d * d / (kPi * kPi * n * n);
    case AXX_SEQ_SIN:  // :143-145
      return gamma * gamma * (3.0 / 4.0) * G * G * d * d * d / (kPi * kPi * n * n);
    case AXX_SEQ_APODCOS:  // :196-199
      return gamma * gamma * (1.0 / 4.0) * G * G * d * d * d / (kPi * kPi * n * n) *
             (1.0 - 1.0 / (8.0 * n));
    case AXX_SEQ_SQUARE: {  // :256-263
      const double nu = n / d;
      const double a1 = (1. - std::pow(-1., 2. * n) + 4. * d * nu) / (4. * nu);
      return G * G * gamma * gamma * (d / (6. * nu * nu) + sp * (d - a1) * (d - a1));
    }
  }
  return 0.0;
}

static bool finite(double x) { return std::isfinite(x); }

std::string plan_sequences(const axx_sequence *seqs, int nseq, int steps, double dt,
                           double gamma, SeqPlan &out) {
  out = SeqPlan();
  if (nseq < 0 || nseq > AXX_MAX_SEQ) return "nseq must be in [0, 256]";
  if (nseq > 0 && !seqs) return "seqs is NULL";
  std::map<std::tuple<int, int, double, double>, int> keys;
  std::vector<std::vector<int>> members;
  for (int m = 0; m < nseq; ++m) {
    const axx_sequence &q = seqs[m];
    if (q.kind < 0 || q.kind > 4) return "unknown sequence kind";
    if (q.kind != AXX_SEQ_PGSE && q.num_periods < 1) return "OGSE needs num_periods >= 1";
    if (!(q.duration > 0.0) || !(q.spacing >= 0.0) || !finite(q.G) || !finite(q.gx) ||
        !finite(q.gy) || !finite(q.gz) || !finite(q.duration) || !finite(q.spacing))
      return "sequence parameters must be finite, duration > 0, spacing >= 0";
    const int np = q.kind == AXX_SEQ_PGSE ? 0 : q.num_periods;
    auto key = std::make_tuple(q.kind, np, q.duration, q.spacing);
    auto it = keys.find(key);
    int w;
    if (it == keys.end()) {
      w = (int)members.size();
      keys[key] = w;
      members.emplace_back();
    } else {
      w = it->second;
    }
    members[w].push_back(m);
    out.seq_wave.push_back(w);
  }
  out.W = (int)members.size();
  // waveform tables s_w(i*dt), i = 0..steps-1 (time = timestep * i in FP64,
  // kernelLattice.cuh:84)
  out.wave.assign((size_t)out.W * steps, 0.f);
  for (int w = 0; w < out.W; ++w) {
    const axx_sequence &q = seqs[members[w][0]];
    for (int i = 0; i < steps; ++i)
      out.wave[(size_t)w * steps + i] = (float)wave_unit(q, dt * (double)i);
  }
  // channels: an orthonormal basis of each waveform's gradient directions
  std::vector<int> first_channel(out.W);
  for (int w = 0; w < out.W; ++w) {
    std::vector<std::array<double, 3>> basis;
    for (int m : members[w]) {
      const double g[3] = {seqs[m].gx, seqs[m].gy, seqs[m].gz};
      const double gn = std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
      if (gn == 0.0) continue;
      double r[3] = {g[0], g[1], g[2]};
      for (auto &p : basis) {
        const double d = r[0] * p[0] + r[1] * p[1] + r[2] * p[2];
        for (int k = 0; k < 3; ++k) r[k] -= d * p[k];
      }
      const double rn = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
      if (rn > 1e-9 * gn && basis.size() < 3) basis.push_back({r[0] / rn, r[1] / rn, r[2] / rn});
    }
    if (basis.size() == 3) basis = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    if (basis.empty()) basis.push_back({1, 0, 0});
    first_channel[w] = (int)out.channels.size();
    for (auto &p : basis) {
      Channel c;
      c.wave = w;
      for (int k = 0; k < 3; ++k) c.p[k] = (float)p[k];
      out.channels.push_back(c);
    }
  }
  const int K = (int)out.channels.size();
  out.coef.assign((size_t)nseq * K, 0.0);
  for (int m = 0; m < nseq; ++m) {
    const int w = out.seq_wave[m];
    const double g[3] = {seqs[m].gx, seqs[m].gy, seqs[m].gz};
    // solve sum_c alpha_c p_c = g over the waveform's channels (least squares
    // with the FP32-rounded p_c; exact when the p_c are axis vectors)
    int c0 = first_channel[w], c1 = c0;
    while (c1 < K && out.channels[c1].wave == w) ++c1;
    const int n = c1 - c0;
    double A[3][3] = {{0}}, rhs[3] = {0};
    for (int a = 0; a < n; ++a) {
      const float *pa = out.channels[c0 + a].p;
      for (int b = 0; b < n; ++b) {
        const float *pb = out.channels[c0 + b].p;
        A[a][b] = (double)pa[0] * pb[0] + (double)pa[1] * pb[1] + (double)pa[2] * pb[2];
      }
      rhs[a] = (double)pa[0] * g[0] + (double)pa[1] * g[1] + (double)pa[2] * g[2];
    }
    // Gaussian elimination on the n x n Gram matrix (n <= 3)
    double alpha[3] = {0, 0, 0};
    for (int col = 0; col < n; ++col) {
      int piv = col;
      for (int r = col + 1; r < n; ++r)
        if (std::fabs(A[r][col]) > std::fabs(A[piv][col])) piv = r;
      std::swap(A[col], A[piv]);
      std::swap(rhs[col], rhs[piv]);
      for (int r = col + 1; r < n; ++r) {
        const double f = A[r][col] / A[col][col];
        for (int k = col; k < n; ++k) A[r][k] -= f * A[col][k];
        rhs[r] -= f * rhs[col];
      }
    }
    for (int r = n - 1; r >= 0; --r) {
      double s = rhs[r];
      for (int k = r + 1; k < n; ++k) s -= A[r][k] * alpha[k];
      alpha[r] = s / A[r][r];
    }
    for (int a = 0; a < n; ++a)
      out.coef[(size_t)m * K + c0 + a] = gamma * dt * seqs[m].G * alpha[a];
  }
  return "";
}

// ---- substrates -------------------------------------------------------------

static void slot_entry(double D, double T2, double kappa, double dt, bool relax, float4 &e) {
  const double speed = std::sqrt(6.0 * D / dt);  // kernelLattice.cuh:50
  e.x = (float)speed;
  e.y = (float)(speed * dt);
  e.z = (relax && T2 > 0.0) ? (float)(dt / T2) : 0.0f;
  e.w = (float)(4.0 * kappa);  // boundaryCheck.cuh:95
}

static std::string check_basis(const axx_basis &b) {
  if (b.type == AXX_PRIM_PLANE) {
    if (!finite(b.cx) || !finite(b.cy) || !finite(b.cz) || !finite(b.nx) || !finite(b.ny) ||
        !finite(b.nz) || !finite(b.eps) || b.eps < 0.0)
      return "plane parameters must be finite (eps >= 0)";
    if (!(b.nx * b.nx + b.ny * b.ny + b.nz * b.nz > 1e-24)) return "plane normal must be nonzero";
    return "";
  }
  if (b.type == AXX_PRIM_CYLINDER)
    return "arbitrary-axis cylinders are not supported by this entry point";
  if (b.type != AXX_PRIM_CYLINDER_Z && b.type != AXX_PRIM_SPHERE) return "unknown basis type";
  if (!(b.radius > 0.0) || !finite(b.radius)) return "basis radius must be > 0";
  if (!(b.D >= 0.0) || !finite(b.D)) return "basis D must be >= 0";
  if (!finite(b.cx) || !finite(b.cy) || !finite(b.cz) || !finite(b.T2) ||
      !finite(b.permeability) || !finite(b.eps) || b.permeability < 0.0 || b.eps < 0.0)
    return "basis parameters must be finite (kappa, eps >= 0)";
  return "";
}

static float4 geo_of(double cx, double cy, double cz, double R) {
  return make_float4((float)cx, (float)cy, (float)cz, (float)(-(R * R)));
}

// A plane instance: geo = (n, n.c) with the unit normal n and a point c of
// the plane; aux.x is unused.
static float4 plane_geo(const double n[3], double cx, double cy, double cz) {
  return make_float4((float)n[0], (float)n[1], (float)n[2],
                     (float)(n[0] * cx + n[1] * cy + n[2] * cz));
}

static void unit_normal(const axx_basis &b, double n[3]) {
  const double m = std::sqrt(b.nx * b.nx + b.ny * b.ny + b.nz * b.nz);
  n[0] = b.nx / m;
  n[1] = b.ny / m;
  n[2] = b.nz / m;
}

static float4 aux_of(const axx_basis &b, int slot) {
  float4 a;
  a.x = b.type == AXX_PRIM_PLANE ? 1.0f : (float)(1.0 / b.radius);
  a.y = (float)b.eps;
  int s = slot, t = b.type;
  std::memcpy(&a.z, &s, 4);
  std::memcpy(&a.w, &t, 4);
  return a;
}

// One basis instance (a basis or a periodic ghost of it) during planning.
struct Inst {
  int k;
  double cx, cy, cz, R;
  int type;
  double n[3];  // unit normal of a plane
};

// A plane meets a box when the signed distances n.(x - c) of the box's
// corners do not all have one sign.
static bool plane_meets(const Inst &q, double x0, double x1, double y0, double y1, double z0,
                        double z1) {
  double lo = 0.0, hi = 0.0;
  const double xs[2] = {x0, x1}, ys[2] = {y0, y1}, zs[2] = {z0, z1};
  for (int i = 0; i < 8; ++i) {
    const double d = q.n[0] * (xs[i & 1] - q.cx) + q.n[1] * (ys[(i >> 1) & 1] - q.cy) +
                     q.n[2] * (zs[i >> 2] - q.cz);
    lo = i ? std::min(lo, d) : d;
    hi = i ? std::max(hi, d) : d;
  }
  return lo <= 0.0 && hi >= 0.0;
}

// Uniform gx x gy x gz grid over the a x b x c cell: per grid cell, the
// instances that can be met from inside it within one step (the cell box
// dilated by dil, plus a slack for the FP32 rounding of the cell index), in
// ascending instance (basis) order.  The outer cells reach beyond the cell
// edge (positions are clamped into the grid).  Each instance is tested only
// against the cells its dilated bounding box can reach.
static void build_grid(GeomPlan &g, const std::vector<Inst> &inst, double A, double B, double C,
                       double dil, int gx, int gy, int gz) {
  g.gx = gx;
  g.gy = gy;
  g.gz = gz;
  g.inv_hx = (float)((double)gx / A);
  g.inv_hy = (float)((double)gy / B);
  g.inv_hz = (float)((double)gz / C);
  const int ncell = gx * gy * gz;
  const double sx = 1e-5 * A / gx, sy = 1e-5 * B / gy, sz = 1e-5 * C / gz;
  auto lo_of = [](int i, double side, int n) { return i == 0 ? -1e300 : side * i / n; };
  auto hi_of = [](int i, double side, int n) { return i == n - 1 ? 1e300 : side * (i + 1) / n; };
  auto range = [](double lo, double hi, double side, int n, int &i0, int &i1) {
    const double hh = side / n;
    i0 = (int)std::max(0.0, std::min((double)n - 1, std::floor(lo / hh) - 1));
    i1 = (int)std::max(0.0, std::min((double)n - 1, std::floor(hi / hh) + 1));
  };
  std::vector<std::vector<uint16_t>> lists(ncell);
  for (size_t n = 0; n < inst.size(); ++n) {
    const Inst &q = inst[n];
    int x0 = 0, x1 = gx - 1, y0 = 0, y1 = gy - 1, z0 = 0, z1 = gz - 1;
    if (q.type != AXX_PRIM_PLANE) {
      const double r = q.R + dil;
      range(q.cx - r, q.cx + r, A, gx, x0, x1);
      range(q.cy - r, q.cy + r, B, gy, y0, y1);
      if (q.type == AXX_PRIM_SPHERE) range(q.cz - r, q.cz + r, C, gz, z0, z1);
    }
    for (int iz = z0; iz <= z1; ++iz)
      for (int iy = y0; iy <= y1; ++iy)
        for (int ix = x0; ix <= x1; ++ix) {
          const double bx0 = lo_of(ix, A, gx) - dil - sx, bx1 = hi_of(ix, A, gx) + dil + sx;
          const double by0 = lo_of(iy, B, gy) - dil - sy, by1 = hi_of(iy, B, gy) + dil + sy;
          const double bz0 = lo_of(iz, C, gz) - dil - sz, bz1 = hi_of(iz, C, gz) + dil + sz;
          bool meets;
          if (q.type == AXX_PRIM_PLANE) {
            meets = plane_meets(q, bx0, bx1, by0, by1, bz0, bz1);
          } else {
            auto axis = [](double c, double lo, double hi) {
              return c < lo ? lo - c : (c > hi ? c - hi : 0.0);
            };
            const double ex = axis(q.cx, bx0, bx1), ey = axis(q.cy, by0, by1);
            double d2 = ex * ex + ey * ey;
            if (q.type == AXX_PRIM_SPHERE) {
              const double ez = axis(q.cz, bz0, bz1);
              d2 += ez * ez;
            }
            meets = d2 < q.R * q.R;
          }
          if (meets) lists[(iz * gy + iy) * gx + ix].push_back((uint16_t)n);
        }
  }
  g.cstart.assign(ncell + 1, 0);
  g.clist.clear();
  for (int c = 0; c < ncell; ++c) {
    g.clist.insert(g.clist.end(), lists[c].begin(), lists[c].end());
    g.cstart[c + 1] = (uint32_t)g.clist.size();
  }
}

std::string plan_lattice(const axx_lattice *lat, const axx_basis *basis, int nbasis, double dt,
                         uint32_t flags, GeomPlan &g, size_t list_budget) {
  g = GeomPlan();
  if (!lat) return "lattice is NULL";
  if (!(lat->a > 0.0) || !(lat->b > 0.0) || !(lat->c > 0.0)) return "cell sides must be > 0";
  if (!(lat->D >= 0.0) || !finite(lat->D)) return "lattice D must be >= 0";
  if (nbasis < 0 || nbasis > 60000) return "nbasis must be in [0, 60000]";
  if (nbasis > 0 && !basis) return "basis is NULL";
  if (flags & AXX_FLAG_LATTICE_PICKING)
    return "lattice picking exists only in the single-pore walk (kernelPhase.cuh:31-35)";
  const bool relax = flags & AXX_FLAG_RELAXATION;
  bool any_cyl = false, any_sph = false, any_plane = false;
  for (int k = 0; k < nbasis; ++k) {
    std::string e = check_basis(basis[k]);
    if (!e.empty()) return e;
    if (basis[k].type == AXX_PRIM_SPHERE) any_sph = true;
    else if (basis[k].type == AXX_PRIM_PLANE) any_plane = true;
    else any_cyl = true;
  }
  if (relax) {
    if (!(lat->T2 > 0.0)) return "relaxation needs lattice T2 > 0";
    for (int k = 0; k < nbasis; ++k)
      if (basis[k].type != AXX_PRIM_PLANE && !(basis[k].T2 > 0.0))
        return "relaxation needs basis T2 > 0";
  }
  // planes run in the mixed-type kernels (per-instance type)
  g.geom = nbasis == 0 ? AXX_GEOM_FREE
                       : ((any_cyl && any_sph) || any_plane
                              ? AXX_GEOM_MIX
                              : (any_sph ? AXX_GEOM_SPH : AXX_GEOM_CYL));
  g.slot_tab.resize(nbasis + 1);
  g.slot_region.resize(nbasis + 1);
  for (int k = 0; k < nbasis; ++k) {
    if (basis[k].type == AXX_PRIM_PLANE) {
      // never a walker's region; only its zero transmission is read
      slot_entry(lat->D, lat->T2, 0.0, dt, relax, g.slot_tab[k]);
    } else {
      slot_entry(basis[k].D, basis[k].T2, basis[k].permeability, dt, relax, g.slot_tab[k]);
    }
    g.slot_region[k] = basis[k].region;
  }
  slot_entry(lat->D, lat->T2, 0.0, dt, relax, g.slot_tab[nbasis]);
  g.slot_region[nbasis] = 0;  // Lattice::inRegion returns 0 outside every basis
  g.ecs_slot = nbasis;
  float lmax = 0.f;
  for (auto &e : g.slot_tab) lmax = std::max(lmax, e.y);
  g.lmax = lmax;
  const double A = lat->a, B = lat->b, C = lat->c;
  if (2.0 * (double)lmax >= std::min(A, std::min(B, C)))
    return "the step length must be below half the smallest cell side";
  if (nbasis == 0) {
    g.cstart = {0, 0};
    return "";
  }
  // instances: each basis, then its periodic ghosts that can be reached from
  // the cell within one step and do not coincide with a listed basis
  const double dil = (double)lmax * 1.01 + 1e-7 * std::max(A, std::max(B, C));
  const double tol = 1e-9 * std::max(A, std::max(B, C));
  std::vector<Inst> inst;
  auto reach = [&](const Inst &q) {
    if (q.type == AXX_PRIM_PLANE)
      return plane_meets(q, -dil, A + dil, -dil, B + dil, -dil, C + dil);
    // distance from the centre to the cell box dilated by dil
    auto axis = [](double c, double lo, double hi) {
      return c < lo ? lo - c : (c > hi ? c - hi : 0.0);
    };
    const double ex = axis(q.cx, -dil, A + dil), ey = axis(q.cy, -dil, B + dil);
    double d2 = ex * ex + ey * ey;
    if (q.type == AXX_PRIM_SPHERE) {
      const double ez = axis(q.cz, -dil, C + dil);
      d2 += ez * ez;
    }
    return d2 < q.R * q.R;
  };
  auto coincides = [&](const Inst &q) {
    for (int j = 0; j < nbasis; ++j) {
      const axx_basis &o = basis[j];
      if (o.type != q.type) continue;
      if (q.type == AXX_PRIM_PLANE) {
        // the same plane: parallel normals (either sense) and q's point on it
        double n[3];
        unit_normal(o, n);
        const double cr = std::fabs(n[1] * q.n[2] - n[2] * q.n[1]) +
                          std::fabs(n[2] * q.n[0] - n[0] * q.n[2]) +
                          std::fabs(n[0] * q.n[1] - n[1] * q.n[0]);
        const double d = n[0] * (q.cx - o.cx) + n[1] * (q.cy - o.cy) + n[2] * (q.cz - o.cz);
        if (cr < 1e-12 && std::fabs(d) <= tol) return true;
        continue;
      }
      if (std::fabs(o.radius - q.R) > tol) continue;
      if (std::fabs(o.cx - q.cx) > tol || std::fabs(o.cy - q.cy) > tol) continue;
      if (q.type == AXX_PRIM_SPHERE && std::fabs(o.cz - q.cz) > tol) continue;
      return true;
    }
    return false;
  };
  // image offsets along one axis that can bring a basis within reach of the
  // cell: every offset whose translate of [c - R, c + R] meets the dilated
  // cell (one cell each way for a basis inside the cell and smaller than it;
  // more for a basis centred far outside or larger than a cell side).  A
  // plane's images along its normal: one each way is enough for the walls
  // of a cell.
  auto offsets = [&](double c, double R, double side, int &lo, int &hi) {
    lo = std::max(-64, (int)std::floor((-dil - R - c) / side));
    hi = std::min(64, (int)std::ceil((side + dil + R - c) / side));
  };
  for (int k = 0; k < nbasis; ++k) {
    const axx_basis &b = basis[k];
    Inst q0{k, b.cx, b.cy, b.cz, b.radius, b.type, {0.0, 0.0, 0.0}};
    if (b.type == AXX_PRIM_PLANE) unit_normal(b, q0.n);
    inst.push_back(q0);
    int i0 = -1, i1 = 1, j0 = -1, j1 = 1, l0 = -1, l1 = 1;
    if (b.type != AXX_PRIM_PLANE) {
      offsets(b.cx, b.radius, A, i0, i1);
      offsets(b.cy, b.radius, B, j0, j1);
      offsets(b.cz, b.radius, C, l0, l1);
    }
    if (b.type == AXX_PRIM_CYLINDER_Z) l0 = l1 = 0;
    for (int i = i0; i <= i1; ++i)
      for (int j = j0; j <= j1; ++j)
        for (int l = l0; l <= l1; ++l) {
          if (i == 0 && j == 0 && l == 0) continue;
          Inst q = q0;
          q.cx += A * i;
          q.cy += B * j;
          q.cz += C * l;
          if (!reach(q) || coincides(q)) continue;
          inst.push_back(q);
        }
  }
  if (inst.size() > 65535) return "too many basis instances (ghosts included)";
  for (auto &q : inst) {
    g.geo.push_back(q.type == AXX_PRIM_PLANE ? plane_geo(q.n, q.cx, q.cy, q.cz)
                                             : geo_of(q.cx, q.cy, q.cz, q.R));
    g.aux.push_back(aux_of(basis[q.k], q.k));
  }
  if (g.geom == AXX_GEOM_CYL) {
    // the annulus test of the cylinder lists: (R + h)^2 in the unused cz,
    // h = half the longest step plus a slack far above FP32 position rounding
    const double hh = 0.5 * (double)lmax + 0.01 * (double)lmax + 1e-6 * std::max(A, B);
    for (size_t n = 0; n < inst.size(); ++n) g.geo[n].z = (float)((inst[n].R + hh) * (inst[n].R + hh));
    g.ann_h2x2 = (float)(2.0 * hh * hh);
  }
  // grid over the cell: about one basis per grid cell's area
  const double h = std::max(2.0 * (double)lmax, std::sqrt(A * B / (double)nbasis));
  auto cells_along = [&](double side, double hh, int cap) {
    return (int)std::min((double)cap, std::max(1.0, std::floor(side / hh)));
  };
  const bool flat = !(any_sph || any_plane);  // z-cylinders only: a 2-D grid
  build_grid(g, inst, A, B, C, dil, cells_along(A, h, 64), cells_along(B, h, 64),
             flat ? 1 : cells_along(C, h, 64));
  // Finer 2-D grids leave fewer candidates per move (a grid cell about a
  // third of a basis across lists about 1.3 cylinders, against 3.3 at one
  // basis per cell), as long as the staged tables stay within the budget.
  // Cells of few bases (a hexagonal cell of four) fit grids up to 16 times
  // finer, which leave under one candidate per move.
  if (list_budget > 0 && flat && inst.size() > 1) {
    const size_t fixed = inst.size() * 32;
    for (double f : {16.0, 12.0, 8.0, 6.0, 5.0, 4.0, 3.5, 3.0, 2.5, 2.0, 1.5}) {
      const int gx = cells_along(A, h / f, 256), gy = cells_along(B, h / f, 256);
      if (gx <= g.gx && gy <= g.gy) break;
      // a cheap lower bound first: the cell starts alone
      if (fixed + ((size_t)gx * gy + 1) * 4 > list_budget) continue;
      GeomPlan t = g;
      build_grid(t, inst, A, B, C, dil, gx, gy, 1);
      if (fixed + t.cstart.size() * 4 + t.clist.size() * 2 <= list_budget) {
        g = t;
        break;
      }
    }
  }
  return "";
}

std::string plan_single(const axx_basis *basis, double dt, GeomPlan &g, float &speed,
                        float &step) {
  g = GeomPlan();
  if (!basis) return "basis is NULL";
  std::string e = check_basis(*basis);
  if (!e.empty()) return e;
  if (basis->type == AXX_PRIM_PLANE) return "a plane is not a pore (it has no inside)";
  g.geom = basis->type == AXX_PRIM_SPHERE ? AXX_GEOM_SPH : AXX_GEOM_CYL;
  g.geo.push_back(geo_of(basis->cx, basis->cy, basis->cz, basis->radius));
  g.aux.push_back(aux_of(*basis, 0));
  g.cstart = {0, 1};
  g.clist = {0};
  g.slot_tab.resize(2);
  slot_entry(basis->D, basis->T2, 0.0, dt, false, g.slot_tab[0]);
  slot_entry(basis->D, basis->T2, 0.0, dt, false, g.slot_tab[1]);
  g.slot_region = {basis->region, 0};
  g.ecs_slot = 1;
  // updateWalkersPhase: speed = sqrt(6 D / dt), step = speed * dt (kernelPhase.cuh:16-17)
  const double sp = std::sqrt(6.0 * basis->D / dt);
  speed = (float)sp;
  step = (float)(sp * dt);
  g.lmax = step;
  return "";
}

}  // namespace axx
