// substrate.cpp -- host generator of gamma-distributed cylinder packings.
//
// Follows RPSLatticeInitializer (src/substrate/RPSinitializer.h): radii from a
// gamma distribution truncated to (rmin, rmax) and sorted
// (gammaRadialDist :76-101), centres by random sequential addition with a
// periodic overlap test, largest first (uniformCenterDist :103-129), region =
// index + 1 and periodic images of the cylinders that cross the cell edge
// (correctEdges :131-186, circleIntersectsLattice :251-276).  The cell side is
// chosen so that the cylinders' area fraction is the requested one.  When
// random sequential addition cannot place every cylinder at that density
// (its jamming limit is near 0.55 for equal discs), it places them at a lower
// fraction and the cell is compressed to the requested one in small steps,
// each followed by pairwise periodic overlap removal until no two cylinders
// overlap.  Every
// pair keeps a gap of 1 % of its radius sum (kGap).
//
// Randomness: SplitMix64 (Steele, Lea, Flood, OOPSLA 2014) for uniforms,
// Box-Muller normals, and the Marsaglia-Tsang (ACM TOMS 26(3), 2000) gamma
// sampler.  The reference's Numerical Recipes generators are not used, so
// packings agree with the reference in distribution, not draw by draw.
#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/axx.h"

namespace {

struct SplitMix {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
  double normal() {
    const double u1 = uniform(), u2 = uniform();
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  }
  // Gamma(shape k >= 1, scale theta), Marsaglia & Tsang.
  double gamma(double k, double theta) {
    if (k < 1.0) {
      const double u = uniform();
      return gamma(k + 1.0, theta) * std::pow(u, 1.0 / k);
    }
    const double d = k - 1.0 / 3.0, c = 1.0 / std::sqrt(9.0 * d);
    for (;;) {
      double x, v;
      do {
        x = normal();
        v = 1.0 + c * x;
      } while (v <= 0.0);
      v = v * v * v;
      const double u = uniform();
      if (std::log(u) < 0.5 * x * x + d - d * v + d * std::log(v)) return d * v * theta;
    }
  }
};

double min_image(double d, double L) { return d - L * std::nearbyint(d / L); }

// Minimum separation of two cylinders, relative to the sum of their radii.
// Touching cylinders form wedges in which a reflected walker never runs out
// of boundary hits; a 1 % gap keeps every wedge open.
constexpr double kGap = 1.01;

bool overlaps(const std::vector<double> &x, const std::vector<double> &y,
              const std::vector<double> &r, int i, int upto, double L) {
  for (int j = 0; j < upto; ++j) {
    if (j == i) continue;
    const double dx = min_image(x[i] - x[j], L), dy = min_image(y[i] - y[j], L);
    const double s = (r[i] + r[j]) * kGap;
    if (dx * dx + dy * dy < s * s) return true;
  }
  return false;
}

// Pairwise overlap removal: each pair closer than the minimum separation
// moves apart along its centre line by half the shortfall (plus 0.1 % and
// 1e-9 of the cell).
// Returns true when every pair is separated.
bool relax(std::vector<double> &x, std::vector<double> &y, const std::vector<double> &r,
           double L, int iters) {
  const int n = (int)x.size();
  for (int it = 0; it < iters; ++it) {
    bool any = false;
    for (int i = 0; i < n; ++i)
      for (int j = i + 1; j < n; ++j) {
        double dx = min_image(x[i] - x[j], L), dy = min_image(y[i] - y[j], L);
        const double s = (r[i] + r[j]) * kGap;
        double d2 = dx * dx + dy * dy;
        if (d2 >= s * s) continue;
        any = true;
        double d = std::sqrt(d2);
        if (d < 1e-12 * L) {
          dx = 1.0;
          dy = 0.0;
          d = 1.0;
          d2 = 0.0;
        }
        // plus 1e-9 of the cell: an overlap below the rounding of the
        // centres would otherwise be pushed by less than one ulp, forever
        const double push = 0.5 * (s - std::sqrt(d2)) * 1.001 + 1e-9 * L;
        const double ux = dx / d, uy = dy / d;
        x[i] += push * ux;
        y[i] += push * uy;
        x[j] -= push * ux;
        y[j] -= push * uy;
      }
    for (int i = 0; i < n; ++i) {
      x[i] -= L * std::floor(x[i] / L);
      y[i] -= L * std::floor(y[i] / L);
    }
    if (!any) return true;
  }
  return false;
}

bool circle_meets_cell(double x, double y, double r, double L) {
  // RPSLatticeInitializer::circleIntersectsLattice, square cell of side L
  const double h = L / 2.0;
  const double dx = std::fabs(x - h), dy = std::fabs(y - h);
  if (dx > h + r || dy > h + r) return false;
  if (dx <= h || dy <= h) return true;
  return (dx - h) * (dx - h) + (dy - h) * (dy - h) <= r * r;
}

}  // namespace

extern "C" axx_status axx_substrate_pack(uint64_t seed, int n, const double *radii,
                                         double fraction, double D_in, double T2_in,
                                         double permeability, int max_out, axx_basis *out,
                                         int *nout, double *side, double *achieved) {
  if (n < 1 || n > 20000 || !radii || !(fraction > 0.0 && fraction < 0.9) || !out || !nout ||
      !side || !achieved || max_out < n)
    return AXX_ERR_INVALID_ARG;
  std::vector<double> r(radii, radii + n);
  for (double v : r)
    if (!(v > 0.0) || !std::isfinite(v)) return AXX_ERR_INVALID_ARG;
  std::sort(r.begin(), r.end());
  SplitMix rng{seed * 0x2545F4914F6CDD1Dull + 0x7654321ull};
  double area = 0.0;
  for (double v : r) area += 3.141592653589793 * v * v;
  const double L = std::sqrt(area / fraction);
  std::vector<double> x(n), y(n);
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = n - 1 - i;
  // random sequential addition, largest radius first (index n-1 down to 0),
  // in a cell of side Lc; false when a cylinder finds no place in 2,000 draws
  auto rsa = [&](double Lc) {
    std::vector<double> px, py, pr;
    for (int idx = 0; idx < n; ++idx) {
      const int i = order[idx];
      bool ok = false;
      for (int t = 0; t < 2000 && !ok; ++t) {
        px.push_back(rng.uniform() * Lc);
        py.push_back(rng.uniform() * Lc);
        pr.push_back(r[i]);
        const int me = (int)px.size() - 1;
        if (!overlaps(px, py, pr, me, me, Lc)) {
          ok = true;
        } else {
          px.pop_back();
          py.pop_back();
          pr.pop_back();
        }
      }
      if (!ok) return false;
    }
    for (int idx = 0; idx < n; ++idx) {
      x[order[idx]] = px[idx];
      y[order[idx]] = py[idx];
    }
    return true;
  };
  if (!rsa(L)) {
    // Addition jammed (its limit is near 0.55 for equal discs): add at a
    // lower fraction, then compress the cell in steps of 0.01 in fraction,
    // scaling the centres with it and removing the overlaps after each step.
    double fc = std::min(0.5, fraction);
    while (!rsa(std::sqrt(area / fc))) {
      fc -= 0.05;
      if (fc < 0.1) return AXX_ERR_UNSUPPORTED;
    }
    double Lc = std::sqrt(area / fc);
    while (fc < fraction) {
      fc = std::min(fraction, fc + 0.01);
      const double Ln = fc == fraction ? L : std::sqrt(area / fc);
      for (int i = 0; i < n; ++i) {
        x[i] *= Ln / Lc;
        y[i] *= Ln / Lc;
      }
      Lc = Ln;
      if (!relax(x, y, r, Lc, 20000)) return AXX_ERR_UNSUPPORTED;
    }
  }
  // originals, then images of the cylinders that cross the cell edge
  int cnt = 0;
  auto emit = [&](int i, double cx, double cy) {
    if (cnt >= max_out) return false;
    axx_basis &b = out[cnt++];
    b.type = AXX_PRIM_CYLINDER_Z;
    b.region = i + 1;
    b.cx = cx;
    b.cy = cy;
    b.cz = 0.0;
    b.radius = r[i];
    b.D = D_in;
    b.T2 = T2_in;
    b.T1 = 0.0;
    b.permeability = permeability;
    // the reference's initializer default-constructs its cylinders, whose
    // minimum hit distance is cylEPS = 1e-14 (cylinderXY.cuh:26); a smaller
    // one lets the reference's expanded quadratic accept the rounding-level
    // root of the surface a walker was just reflected from
    b.eps = 1e-14;
    b.nx = b.ny = b.nz = 0.0;
    return true;
  };
  for (int i = 0; i < n; ++i)
    if (!emit(i, x[i], y[i])) return AXX_ERR_INVALID_ARG;
  for (int i = 0; i < n; ++i) {
    const bool outside = x[i] + r[i] > L || x[i] - r[i] < 0.0 || y[i] + r[i] > L ||
                         y[i] - r[i] < 0.0;
    if (!outside) continue;
    for (int a = -1; a <= 1; ++a)
      for (int b = -1; b <= 1; ++b) {
        if (a == 0 && b == 0) continue;
        const double cx = x[i] + L * a, cy = y[i] + L * b;
        if (circle_meets_cell(cx, cy, r[i], L))
          if (!emit(i, cx, cy)) return AXX_ERR_INVALID_ARG;
      }
  }
  *nout = cnt;
  *side = L;
  *achieved = area / (L * L);
  return AXX_OK;
}

extern "C" axx_status axx_substrate_rps_gamma(uint64_t seed, int n, double shape, double mean,
                                              double rmin, double rmax, double fraction,
                                              double D_in, double T2_in, double permeability,
                                              int max_out, axx_basis *out, int *nout,
                                              double *side, double *achieved) {
  if (n < 1 || n > 20000 || !(shape > 0.0) || !(mean > 0.0) || !(rmax > rmin))
    return AXX_ERR_INVALID_ARG;
  SplitMix rng{seed * 0x2545F4914F6CDD1Dull + 0x1234567ull};
  std::vector<double> r(n);
  for (int i = 0; i < n; ++i) {
    double d;
    do {
      d = rng.gamma(shape, mean / shape);
    } while (!(d > rmin && d < rmax));
    r[i] = d;
  }
  return axx_substrate_pack(rng.next(), n, r.data(), fraction, D_in, T2_in, permeability,
                            max_out, out, nout, side, achieved);
}
