// Property check of the lattice planner's cell lists (host code only):
// every periodic image of a basis cylinder that a move of the longest step
// can meet, or that contains the move's start, is in the candidate list of
// the grid cell the walk kernel files the start under (FP32 position, the
// kernel's cell index).  The images are enumerated here independently of the
// planner's ghost selection.  Substrates: hexagonal cells (four cylinders,
// examples/hexPhase.cu:110-124) at several fractions and radii, and random
// packs of cylinders with random radii, each planned with the walk's table
// budgets and without one; random packs of spheres (a 3-D grid).
//
// Output: one line per plan, "plan <name> <budget> <gx> <gy> <cand/cell>
// <instances> <checked> <violations>", then "done".
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../axonexa_gb300/csrc/host_plan.h"

using namespace axx;

namespace {

struct Cyl {
  double x, y, r;
  double z = 0.0;
  bool sphere = false;
};

int cell_index(float x, float inv, int n) {
  const float t = std::fmaf(x, inv, -0.5f);
  const float f = t + 12582912.0f;
  int32_t i;
  std::memcpy(&i, &f, 4);
  i -= 0x4B400000;
  return i < 0 ? 0 : (i > n - 1 ? n - 1 : i);
}

// Whether the segment a -> b meets the boundary of the circle (cylinders:
// xy) or sphere (its distance range to the centre spans r, with a margin),
// or a lies inside it.
bool reaches(const double a[3], const double b[3], const Cyl &c, double margin) {
  const double cz = c.sphere ? c.z : 0.0, az = c.sphere ? a[2] : 0.0, bz = c.sphere ? b[2] : 0.0;
  const double dx = b[0] - a[0], dy = b[1] - a[1], dz = bz - az;
  const double px = a[0] - c.x, py = a[1] - c.y, pz = az - cz;
  const double dd = dx * dx + dy * dy + dz * dz;
  double t = dd > 0.0 ? -(px * dx + py * dy + pz * dz) / dd : 0.0;
  t = t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t);
  const double qx = px + t * dx, qy = py + t * dy, qz = pz + t * dz;
  const double dmin = std::sqrt(qx * qx + qy * qy + qz * qz);
  const double da = std::sqrt(px * px + py * py + pz * pz);
  const double ex = b[0] - c.x, ey = b[1] - c.y, ez = bz - cz;
  const double db = std::sqrt(ex * ex + ey * ey + ez * ez);
  const double dmax = da > db ? da : db;
  if (da < c.r + margin) return true;  // starts inside (or on) the boundary
  return dmin <= c.r + margin && dmax >= c.r - margin;
}

int check(const char *name, double A, double B, const std::vector<Cyl> &cyl, size_t budget,
          int samples, std::mt19937_64 &rng) {
  axx_lattice lat{};
  lat.a = A;
  lat.b = B;
  lat.c = A;
  lat.T2 = 60.0;
  lat.D = 2.0e-6;
  std::vector<axx_basis> bs(cyl.size());
  for (size_t k = 0; k < cyl.size(); ++k) {
    axx_basis &b = bs[k];
    std::memset(&b, 0, sizeof b);
    b.cx = cyl[k].x;
    b.cy = cyl[k].y;
    b.cz = cyl[k].z;
    b.radius = cyl[k].r;
    b.type = cyl[k].sphere ? AXX_PRIM_SPHERE : AXX_PRIM_CYLINDER_Z;
    b.D = 1.7e-6;
    b.T2 = 80.0;
    b.region = (int)k + 1;
    b.permeability = 1e-5;
  }
  GeomPlan g;
  const std::string e = plan_lattice(&lat, bs.data(), (int)bs.size(), 0.005,
                                     AXX_FLAG_PERMEABLE | AXX_FLAG_RELAXATION, g, budget);
  if (!e.empty()) {
    std::printf("error %s: %s\n", name, e.c_str());
    return 1;
  }
  const double L = (double)g.lmax;
  const double tol = 1e-6 * (A > B ? A : B);
  // every image of every basis within two cells
  std::vector<Cyl> img;
  for (size_t k = 0; k < cyl.size(); ++k)
    for (int i = -2; i <= 2; ++i)
      for (int j = -2; j <= 2; ++j)
        for (int l = -2; l <= 2; ++l) {
          if (!cyl[k].sphere && l != 0) continue;
          Cyl c = cyl[k];
          c.x += i * A;
          c.y += j * B;
          c.z += l * A;
          img.push_back(c);
        }
  std::uniform_real_distribution<double> U(0.0, 1.0);
  long long checked = 0, bad = 0;
  for (int s = 0; s < samples; ++s) {
    // an FP32 start in the cell, as the walk holds it; every other start
    // sits within a few ulps of a grid line, where the cell index rounds
    float fx = (float)(U(rng) * A), fy = (float)(U(rng) * B), fz = (float)(U(rng) * A);
    if (s & 1) {
      auto snap = [&](float &v, double side, int n) {
        const int i = (int)(U(rng) * n), u = (int)(U(rng) * 7) - 3;
        v = (float)(i * (side / n));
        for (int k = 0; k < (u < 0 ? -u : u); ++k) v = std::nextafterf(v, u < 0 ? -1.0f : 1.0f);
      };
      snap(fx, A, g.gx);
      snap(fy, B, g.gy);
      snap(fz, A, g.gz);
      if (!(fx >= 0.0f) || !(fy >= 0.0f) || !(fz >= 0.0f)) continue;
    }
    if (!(fx < (float)A) || !(fy < (float)B) || !(fz < (float)A)) continue;
    const double a[3] = {fx, fy, fz};
    const double phi = 2.0 * kPi * U(rng), cz = 2.0 * U(rng) - 1.0;
    const double sxy = std::sqrt(1.0 - cz * cz);
    const double b[3] = {a[0] + L * sxy * std::cos(phi), a[1] + L * sxy * std::sin(phi),
                         a[2] + L * cz};
    int cell = cell_index(fx, g.inv_hx, g.gx) + g.gx * cell_index(fy, g.inv_hy, g.gy);
    if (g.gz > 1) cell += g.gx * g.gy * cell_index(fz, g.inv_hz, g.gz);
    const uint32_t b0 = g.cstart[cell], b1 = g.cstart[cell + 1];
    for (size_t m = 0; m < img.size(); ++m) {
      if (!reaches(a, b, img[m], tol)) continue;
      ++checked;
      bool found = false;
      for (uint32_t j = b0; j < b1 && !found; ++j) {
        // the same circle: centre and radius (an image that coincides with
        // another basis is listed once, as that basis)
        const float4 q = g.geo[g.clist[j]];
        found = std::fabs(q.x - img[m].x) < tol && std::fabs(q.y - img[m].y) < tol &&
                (!img[m].sphere || std::fabs(q.z - img[m].z) < tol) &&
                std::fabs(std::sqrt(-(double)q.w) - img[m].r) < tol;
      }
      if (!found) ++bad;
    }
  }
  std::printf("plan %s %zu %d %d %.4f %zu %lld %lld\n", name, budget, g.gx, g.gy,
              (double)g.cstart.back() / (double)(g.cstart.size() - 1), g.geo.size(), checked,
              bad);
  return 0;
}

// Non-overlapping cylinders of random radii by random sequential addition
// in the periodic a x a cell (minimum-image distances).
std::vector<Cyl> random_pack(double a, int n, double rmin, double rmax, std::mt19937_64 &rng) {
  std::uniform_real_distribution<double> U(0.0, 1.0);
  std::vector<Cyl> out;
  for (int tries = 0; (int)out.size() < n && tries < 200000; ++tries) {
    Cyl c{U(rng) * a, U(rng) * a, rmin + (rmax - rmin) * U(rng)};
    bool ok = true;
    for (const Cyl &o : out) {
      double dx = std::fabs(c.x - o.x), dy = std::fabs(c.y - o.y);
      dx = dx > a / 2 ? a - dx : dx;
      dy = dy > a / 2 ? a - dy : dy;
      if (dx * dx + dy * dy < (c.r + o.r) * (c.r + o.r) * 1.0001) {
        ok = false;
        break;
      }
    }
    if (ok) out.push_back(c);
  }
  return out;
}

}  // namespace

int main(int argc, char **argv) {
  const int samples = argc > 1 ? std::atoi(argv[1]) : 20000;
  const size_t budgets[] = {0, 45670, 16000};
  std::mt19937_64 rng(20261204);
  int rc = 0;
  for (double f : {0.4, 0.55, 0.7})
    for (double r_um : {1.5, 4.0}) {
      const double r = r_um * 1e-3;
      const double d = std::sqrt(2.0 * kPi * r * r / (std::sqrt(3.0) * f));
      const double h = d * 0.86602540378443864676;
      const std::vector<Cyl> hex = {{d / 2, 0.0, r}, {0.0, h, r}, {d / 2, 2 * h, r}, {d, h, r}};
      char name[64];
      std::snprintf(name, sizeof name, "hex_f%.2f_r%.1f", f, r_um);
      for (size_t b : budgets) rc |= check(name, d, 2 * h, hex, b, samples, rng);
    }
  for (int n : {12, 60}) {
    const double a = 0.03;
    const std::vector<Cyl> pack = random_pack(a, n, 0.0008, 0.0025, rng);
    char name[64];
    std::snprintf(name, sizeof name, "random_%zu", pack.size());
    for (size_t b : budgets) rc |= check(name, a, a, pack, b, samples, rng);
  }
  for (int n : {6, 30}) {
    const double a = 0.03;
    std::vector<Cyl> pack;
    std::uniform_real_distribution<double> U(0.0, 1.0);
    for (int tries = 0; (int)pack.size() < n && tries < 200000; ++tries) {
      Cyl c{U(rng) * a, U(rng) * a, 0.002 + 0.003 * U(rng)};
      c.z = U(rng) * a;
      c.sphere = true;
      bool ok = true;
      for (const Cyl &o : pack) {
        double d2 = 0.0;
        for (double v : {c.x - o.x, c.y - o.y, c.z - o.z}) {
          v = std::fabs(v);
          v = v > a / 2 ? a - v : v;
          d2 += v * v;
        }
        if (d2 < (c.r + o.r) * (c.r + o.r) * 1.0001) {
          ok = false;
          break;
        }
      }
      if (ok) pack.push_back(c);
    }
    char name[64];
    std::snprintf(name, sizeof name, "spheres_%zu", pack.size());
    rc |= check(name, a, a, pack, 0, samples, rng);
  }
  std::printf("done\n");
  return rc;
}
