// oracle.cpp -- CPU oracle of the axonexa random-walker phase path.
//
// TEST INFRASTRUCTURE ONLY (the checker; see oracle.h).  Compile with
// -ffp-contract=off so that no multiply-add is fused behind the code's back:
// every fused operation here is an explicit std::fma.
//
// Reference citations are to the axonexa project tree (src/...).
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <limits>
#include <map>
#include <thread>
#include <type_traits>
#include <vector>

namespace {

const double kPI = 3.1415926535897932384626433832795;  // examples/*.cu PI
const double kGAMMA = 267500.0;                          // examples/gammadist.cu:5

// ---------------------------------------------------------------- Philox ---
// Philox4x32-10 (Salmon et al., SC'11): multipliers 0xD2511F53, 0xCD9E8D57,
// Weyl increments 0x9E3779B9, 0xBB67AE85.
void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = (uint32_t)p1;
    c[2] = n2;
    c[3] = (uint32_t)p0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

// The per-walker stream: word k = Philox(key = seed, ctr = (k/4, 0, w_lo,
// w_hi))[k % 4]; draws start at word 1.  This is what the reference's
// curandState stands for (curand_init(seed, tid, 0), kernelSetup.cuh:1-5).
struct Stream {
  uint64_t seed, walker;
  uint32_t word;  // next word index
  uint32_t cached_blk = 0xffffffffu;
  uint32_t buf[4];
  uint32_t next_word() {
    const uint32_t blk = word >> 2;
    if (blk != cached_blk) {
      uint32_t c[4] = {blk, 0u, (uint32_t)walker, (uint32_t)(walker >> 32)};
      philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
      std::memcpy(buf, c, 16);
      cached_blk = blk;
    }
    return buf[word++ & 3u];
  }
  // curand_uniform stand-in: ((x >> 9) + 1/2) * 2^-23, a float in (0, 1)
  float uniform() { return (float)(next_word() >> 9) * 1.1920928955078125e-07f + 5.9604644775390625e-08f; }
};

// ------------------------------------------------------------- sequences ---
struct V3 {
  double x, y, z;
};
V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 operator*(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
V3 operator/(V3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }  // vector3.cuh:155-158
double mag(V3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }

// G(t) of one sequence: RectGrad :36-54, CosGFunc :94-113, SinGFunc
// :148-167, ApodCosGFunc :202-228, SWOGSEFunc :265-283 (gfunctors.cuh).  The
// square wave uses (-1)^floor(2 t nu); the reference's pow(-1., 2 t nu) is
// NaN for non-integer exponents.
V3 gfunc(const orc_sequence &q, double time) {
  const V3 gh = {q.gx, q.gy, q.gz};
  const double G = q.G, dur = q.duration, sp = q.spacing;
  const double n = (double)q.num_periods;
  auto amp = [&](double t) -> double {
    switch (q.kind) {
      case 1: return std::cos(2.0 * kPI * t / (dur / n));
      case 2: return std::sin(2.0 * kPI * t / (dur / n));
      case 3: {
        const double period = dur / n;
        if (t >= period / 4.0 && t < dur - period / 4.0) return std::cos(2.0 * kPI * t / period);
        return std::sin(4.0 * kPI * t / period);
      }
      case 4: {
        const double k = std::floor(2.0 * t * (n / dur));
        return std::fmod(k, 2.0) != 0.0 ? -1.0 : 1.0;
      }
    }
    return 1.0;
  };
  if (q.kind == 0) {
    if (time < dur) return gh * G;
    if (time >= sp + dur && time < 2.0 * dur + sp) return gh * -G;
    return gh * 0.0;
  }
  if (time < dur) return (gh * G) * amp(time);
  if (time >= sp + dur && time < 2.0 * dur + sp) return (gh * -G) * amp(time - sp - dur);
  return {0.0, 0.0, 0.0};
}

// ----------------------------------------------------- reference geometry ---
// Cylinder_XY (cylinderXY.cuh) and Sphere (Sphere.cuh) in FP64 with the
// reference's operation order.
int sgn(double v) { return (0.0 < v) - (v < 0.0); }  // misc.cuh:3

struct RefBasis {
  const orc_basis *b;
  bool sph() const { return b->type == 1; }
  bool plane() const { return b->type == 2; }
  bool inside(V3 r) const {  // cylinderXY.cuh:69-74, Sphere.cuh:89-94
    // Plane (plane.cuh:1-40) defines no inside; Lattice's region, D and T2
    // lookups pass over it to the next basis or the lattice
    if (plane()) return false;
    const double cx = b->cx, cy = b->cy, cz = b->cz, R = b->radius;
    if (sph())
      return (r.x - cx) * (r.x - cx) + (r.y - cy) * (r.y - cy) + (r.z - cz) * (r.z - cz) < R * R;
    return (r.x - cx) * (r.x - cx) + (r.y - cy) * (r.y - cy) < R * R;
  }
  // cylinderXY.cuh:82-122, Sphere.cuh:102-139
  bool intersect(V3 ri, V3 rf, double &v) const {
    if (plane()) {  // plane.cuh:19-28 (doub_equal: |x| < 1e-14)
      const V3 dr = rf - ri;
      const V3 n{b->nx, b->ny, b->nz}, pdr = V3{b->cx, b->cy, b->cz} - ri;
      v = dot(n, pdr) / dot(n, dr);
      return v > 0.0 && v < 1.0 && !(std::fabs(v * mag(dr) - 0.0) < 1e-14);
    }
    const double cx = b->cx, cy = b->cy, cz = b->cz, R = b->radius;
    const V3 dr = rf - ri;
    const double step_mag = mag(dr);
    double a, bb, c;
    if (sph()) {
      a = dr.x * dr.x + dr.y * dr.y + dr.z * dr.z;
      bb = 2.0 * ri.x * dr.x - 2.0 * dr.x * cx + 2.0 * ri.y * dr.y - 2.0 * dr.y * cy +
           2.0 * ri.z * dr.z - 2.0 * dr.z * cz;
      c = ri.x * ri.x + ri.y * ri.y + ri.z * ri.z - 2 * ri.x * cx - 2 * ri.y * cy - 2 * ri.z * cz +
          cx * cx + cy * cy + cz * cz - R * R;
    } else {
      a = dr.x * dr.x + dr.y * dr.y;
      bb = 2.0 * ri.x * dr.x - 2.0 * dr.x * cx + 2.0 * ri.y * dr.y - 2.0 * dr.y * cy;
      c = ri.x * ri.x + ri.y * ri.y - 2.0 * ri.x * cx - 2.0 * ri.y * cy + cx * cx + cy * cy -
          R * R;
    }
    const double q = -.5 * (bb + sgn(bb) * std::sqrt(bb * bb - 4 * a * c));
    const double root1 = q / a, root2 = c / q;
    const double eps = b->eps;
    const bool s1 = root1 > 0.0 && root1 < 1.0 && bb * bb > 4 * a * c &&
                    !(std::fabs(root1 * step_mag - 0.0) < eps);
    const bool s2 = root2 > 0.0 && root2 < 1.0 && bb * bb > 4 * a * c &&
                    !(std::fabs(root2 * step_mag - 0.0) < eps);
    const bool s3 = std::fabs(root1) < std::fabs(root2);
    if ((s1 && s2 && s3) || (s1 && !s2)) {
      v = root1;
      return true;
    }
    if ((s1 && s2 && !s3) || (s2 && !s1)) {
      v = root2;
      return true;
    }
    return false;
  }
  V3 normal(V3 r) const {  // cylinderXY.cuh:125-131, Sphere.cuh:142-149
    if (plane()) return {b->nx, b->ny, b->nz};  // plane.cuh:32
    const double nx = r.x - b->cx, ny = r.y - b->cy;
    if (sph()) {
      const double nz = r.z - b->cz;
      const double m = std::sqrt(nx * nx + ny * ny + nz * nz);
      return {nx / m, ny / m, nz / m};
    }
    const double m = std::sqrt(nx * nx + ny * ny);
    return {nx / m, ny / m, 0.0};
  }
};

// Lattice (lattice.cuh:3-254) over the listed bases only.
struct RefLattice {
  double a, b, c, D, T2;
  std::vector<RefBasis> B;
  void lmod(V3 &r) const {  // :66-88
    if (r.x > a) r.x = std::fmod(r.x, a);
    if (r.x < 0.0) r.x = std::fmod(r.x, a) + a;
    if (r.y > b) r.y = std::fmod(r.y, b);
    if (r.y < 0.0) r.y = std::fmod(r.y, b) + b;
    if (r.z > c) r.z = std::fmod(r.z, c);
    if (r.z < 0.0) r.z = std::fmod(r.z, c) + c;
  }
  bool in_cell(V3 r) const {  // :150-156
    return !(r.x > a || r.x < 0.0 || r.y > b || r.y < 0.0 || r.z > c || r.z < 0.0);
  }
  void correct(V3 &r) const {  // :60-64
    if (!in_cell(r)) lmod(r);
  }
  double getD(V3 r) const {  // :118-132 (a basis counts if its value is > 0)
    lmod(r);
    for (auto &q : B)
      if (q.inside(r) && q.b->D > 0) return q.b->D;
    return D;
  }
  double getT2(V3 r) const {  // :90-102
    lmod(r);
    for (auto &q : B)
      if (q.inside(r) && q.b->T2 > 0) return q.b->T2;
    return T2;
  }
  int first_inside(V3 r) const {  // index form of inRegion (:134-148)
    lmod(r);
    for (size_t i = 0; i < B.size(); ++i)
      if (B[i].inside(r)) return (int)i;
    return -1;
  }
  int region(V3 r) const {
    const int i = first_inside(r);
    return i < 0 ? 0 : B[i].b->region;
  }
  // intersectionCheckPermeable / Impermeable (:158-247)
  bool check(V3 ri, V3 rf, double &v, V3 &n, double &perm) const {
    const V3 dr = rf - ri;
    V3 m1f = rf;
    lmod(m1f);
    const V3 m1i = m1f - dr;
    V3 m2i = ri;
    lmod(m2i);
    const V3 m2f = m2i + dr;
    double vt = 0.0, best = 10.0;
    for (auto &q : B) {
      if (q.intersect(m1i, m1f, vt) && vt < best) {
        best = vt;
        n = q.normal(dr * best + m1i);
        perm = q.b->permeability;
      }
      if (q.intersect(m2i, m2f, vt) && vt < best) {
        best = vt;
        n = q.normal(dr * best + m2i);
        perm = q.b->permeability;
      }
    }
    v = best;
    return best < 5.0;
  }
};

// --------------------------------------------------------- kernel geometry ---
// The GPU kernel's formulation (axonexa_gb300/csrc/walk_kernel.cuh restated):
// instances = bases plus periodic ghosts, centre-relative quadratic in the
// distance along the unit direction, last-hit instance tested on its surface.
template <typename T>
T fmaT(T a, T b, T c) {
  return std::fma(a, b, c);
}

template <typename T>
struct KInst {
  T cx, cy, cz, negR2, invR, eps;  // a plane: (cx, cy, cz) = unit normal, negR2 = n.c
  int slot;
  bool sph, plane;
};

template <typename T>
struct KGeom {
  std::vector<KInst<T>> inst;
  std::vector<T> speed, step, t2term, kappa4;
  std::vector<int> region;
  int ecs = 0;
  T a = 0, b = 0, c = 0;
};

template <typename T>
T c0_of(const KInst<T> &g, T x, T y, T z) {
  const T px = x - g.cx, py = y - g.cy;
  if (g.sph) {
    const T pz = z - g.cz;
    return fmaT(px, px, fmaT(py, py, fmaT(pz, pz, g.negR2)));
  }
  return fmaT(px, px, fmaT(py, py, g.negR2));
}

template <typename T>
int k_lookup(const KGeom<T> &G, T x, T y, T z) {
  for (const auto &g : G.inst)
    if (!g.plane && c0_of(g, x, y, z) < T(0)) return g.slot;
  return G.ecs;
}

template <typename T>
T k_seg_hit(const KInst<T> &g, bool on_surface, T sx, T sy, T sz, T dx, T dy, T dz, T aa, T rem) {
  const T inf = std::numeric_limits<T>::infinity();
  if (g.plane) {  // (n.c - n.s) / n.d along the unit direction
    if (on_surface) return inf;
    const T np = fmaT(g.cx, sx, fmaT(g.cy, sy, g.cz * sz));
    const T dn = fmaT(g.cx, dx, fmaT(g.cy, dy, g.cz * dz));
    const T s = (g.negR2 - np) / dn;
    if (!(s > T(0) && s < rem && s >= g.eps)) return inf;
    return s;
  }
  const T px = sx - g.cx, py = sy - g.cy;
  const T pz = g.sph ? (sz - g.cz) : T(0);
  T bh, c0, c1;
  const T ex = fmaT(rem, dx, px), ey = fmaT(rem, dy, py);
  if (g.sph) {
    const T ez = fmaT(rem, dz, pz);
    bh = fmaT(px, dx, fmaT(py, dy, pz * dz));
    c0 = fmaT(px, px, fmaT(py, py, fmaT(pz, pz, g.negR2)));
    c1 = fmaT(ex, ex, fmaT(ey, ey, fmaT(ez, ez, g.negR2)));
  } else {
    bh = fmaT(px, dx, py * dy);
    c0 = fmaT(px, px, fmaT(py, py, g.negR2));
    c1 = fmaT(ex, ex, fmaT(ey, ey, g.negR2));
  }
  if (on_surface) c0 = T(0);
  T s;
  if (c0 < T(0)) {
    if (c1 < T(0)) return inf;
    const T disc = fmaT(bh, bh, -(aa * c0));
    const T sq = std::sqrt(disc);
    s = (bh <= T(0)) ? (sq - bh) / aa : (-c0) / (bh + sq);
  } else if (c0 > T(0)) {
    if (bh >= T(0)) return inf;
    if (c1 > T(0) && fmaT(aa, rem, bh) <= T(0)) return inf;
    const T disc = fmaT(bh, bh, -(aa * c0));
    if (disc <= T(0)) return inf;
    const T sq = std::sqrt(disc);
    s = c0 / (sq - bh);
  } else {
    if (bh >= T(0)) return inf;
    s = (T(-2) * bh) / aa;
  }
  if (!(s > T(0) && s < rem && s >= g.eps)) return inf;
  return s;
}

template <typename T>
struct KMove {
  T fx, fy, fz;
  int hits;
  bool capped;
  bool crossed;  // transmitted through a permeable wall
};

template <typename T>
// L: length of the move's segment; Lb: its path budget, which replaces the
// segment length at the first hit (they differ for lattice picking, whose
// diagonal segment is sqrt(3) L long while boundaryNormal budgets
// speed * (dt - t_hit)).
KMove<T> k_boundary(const KGeom<T> &G, T sx, T sy, T sz, T dx, T dy, T dz, T L, T v, bool perm,
                    Stream &st, T Lb) {
  KMove<T> o{T(0), T(0), T(0), 0, false, false};
  T rem = L;
  int last = -1;
  for (;;) {
    const T aa_c = fmaT(dx, dx, dy * dy);
    const T aa_s = fmaT(dx, dx, fmaT(dy, dy, dz * dz));
    T best = std::numeric_limits<T>::infinity();
    int bk = -1;
    for (size_t k = 0; k < G.inst.size(); ++k) {
      const KInst<T> &g = G.inst[k];
      const T s = k_seg_hit(g, (int)k == last, sx, sy, sz, dx, dy, dz, g.sph ? aa_s : aa_c, rem);
      if (s < best) {
        best = s;
        bk = (int)k;
      }
    }
    if (bk < 0) break;
    if (o.hits == 1024) {  // the kernel's reflection cap
      o.capped = true;
      o.fx = sx;
      o.fy = sy;
      o.fz = sz;
      return o;
    }
    const T hx = fmaT(best, dx, sx), hy = fmaT(best, dy, sy), hz = fmaT(best, dz, sz);
    const T rem_before = rem;
    rem = (o.hits == 0 ? Lb : rem) - best;
    ++o.hits;
    const KInst<T> &g = G.inst[bk];
    if (perm) {
      const T u = (T)st.uniform();
      const T ptr = G.kappa4[g.slot] / v;
      if (!(u > ptr)) {
        const T tx = fmaT(rem_before, dx, sx), ty = fmaT(rem_before, dy, sy),
                tz = fmaT(rem_before, dz, sz);
        const int ts = k_lookup(G, tx, ty, tz);
        const T remt = (rem * G.speed[ts]) / v;
        o.fx = fmaT(remt, dx, hx);
        o.fy = fmaT(remt, dy, hy);
        o.fz = fmaT(remt, dz, hz);
        o.crossed = true;
        return o;
      }
    }
    const bool n3 = g.sph || g.plane;
    const T nx = g.plane ? g.cx : (hx - g.cx) * g.invR;
    const T ny = g.plane ? g.cy : (hy - g.cy) * g.invR;
    const T nz = g.plane ? g.cz : (g.sph ? (hz - g.cz) * g.invR : T(0));
    const T dn = n3 ? fmaT(dx, nx, fmaT(dy, ny, dz * nz)) : fmaT(dx, nx, dy * ny);
    const T t = T(-2) * dn;
    dx = fmaT(t, nx, dx);
    dy = fmaT(t, ny, dy);
    if (n3) dz = fmaT(t, nz, dz);
    sx = hx;
    sy = hy;
    sz = hz;
    last = bk;
  }
  o.fx = fmaT(rem, dx, sx);
  o.fy = fmaT(rem, dy, sy);
  o.fz = fmaT(rem, dz, sz);
  return o;
}

// sin/cos(2*pi*u): quadrant reduction of u and Taylor polynomials of
// sin(2*pi*f), cos(2*pi*f), |f| <= 1/8, coefficients (2*pi)^k/k! rounded to
// the working precision.
template <typename T>
void k_sincos_2pi(T u, T &s, T &c) {
  const T q = std::nearbyint(u * T(4));
  const T f = fmaT(q, T(-0.25), u);
  const T f2 = f * f;
  T ps, pc;
  if (std::is_same<T, float>::value) {
    ps = fmaT(f2, (T)0x1.5078340p+5f, (T)-0x1.32d2ccp+6f);
    ps = fmaT(f2, ps, (T)0x1.466bc6p+6f);
    ps = fmaT(f2, ps, (T)-0x1.4abbcep+5f);
    ps = fmaT(f2, ps, (T)0x1.921fb6p+2f);
    pc = fmaT(f2, (T)-0x1.a6d1f2p+4f, (T)0x1.e1f506p+5f);
    pc = fmaT(f2, pc, (T)-0x1.55d3c8p+6f);
    pc = fmaT(f2, pc, (T)0x1.03c1f0p+6f);
    pc = fmaT(f2, pc, (T)-0x1.3bd3ccp+4f);
  } else {
    // FP64: more terms of the same series
    const double tp = 2.0 * kPI;
    double cs_[9], cc_[9];
    double fac = 1.0, pw = 1.0;
    int ns = 0, nc = 0;
    for (int k = 0; k <= 17; ++k) {
      if (k > 0) {
        fac *= k;
        pw *= tp;
      }
      const double term = pw / fac * (((k / 2) % 2) ? -1.0 : 1.0);
      if (k % 2) cs_[ns++] = term;
      else cc_[nc++] = term;
    }
    T a = (T)cs_[ns - 1];
    for (int k = ns - 2; k >= 0; --k) a = fmaT(f2, a, (T)cs_[k]);
    ps = a;
    T b = (T)cc_[nc - 1];
    for (int k = nc - 2; k >= 1; --k) b = fmaT(f2, b, (T)cc_[k]);
    pc = b;
  }
  const T sn = f * ps;
  const T cs = fmaT(f2, pc, T(1));
  const int qi = ((int)q) & 3;
  const T s1 = (qi & 1) ? cs : sn;
  const T c1 = (qi & 1) ? sn : cs;
  s = (qi & 2) ? -s1 : s1;
  c = ((qi + 1) & 2) ? -c1 : c1;
}

template <typename T>
void k_direction(T u1, T u2, T &dx, T &dy, T &dz) {
  T sp, cp;
  k_sincos_2pi(u1, sp, cp);
  const T z = fmaT(T(2), u2, T(-1));
  const T st = std::sqrt(fmaT(-z, z, T(1)));
  dx = st * cp;
  dy = st * sp;
  dz = z;
}

template <typename T>
T k_wrap(T x, T a) {
  if (x > a) return x - a;
  if (x < T(0)) return x + a;
  return x;
}

// Kernel geometry: slot tables (speed, step, dt/T2, 4 kappa) from FP64
// formulas rounded to T, bases then all periodic ghosts that coincide with no
// listed basis.
template <typename T>
void k_build(const orc_lattice *lat, const orc_basis *basis, int nbasis, double dt, bool relax,
             bool single, KGeom<T> &G) {
  auto slot = [&](double D, double T2, double kappa) {
    const double sp = std::sqrt(6.0 * D / dt);
    G.speed.push_back((T)sp);
    G.step.push_back((T)(sp * dt));
    G.t2term.push_back((relax && T2 > 0.0) ? (T)(dt / T2) : T(0));
    G.kappa4.push_back((T)(4.0 * kappa));
  };
  for (int k = 0; k < nbasis; ++k) {
    if (basis[k].type == 2) slot(lat->D, lat->T2, 0.0);  // a plane transmits nothing
    else slot(basis[k].D, basis[k].T2, basis[k].permeability);
    G.region.push_back(basis[k].region);
  }
  if (single) slot(basis[0].D, basis[0].T2, 0.0);
  else slot(lat->D, lat->T2, 0.0);
  G.region.push_back(0);
  G.ecs = nbasis;
  auto unit = [](const orc_basis &b, double n[3]) {
    const double m = std::sqrt(b.nx * b.nx + b.ny * b.ny + b.nz * b.nz);
    n[0] = b.nx / m;
    n[1] = b.ny / m;
    n[2] = b.nz / m;
  };
  auto add = [&](int k, double cx, double cy, double cz) {
    const orc_basis &b = basis[k];
    KInst<T> g;
    g.plane = b.type == 2;
    if (g.plane) {
      double n[3];
      unit(b, n);
      g.cx = (T)n[0];
      g.cy = (T)n[1];
      g.cz = (T)n[2];
      g.negR2 = (T)(n[0] * cx + n[1] * cy + n[2] * cz);
      g.invR = T(1);
    } else {
      g.cx = (T)cx;
      g.cy = (T)cy;
      g.cz = (T)cz;
      g.negR2 = (T)(-(b.radius * b.radius));
      g.invR = (T)(1.0 / b.radius);
    }
    g.eps = (T)b.eps;
    g.slot = k;
    g.sph = b.type == 1;
    G.inst.push_back(g);
  };
  if (single) {
    add(0, basis[0].cx, basis[0].cy, basis[0].cz);
    return;
  }
  G.a = (T)lat->a;
  G.b = (T)lat->b;
  G.c = (T)lat->c;
  const double A = lat->a, B = lat->b, C = lat->c;
  const double tol = 1e-9 * std::max(A, std::max(B, C));
  for (int k = 0; k < nbasis; ++k) {
    const orc_basis &b = basis[k];
    add(k, b.cx, b.cy, b.cz);
    const int zr = b.type == 0 ? 0 : 1;
    for (int i = -1; i <= 1; ++i)
      for (int j = -1; j <= 1; ++j)
        for (int l = -zr; l <= zr; ++l) {
          if (i == 0 && j == 0 && l == 0) continue;
          const double cx = b.cx + A * i, cy = b.cy + B * j, cz = b.cz + C * l;
          bool dup = false;
          for (int o = 0; o < nbasis && !dup; ++o) {
            const orc_basis &q = basis[o];
            if (q.type != b.type) continue;
            if (b.type == 2) {  // the same plane: parallel normals, the point on it
              double n[3], m[3];
              unit(q, n);
              unit(b, m);
              const double cr = std::fabs(n[1] * m[2] - n[2] * m[1]) +
                                std::fabs(n[2] * m[0] - n[0] * m[2]) +
                                std::fabs(n[0] * m[1] - n[1] * m[0]);
              const double d = n[0] * (cx - q.cx) + n[1] * (cy - q.cy) + n[2] * (cz - q.cz);
              dup = cr < 1e-12 && std::fabs(d) <= tol;
              continue;
            }
            if (std::fabs(q.radius - b.radius) > tol) continue;
            if (std::fabs(q.cx - cx) > tol || std::fabs(q.cy - cy) > tol) continue;
            if (b.type == 1 && std::fabs(q.cz - cz) > tol) continue;
            dup = true;
          }
          if (!dup) add(k, cx, cy, cz);
        }
  }
}

// ------------------------------------------------------------- one walker ---
struct WalkIn {
  const orc_lattice *lat;
  const orc_basis *basis;
  int nbasis;
  const orc_sequence *seqs;
  int nseq;
  const orc_params *p;
  double gamma;
  bool single, relax, perm, reject;
  bool pick = false;  // LATTICE_PICKING (single pore): +-L steps along each axis
};

struct WalkOut {
  std::vector<double> phase;
  double t2factor = 0.0;  // the value whose exp weights the signal
  int64_t caps = 0;
  bool start_in = false;  // lattice walks: the start lies inside a basis (region != 0)
};

struct TraceRow {
  double *init_pos, *pos;
  int32_t *region, *hits, *words;
};

// Reference-order FP64 walk: updateWalkersLatticePhase
// (kernelLattice.cuh:1-104) or updateWalkersPhase (kernelPhase.cuh:4-66).
// on_move (optional) sees the start (i = 0) and the position after every
// move i (bounded for the single pore, wrapped for lattices).
void walk_ref(const WalkIn &in, const RefLattice &L, int64_t w, WalkOut &out, TraceRow *tr,
              const std::function<void(int, const V3 &)> *on_move = nullptr) {
  const orc_params &p = *in.p;
  const double dt = p.timestep;
  Stream st{p.seed, (uint64_t)(w + p.walker_offset), 1u};
  V3 r{0, 0, 0};
  if (in.single) {
    // Basis::unifRand(curandState) by value: draws on a copy of the stream
    // (cylinderXY.cuh:45-55, Sphere.cuh:55-63)
    Stream cp = st;
    const orc_basis &b = in.basis[0];
    const RefBasis rb{&b};
    if (b.type == 1) {
      const double R = b.radius;
      // first draw: three statements x, y, z (Sphere.cuh:57-59); retries pass
      // three draws as Vector3 constructor arguments (:62-64), an evaluation
      // order C++ leaves unspecified -- drawn here z, y, x, as the compiled
      // reference consumes them
      r.x = R * (2.0 * cp.uniform() - 1);
      r.y = R * (2.0 * cp.uniform() - 1);
      r.z = R * (2.0 * cp.uniform() - 1);
      for (int t = 0; t < 100000 && !rb.inside(r); ++t) {
        r.z = R * (2.0 * cp.uniform() - 1);
        r.y = R * (2.0 * cp.uniform() - 1);
        r.x = R * (2.0 * cp.uniform() - 1);
      }
    } else {
      const double R = b.radius;
      for (int t = 0; t < 100000; ++t) {
        r.x = R * (2.0 * cp.uniform() - 1) + b.cx;
        r.y = R * (2.0 * cp.uniform() - 1) + b.cy;
        r.z = 2.0 * R * cp.uniform();
        if (rb.inside(r)) break;
      }
    }
  } else if (p.init_mode == 2) {
    // Basis::randUnif (cylinderXY.cuh:176-183, Sphere.cuh:384-391)
    const orc_basis &b = in.basis[p.init_arg];
    const RefBasis rb{&b};
    const V3 cen = {b.cx, b.cy, b.type == 1 ? b.cz : 0.0};
    for (int t = 0; t < 100000; ++t) {
      // constructor arguments: drawn z, y, x (see the single-pore sphere above)
      const double z = (2.0 * st.uniform() - 1.0) * b.radius;
      const double y = (2.0 * st.uniform() - 1.0) * b.radius;
      const double x = (2.0 * st.uniform() - 1.0) * b.radius;
      r = V3{x, y, z} + cen;
      if (rb.inside(r)) break;
    }
  } else {
    // Lattice::initializeUniformly / initializeInRegion (lattice.cuh:31-58)
    for (int t = 0; t < 100000; ++t) {
      r.x = st.uniform() * L.a;
      r.y = st.uniform() * L.b;
      r.z = st.uniform() * L.c;
      if (p.init_mode == 0 || L.region(r) == p.init_arg) break;
    }
  }
  if (tr) {
    tr->init_pos[0] = r.x;
    tr->init_pos[1] = r.y;
    tr->init_pos[2] = r.z;
  }
  V3 ru = r;
  out.start_in = !in.single && L.region(r) != 0;
  if (on_move) (*on_move)(0, r);
  for (int j = 0; j < in.nseq; ++j) out.phase[j] = in.gamma * dot(gfunc(in.seqs[j], 0.0), r) * dt;
  double T2f = 0.0;
  const orc_basis *b0 = in.single ? &in.basis[0] : nullptr;
  const double speed0 = in.single ? std::sqrt(6.0 * b0->D / dt) : 0.0;
  for (int i = 1; i < p.steps; ++i) {
    V3 ri = r;
    const double speed = in.single ? speed0 : std::sqrt(6.0 * L.getD(r) / dt);
    if (in.pick) {
      // LATTICE_PICKING (kernelPhase.cuh:31-35): stepLength * randomSign per
      // axis, randomSign = curand % 2 ? 1 : -1 (kernelSetup.cuh:13-15); the
      // three draws are Vector3 constructor arguments, consumed z, y, x
      const double stepLength = speed * dt;
      const double sz = (st.next_word() % 2) ? 1 : -1;
      const double sy = (st.next_word() % 2) ? 1 : -1;
      const double sx = (st.next_word() % 2) ? 1 : -1;
      r = r + V3{stepLength * sx, stepLength * sy, stepLength * sz};
    } else {
      const double phi = 2.0 * kPI * st.uniform();
      const double theta = std::acos(2.0 * st.uniform() - 1);
      r = r + V3{speed * dt * std::sin(theta) * std::cos(phi),
                 speed * dt * std::sin(theta) * std::sin(phi), speed * dt * std::cos(theta)};
    }
    int hits = 0;
    if (in.single) {
      const RefBasis rb{b0};
      if (!in.reject) {
        // boundaryNormal (boundaryCheck.cuh:2-32)
        double v = 0.0, acc = 0.0;
        while (rb.intersect(ri, r, v)) {
          ++hits;
          r = (r - ri) * v + ri;
          const V3 I = r - ri;
          const double Im = mag(I);
          acc += Im / speed;
          const V3 n = rb.normal(r);
          ri = r;
          r = r + ((I - (n * 2.0) * dot(n, I)) * (speed / Im)) * (dt - acc);
        }
      } else if (!rb.inside(r)) {
        r = ri;
      }
    } else if (in.reject) {
      if (L.region(ri) != L.region(r)) r = ri;  // kernelLattice.cuh:75-77
    } else if (!in.perm) {
      // boundaryCheckImpermeable (boundaryCheck.cuh:34-64)
      double v = 0.0, acc = 0.0, pm = 0.0;
      V3 n{0, 0, 0}, rc = ri;
      while (L.check(rc, r, v, n, pm)) {
        ++hits;
        r = (r - rc) * v + rc;
        const V3 I = r - rc;
        const double Im = mag(I);
        acc += Im / speed;
        rc = r;
        r = r + ((I - (n * 2.0) * dot(n, I)) * (speed / Im)) * (dt - acc);
      }
    } else {
      // boundaryCheckPermeable (boundaryCheck.cuh:66-113); accumtime enters
      // by value, so the T2 weighting below sees 0 (kernelLattice.cuh:66-68)
      double v = 0.0, acc = 0.0, pm = 0.0;
      V3 n{0, 0, 0}, rc = ri;
      bool transmitted = false;
      const double cur = std::sqrt(6.0 * L.getD(ri) / dt);
      while (L.check(rc, r, v, n, pm) && transmitted == false) {
        ++hits;
        const double trs = std::sqrt(6.0 * L.getD(r) / dt);
        r = (r - rc) * v + rc;
        const V3 I = r - rc;
        const double Im = mag(I);
        acc += Im / cur;
        if (st.uniform() > pm * 4.0 / cur) {
          rc = r;
          r = r + ((I - (n * 2.0) * dot(n, I)) * (cur / Im)) * (dt - acc);
        } else {
          r = r + ((I / Im) * trs) * (dt - acc);
          transmitted = true;
        }
      }
    }
    const V3 pos_for_phase = in.single ? r : (ru = ru + (r - ri), ru);
    for (int j = 0; j < in.nseq; ++j)
      out.phase[j] += in.gamma * dot(gfunc(in.seqs[j], dt * i), pos_for_phase) * dt;
    if (in.relax) {
      if (in.perm) T2f += (0.0 / L.getT2(ri)) + ((dt - 0.0) / L.getT2(r));
      else T2f += dt / L.getT2(ri);
    }
    if (!in.single) L.correct(r);
    if (on_move) (*on_move)(i, r);
    if (tr) {
      const size_t o = (size_t)(i - 1);
      tr->pos[o * 3 + 0] = r.x;
      tr->pos[o * 3 + 1] = r.y;
      tr->pos[o * 3 + 2] = r.z;
      tr->region[o] = in.single ? (RefBasis{b0}.inside(r) ? 0 : -1) : L.first_inside(r);
      tr->hits[o] = hits;
      tr->words[o] = (int32_t)st.word;
    }
  }
  out.t2factor = T2f;
}

// Kernel-formulation walk in T (float: the GPU kernel bit for bit).
template <typename T>
void walk_kern(const WalkIn &in, const KGeom<T> &G, int64_t w, WalkOut &out, TraceRow *tr) {
  const orc_params &p = *in.p;
  const double dt = p.timestep;
  Stream st{p.seed, (uint64_t)(w + p.walker_offset), 1u};
  T x = 0, y = 0, z = 0;
  auto U = [](Stream &s) { return (T)s.uniform(); };
  if (in.single || p.init_mode == 2) {
    const int k = in.single ? 0 : p.init_arg;
    const orc_basis &b = in.basis[k];
    const KInst<T> *g = nullptr;
    for (auto &q : G.inst)
      if (q.slot == k) {
        g = &q;
        break;
      }
    const T R = (T)b.radius, cx = (T)b.cx, cy = (T)b.cy, cz = (T)b.cz;
    const bool sph = b.type == 1;
    Stream cp = st;
    Stream &s = in.single ? cp : st;
    auto draw = [&](T c) { return fmaT(fmaT(T(2), U(s), T(-1)), R, c); };
    if (in.single) {
      x = draw(cx);
      y = draw(cy);
      z = sph ? draw(cz) : (T(2) * R) * U(s);
      for (int t = 0; t < 100000 && !(c0_of(*g, x, y, z) < T(0)); ++t) {
        if (sph) {
          z = draw(cz);
          y = draw(cy);
          x = draw(cx);
        } else {
          x = draw(cx);
          y = draw(cy);
          z = (T(2) * R) * U(s);
        }
      }
    } else {
      for (int t = 0; t < 100000; ++t) {
        const T tz = fmaT(T(2), U(s), T(-1));
        y = draw(cy);
        x = draw(cx);
        z = sph ? fmaT(tz, R, cz) : tz * R;
        if (c0_of(*g, x, y, z) < T(0)) break;
      }
    }
  } else {
    for (int t = 0; t < 100000; ++t) {
      x = U(st) * G.a;
      y = U(st) * G.b;
      z = U(st) * G.c;
      if (p.init_mode == 0 || G.region[k_lookup(G, x, y, z)] == p.init_arg) break;
    }
  }
  if (tr) {
    tr->init_pos[0] = (double)x;
    tr->init_pos[1] = (double)y;
    tr->init_pos[2] = (double)z;
  }
  T ux = x, uy = y, uz = z;
  for (int j = 0; j < in.nseq; ++j)
    out.phase[j] = in.gamma * dot(gfunc(in.seqs[j], 0.0), V3{(double)x, (double)y, (double)z}) * dt;
  T t2s = 0, t2c = 0;
  int slot = in.single ? 0 : k_lookup(G, x, y, z);
  out.start_in = !in.single && G.region[slot] != 0;
  const bool geom = !G.inst.empty();
  for (int i = 1; i < p.steps; ++i) {
    const T v = G.speed[slot], Ls = G.step[slot];
    T dx, dy, dz, Lseg = Ls;
    if (in.pick) {
      // the diagonal of the +-L cube, drawn z, y, x (words' low bits)
      const T k = (T)0.57735026918962576451;
      dz = (st.next_word() & 1u) ? k : -k;
      dy = (st.next_word() & 1u) ? k : -k;
      dx = (st.next_word() & 1u) ? k : -k;
      Lseg = Ls * (T)1.7320508075688772935;
    } else {
      const T u1 = U(st), u2 = U(st);
      k_direction(u1, u2, dx, dy, dz);
    }
    T fx, fy, fz;
    int hits = 0;
    bool crossed = false;
    if (!geom) {
      fx = fmaT(Lseg, dx, x);
      fy = fmaT(Lseg, dy, y);
      fz = fmaT(Lseg, dz, z);
    } else if (in.reject) {
      fx = fmaT(Lseg, dx, x);
      fy = fmaT(Lseg, dy, y);
      fz = fmaT(Lseg, dz, z);
      if (in.single) {
        if (!(c0_of(G.inst[0], fx, fy, fz) < T(0))) {
          fx = x;
          fy = y;
          fz = z;
        }
      } else if (G.region[k_lookup(G, fx, fy, fz)] != G.region[slot]) {
        fx = x;
        fy = y;
        fz = z;
      }
    } else {
      const KMove<T> o = k_boundary(G, x, y, z, dx, dy, dz, Lseg, v, in.perm, st, Ls);
      fx = o.fx;
      fy = o.fy;
      fz = o.fz;
      hits = o.hits;
      crossed = o.crossed;
      out.caps += o.capped ? 1 : 0;
    }
    V3 pp;
    bool wrapped = false;
    if (in.single) {
      pp = {(double)fx, (double)fy, (double)fz};
    } else {
      ux = ux + (fx - x);
      uy = uy + (fy - y);
      uz = uz + (fz - z);
      pp = {(double)ux, (double)uy, (double)uz};
      const T ox = fx, oy = fy, oz = fz;
      fx = k_wrap(fx, G.a);
      fy = k_wrap(fy, G.b);
      fz = k_wrap(fz, G.c);
      wrapped = fx != ox || fy != oy || fz != oz;
    }
    for (int j = 0; j < in.nseq; ++j) out.phase[j] += in.gamma * dot(gfunc(in.seqs[j], dt * i), pp) * dt;
    // specular lattice walks keep their region, looked up again only after a
    // move that wraps across the cell edge or crosses a permeable wall (the
    // kernel's formulation; the reference looks it up every move)
    const bool tracked = !in.single && !in.reject;
    int new_slot = slot;
    if (!in.single && geom && (!tracked || wrapped || crossed)) new_slot = k_lookup(G, fx, fy, fz);
    if (in.relax) {
      const T y2 = G.t2term[in.perm ? new_slot : slot];
      const T yy = y2 - t2c;
      const T t = t2s + yy;
      t2c = (t - t2s) - yy;
      t2s = t;
    }
    x = fx;
    y = fy;
    z = fz;
    slot = new_slot;
    if (tr) {
      const size_t o = (size_t)(i - 1);
      tr->pos[o * 3 + 0] = (double)x;
      tr->pos[o * 3 + 1] = (double)y;
      tr->pos[o * 3 + 2] = (double)z;
      int rs = slot;
      if (in.single) rs = (c0_of(G.inst[0], x, y, z) < T(0)) ? 0 : -1;
      tr->region[o] = (!in.single && rs == G.ecs) ? -1 : rs;
      tr->hits[o] = hits;
      tr->words[o] = (int32_t)st.word;
    }
  }
  out.t2factor = in.relax ? ((double)t2s - (double)t2c) : 0.0;
}

// ------------------------------------------------------ Bloch (mag) path ---
// B-field functors (src/functors/bfunctors.cuh) in FP64 with the reference's
// expressions; `gamma` stands for the GAMMA macro their constructors and
// operator() use (QSC_PGSE, UCN_lowfield).
V3 cross(const V3 &a, const V3 &b) {  // Vector3::operator% (vector3.cuh:179-183)
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

V3 bfield(const orc_field &f, double gamma, const V3 &r, double time) {
  const double B0 = f.B0, G = f.G, gd = f.duration, gs = f.spacing;
  const V3 gv{f.gx, f.gy, f.gz};
  switch (f.kind) {
    case 0:  // QSC_GRE::operator() (:29-50)
      if (time < gd) return {0.0, G * r.z, B0 + G * r.y};
      if (time >= gs + gd && time < 2.0 * gd + gs) return {0.0, -G * r.z, B0 - G * r.y};
      return {0.0, 0.0, B0};
    case 1: {  // QSC_PGSE (:72-118): B1 = PI / |GAMMA rfDuration|, w = GAMMA B0
      const double B1 = kPI / std::fabs(gamma * f.rf_duration);
      if (time < gd) return {0.0, G * r.z, B0 + G * r.y};
      if (time >= f.TE / 2.0 && time < f.TE / 2.0 + f.rf_duration) {
        const double w = gamma * B0;
        return {B1 * std::cos(w * time), -B1 * std::sin(w * time), B0};
      }
      if (time >= gs + gd && time < 2.0 * gd + gs) return {0.0, G * r.z, B0 + G * r.y};
      return {0.0, 0.0, B0};
    }
    case 2: {  // QSC_COS_GRE (:144-191): period = duration / periods
      const double period = gd / (double)f.num_periods;
      auto amp = [&](double t) { return std::cos(2.0 * kPI * t / period); };
      if (time < gd) return {0.0, G * amp(time) * r.z, B0 + G * amp(time) * r.y};
      if (time >= gs + gd && time < 2.0 * gd + gs) {
        const double te = time - gs - gd;
        return {0.0, -G * amp(te) * r.z, B0 - G * amp(te) * r.y};
      }
      return {0.0, 0.0, B0};
    }
    case 3: {  // QSC_GRE_TRAP (:224-271), ramps ampMod1/ampMod2 as written
      const double ramp = f.ramp;
      const double t1 = ramp, t2 = ramp + gd, t3 = 2.0 * t1 + t2, t4 = gs, t5 = t4 + t3;
      auto m1 = [&](double t) { return (G / ramp) * t; };
      auto m2 = [&](double t) { return G - (G / ramp) * t; };
      if (time < t1) {
        const double m = m1(time);
        return {0.0, (G * r.z) * m, B0 + (G * r.y) * m};
      } else if (time >= t1 && time < t2) {
        return {0.0, G * r.z, B0 + G * r.y};
      } else if (time >= t2 && time < t3) {
        const double m = m2(time - t2);
        return {0.0, G * r.z * m, B0 + G * r.y * m};
      } else if (time >= t5 && time < t5 + t1) {
        const double m = m1(time - t5);
        return {0.0, (G * r.z) * m, B0 + (G * r.y) * m};
      } else if (time >= t5 + t1 && time < t5 + t2) {
        return {0.0, G * r.z, B0 + G * r.y};
      } else if (time >= t5 + t2 && time < t5 + t3) {
        const double m = m2(time - t5 - t2);
        return {0.0, G * r.z * m, B0 + G * r.y * m};
      }
      return {0.0, 0.0, B0};
    }
    case 4:    // SIN_GRE (:310-328)
    case 5: {  // COS_GRE (:376-392): period = duration / periods
      const double period = f.kind == 4 ? f.period : gd / ((double)f.num_periods);
      auto amp = [&](double t) {
        return f.kind == 4 ? std::sin(2.0 * kPI * t / period) : std::cos(2.0 * kPI * t / period);
      };
      const double gr = gv.x * r.x + gv.y * r.y + gv.z * r.z;  // Vector3 * Vector3
      if (time < gd) return {0.0, 0.0, B0 + gr * amp(time)};
      if (time >= gs + gd && time < 2.0 * gd + gs) return {0.0, 0.0, B0 - gr * amp(time - gs - gd)};
      return {0.0, 0.0, B0};
    }
    case 6: {  // RECT_GRE (:417-425)
      const double gr = gv.x * r.x + gv.y * r.y + gv.z * r.z;
      if (time < gd) return {0.0, 0.0, B0 + gr};
      if (time >= gs + gd && time < 2.0 * gd + gs) return {0.0, 0.0, B0 - gr};
      return {0.0, 0.0, B0};
    }
    default: {  // UCN_lowfield (:444-466): B1 = PI / (2 |GAMMA rfDuration|), w = GAMMA B0
      const double B1 = kPI / (2.0 * std::fabs(gamma * f.rf_duration));
      const double w = gamma * B0;
      if (time < f.rf_duration)
        return {B1 * std::cos(w * time) - .5 * G * r.x, -B1 * std::sin(w * time) - .5 * G * r.y,
                G * r.z + B0};
      return {-.5 * G * r.x, -.5 * G * r.y, G * r.z + B0};
    }
  }
}

// getStepTimeMin (QSC_PGSE :121-127, UCN_lowfield :469-475)
double step_time_min(const orc_field &f, double time) {
  if (f.kind == 1) return (time >= f.TE / 2.0 && time < f.TE / 2.0 + f.rf_duration) ? f.dtmin : f.dtmax;
  return (time <= f.rf_duration) ? f.dtmin : f.dtmax;
}

// updateMag_noT2_rotate (blochdiff.cuh:147-172): rotation of M about B by
// -GAMMA |B| h.  |B| = 0 leaves M unchanged (the reference divides by 0).
V3 mag_rotate(const V3 &M, const V3 &B, double h, double gamma) {
  const double Bmag = std::sqrt(B.x * B.x + B.y * B.y + B.z * B.z);
  if (!(Bmag > 0.0)) return M;
  const V3 bh = B * (1.0 / Bmag);
  const V3 C = bh * (M.x * bh.x + M.y * bh.y + M.z * bh.z);
  const V3 u = M - C;
  const double ang = -gamma * Bmag * h;
  return (C + u * std::cos(ang)) + cross(bh, u) * std::sin(ang);
}

// updateMagRK4 without relaxation (blochdiff.cuh:29-44); bloch() = (M % B) GAMMA
V3 mag_rk4(const orc_field &f, double gamma, const V3 &r, const V3 &M, double i, double h) {
  auto bl = [&](const V3 &m, const V3 &B) { return cross(m, B) * gamma; };
  const double tn = i * h;
  const V3 k1 = bl(M, bfield(f, gamma, r, tn)) * h;
  const V3 k2 = bl(M + k1 * .5, bfield(f, gamma, r, tn + .5 * h)) * h;
  const V3 k3 = bl(M + k2 * .5, bfield(f, gamma, r, tn + .5 * h)) * h;
  const V3 k4 = bl(M + k3, bfield(f, gamma, r, tn + h)) * h;
  const V3 d = (((k1 + k2 * 2.0) + k3 * 2.0) + k4) * (1.0 / 6.0);
  return {M.x + d.x, M.y + d.y, M.z + d.z};
}

// updateMag_rotate_noT2_multistep (blochdiff.cuh:118-140)
V3 mag_multistep(const orc_field &f, double gamma, const V3 &r, V3 M, int i, double dt) {
  double acc = 0.0, tk = i * dt;
  const double hmin = step_time_min(f, tk);
  do {
    M = mag_rotate(M, bfield(f, gamma, r, tk), hmin, gamma);
    acc += hmin;
    tk += hmin;
  } while (acc < dt);
  return M;
}

// Adaptive Dormand-Prince 5(4) over [i dt, (i+1) dt] with the walker at r,
// the integrator the reference's DORP_NORELAXATION build aims at
// (updateMag_DORP, blochdiff.cuh:69-146, which does not compile).  Tableau
// of Dormand & Prince (1980), J. Comput. Appl. Math. 6:19-26, the fifth-order
// solution propagated; the error of the embedded fourth-order one, scaled per
// component by tol (1 + max(|M5|, |M|)) and taken as an RMS over the three
// components (the reference's error norm), decides.  Sub-steps are
// dt / 2^k, k = 0..K, on a dyadic grid: a step whose error exceeds 1 is
// retried at half the length (down to level K, where it is accepted); after
// an accepted step with error below 1/32 the next step doubles when the grid
// allows.  The product's kernel makes the same decisions in FP32.
V3 mag_dorp(const orc_field &f, double gamma, const V3 &r, V3 M, int i, double dt, int K,
            double tol) {
  static const double c[6] = {0.0, 1.0 / 5.0, 3.0 / 10.0, 4.0 / 5.0, 8.0 / 9.0, 1.0};
  static const double a[6][5] = {{0, 0, 0, 0, 0},
                                 {1.0 / 5.0, 0, 0, 0, 0},
                                 {3.0 / 40.0, 9.0 / 40.0, 0, 0, 0},
                                 {44.0 / 45.0, -56.0 / 15.0, 32.0 / 9.0, 0, 0},
                                 {19372.0 / 6561.0, -25360.0 / 2187.0, 64448.0 / 6561.0,
                                  -212.0 / 729.0, 0},
                                 {9017.0 / 3168.0, -355.0 / 33.0, 46732.0 / 5247.0, 49.0 / 176.0,
                                  -5103.0 / 18656.0}};
  static const double b[6] = {35.0 / 384.0, 0.0, 500.0 / 1113.0, 125.0 / 192.0,
                              -2187.0 / 6784.0, 11.0 / 84.0};
  // e = b - b*, the seventh entry multiplies the derivative at the new point
  static const double e[7] = {71.0 / 57600.0, 0.0, -71.0 / 16695.0, 71.0 / 1920.0,
                              -17253.0 / 339200.0, 22.0 / 525.0, -1.0 / 40.0};
  auto deriv = [&](const V3 &m, double t) { return cross(m, bfield(f, gamma, r, t)) * gamma; };
  const int full = 1 << K;
  int pos = 0, k = 0;
  for (int guard = 0; pos < full && guard < 64 * full; ++guard) {
    const double h = dt / (double)(1 << k);
    const double t0 = i * dt + (double)(pos >> (K - k)) * h;
    V3 fk[7];
    for (int s = 0; s < 6; ++s) {
      V3 y = M;
      for (int q = 0; q < s; ++q) y = y + fk[q] * (h * a[s][q]);
      fk[s] = deriv(y, t0 + c[s] * h);
    }
    V3 y5 = M;
    for (int q = 0; q < 6; ++q) y5 = y5 + fk[q] * (h * b[q]);
    fk[6] = deriv(y5, t0 + h);
    V3 err{0, 0, 0};
    for (int q = 0; q < 7; ++q) err = err + fk[q] * (h * e[q]);
    auto ratio = [&](double d, double m5, double m) {
      return d / (tol * (1.0 + std::max(std::fabs(m5), std::fabs(m))));
    };
    const double rx = ratio(err.x, y5.x, M.x), ry = ratio(err.y, y5.y, M.y),
                 rz = ratio(err.z, y5.z, M.z);
    const double en = std::sqrt((rx * rx + ry * ry + rz * rz) / 3.0);
    if (en <= 1.0 || k == K) {
      M = y5;
      pos += 1 << (K - k);
      if (en < 1.0 / 32.0 && k > 0 && (pos & ((1 << (K - k + 1)) - 1)) == 0) --k;
    } else {
      ++k;
    }
  }
  return M;
}

// The update updateWalkersMag applies for field f at step i (kernelMag.cuh:
// 32-72 for i = 0, :96-134 for i >= 1).  With RK4_NORELAXATION only the i = 0
// update is RK4: the step loop has no branch for it and rotates.
V3 mag_update(const orc_field &f, const orc_mag_params &p, const V3 &r, const V3 &M, int i) {
  const double dt = p.timestep;
  if (p.integrator == 3)
    return mag_dorp(f, p.gamma, r, M, i, dt, p.dorp_levels ? (int)p.dorp_levels : 3,
                    p.dorp_tol > 0.0 ? p.dorp_tol : 1e-6);
  if (p.integrator == 2) return mag_multistep(f, p.gamma, r, M, i, dt);
  if (p.integrator == 1 && i == 0) return mag_rk4(f, p.gamma, r, M, 0.0, dt);
  return mag_rotate(M, bfield(f, p.gamma, r, i * dt), dt, p.gamma);
}

}  // namespace

// ----------------------------------------------------------- mesh pores ---
// A closed triangle mesh as a single pore (the reference's drafts
// src/primitives/mesh.cuh:1-75, triangle.cuh:1-59, which do not compile):
// Triangle::intersect (plane crossing, then barycentric inside test),
// Mesh::intersect (nearest crossing), Mesh::inside (parity of a vertical
// ray).  Restated in the GPU walker's formulation: triangles oriented
// outward, crossings from inside to outside only (n.d > 0, from at most a
// rounding slack beyond the plane), the watertight hit test; the parity of
// the vertical rays up and down must agree.  Every triangle is tested (the
// GPU's grid lists are conservative, so both find the same nearest hit).
template <typename T>
struct KMesh {
  struct Tri {
    T n[3], w, v[3][3];  // unit outward normal, n.v0, the vertices
  };
  std::vector<Tri> tri;
  std::vector<char> vertical;  // |n_z| < 1e-9: never crossed by a vertical line
  T lo[3], hi[3];
  T slack = T(0);  // 4e-6 of the largest |coordinate|: a start rounded beyond a face meets it
};

// Outward orientation: the two triangles of an edge traverse it in opposite
// directions ((b, c) swapped where they do not, breadth-first from the
// lowest unvisited triangle), then each connected component with negative
// signed volume flips.  -1 unless every edge has exactly two triangles.
inline int mesh_orient(const double *vx, const int32_t *in, int ntri, std::vector<int32_t> &tris) {
  tris.assign(in, in + 3 * (size_t)ntri);
  std::map<std::pair<int, int>, std::vector<int>> edges;
  for (int t = 0; t < ntri; ++t)
    for (int j = 0; j < 3; ++j) {
      const int a = tris[3 * t + j], b = tris[3 * t + (j + 1) % 3];
      if (a == b) return -1;
      edges[{std::min(a, b), std::max(a, b)}].push_back(t);
    }
  for (auto &kv : edges)
    if (kv.second.size() != 2) return -1;
  auto dir = [&](int t, int a, int b) {
    for (int j = 0; j < 3; ++j) {
      const int u = tris[3 * t + j], v = tris[3 * t + (j + 1) % 3];
      if (u == a && v == b) return 1;
      if (u == b && v == a) return -1;
    }
    return 0;
  };
  std::vector<int> comp(ntri, -1);
  int nc = 0;
  for (int s0 = 0; s0 < ntri; ++s0) {
    if (comp[s0] >= 0) continue;
    std::vector<int> q{s0};
    comp[s0] = nc;
    for (size_t i = 0; i < q.size(); ++i) {
      const int t = q[i];
      for (int j = 0; j < 3; ++j) {
        const int a = tris[3 * t + j], b = tris[3 * t + (j + 1) % 3];
        for (int u : edges[{std::min(a, b), std::max(a, b)}]) {
          if (u == t) continue;
          if (comp[u] >= 0) {
            if (dir(u, a, b) == dir(t, a, b)) return -1;
            continue;
          }
          if (dir(u, a, b) == dir(t, a, b)) std::swap(tris[3 * u + 1], tris[3 * u + 2]);
          comp[u] = nc;
          q.push_back(u);
        }
      }
    }
    ++nc;
  }
  std::vector<double> vol(nc, 0.0);
  for (int t = 0; t < ntri; ++t) {
    const double *a = &vx[3 * tris[3 * t]], *b = &vx[3 * tris[3 * t + 1]],
                 *c = &vx[3 * tris[3 * t + 2]];
    vol[comp[t]] += a[0] * (b[1] * c[2] - b[2] * c[1]) - a[1] * (b[0] * c[2] - b[2] * c[0]) +
                    a[2] * (b[0] * c[1] - b[1] * c[0]);
  }
  for (int t = 0; t < ntri; ++t)
    if (vol[comp[t]] < 0.0) std::swap(tris[3 * t + 1], tris[3 * t + 2]);
  return 0;
}

template <typename T>
int mesh_build(const double *vx, int nvert, const int32_t *tris_in, int ntri, KMesh<T> &K) {
  for (int i = 0; i < 3 * ntri; ++i)
    if (tris_in[i] < 0 || tris_in[i] >= nvert) return -1;
  std::vector<int32_t> tv;
  if (mesh_orient(vx, tris_in, ntri, tv) != 0) return -1;
  const int32_t *tris = tv.data();
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int t = 0; t < ntri; ++t)
    for (int j = 0; j < 3; ++j) {
      const int v = tris[3 * t + j];
      if (v < 0 || v >= nvert) return -1;
      for (int k = 0; k < 3; ++k) {
        lo[k] = std::min(lo[k], vx[3 * v + k]);
        hi[k] = std::max(hi[k], vx[3 * v + k]);
      }
    }
  for (int k = 0; k < 3; ++k) {
    K.lo[k] = (T)lo[k];
    K.hi[k] = (T)hi[k];
  }
  K.tri.resize(ntri);
  K.vertical.assign(ntri, 0);
  for (int t = 0; t < ntri; ++t) {
    const double *p0 = &vx[3 * tris[3 * t]];
    const double *p1 = &vx[3 * tris[3 * t + 1]];
    const double *p2 = &vx[3 * tris[3 * t + 2]];
    const double u[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
    const double v[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
    double n[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2],
                   u[0] * v[1] - u[1] * v[0]};
    const double nm = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (!(nm > 0.0)) return -1;
    for (double &c : n) c /= nm;
    const double w = n[0] * p0[0] + n[1] * p0[1] + n[2] * p0[2];
    auto &r = K.tri[t];
    for (int k = 0; k < 3; ++k) {
      r.n[k] = (T)n[k];
      r.v[0][k] = (T)p0[k];
      r.v[1][k] = (T)p1[k];
      r.v[2][k] = (T)p2[k];
    }
    r.w = (T)w;
    K.vertical[t] = std::fabs(n[2]) < 1e-9 ? 1 : 0;
  }
  return 0;
}

// The vertical line through (px, py) against the triangle's projection on
// (x, y): edge functions from the vertices relative to the point, zeros
// counted only on "top-left" edges of the counter-clockwise oriented
// projection (each edge or vertex counts for exactly one triangle).
template <typename T>
bool covers_xy(T px, T py, const T (&v)[3][3]) {
  const T ax = v[0][0] - px, ay = v[0][1] - py, bx = v[1][0] - px, by = v[1][1] - py;
  const T cx = v[2][0] - px, cy = v[2][1] - py;
  T e0 = bx * cy - by * cx, e1 = cx * ay - cy * ax, e2 = ax * by - ay * bx;
  const T area = e0 + e1 + e2;
  if (area == T(0)) return false;
  const T sg = area > T(0) ? T(1) : T(-1);
  e0 *= sg;
  e1 *= sg;
  e2 *= sg;
  auto tl = [&](T ux, T uy, T vx, T vy) {
    const T dx = (vx - ux) * sg, dy = (vy - uy) * sg;
    return dy > T(0) || (dy == T(0) && dx < T(0));
  };
  return (e0 > T(0) || (e0 == T(0) && tl(v[1][0], v[1][1], v[2][0], v[2][1]))) &&
         (e1 > T(0) || (e1 == T(0) && tl(v[2][0], v[2][1], v[0][0], v[0][1]))) &&
         (e2 > T(0) || (e2 == T(0) && tl(v[0][0], v[0][1], v[1][0], v[1][1])));
}

// 1 inside, 0 outside, -1 when the rays up and down disagree
template <typename T>
int mesh_side(const KMesh<T> &K, T x, T y, T z) {
  int up = 0, down = 0;
  for (size_t k = 0; k < K.tri.size(); ++k) {
    if (K.vertical[k]) continue;
    const auto &r = K.tri[k];
    if (!covers_xy(x, y, r.v)) continue;
    const T zh = (r.w - fmaT(r.n[0], x, r.n[1] * y)) / r.n[2];
    up += zh > z ? 1 : 0;
    down += zh < z ? 1 : 0;
  }
  if ((up & 1) != (down & 1)) return -1;
  return up & 1;
}

// The watertight ray/triangle test (Woop, Benthin and Wald, JCGT 2013): the
// ray's shear frame (rows m0, m1: 2-D coordinates with the ray at the
// origin; m2: distance along the ray; kz the direction's largest
// component), edge functions as differences of two products, zero edge
// functions counted as hits.
template <typename T>
struct KShear {
  T m[3][3];
};

template <typename T>
KShear<T> k_shear(T dx, T dy, T dz) {
  const T ax = std::fabs(dx), ay = std::fabs(dy), az = std::fabs(dz);
  const int kz = (ax > ay) ? ((ax > az) ? 0 : 2) : ((ay > az) ? 1 : 2);
  int kx = kz == 2 ? 0 : kz + 1, ky = kx == 2 ? 0 : kx + 1;
  const T d[3] = {dx, dy, dz};
  if (d[kz] < T(0)) std::swap(kx, ky);
  const T sx = d[kx] / d[kz], sy = d[ky] / d[kz], sz = T(1) / d[kz];
  KShear<T> M;
  for (int c = 0; c < 3; ++c) {
    M.m[0][c] = c == kx ? T(1) : (c == kz ? -sx : T(0));
    M.m[1][c] = c == ky ? T(1) : (c == kz ? -sy : T(0));
    M.m[2][c] = c == kz ? sz : T(0);
  }
  return M;
}

template <typename T>
T k_watertight(const KShear<T> &M, T px, T py, T pz, const T (&v)[3][3]) {
  T X[3], Y[3], Z[3];
  for (int i = 0; i < 3; ++i) {
    const T a = v[i][0] - px, b = v[i][1] - py, c = v[i][2] - pz;
    X[i] = fmaT(M.m[0][0], a, fmaT(M.m[0][1], b, M.m[0][2] * c));
    Y[i] = fmaT(M.m[1][0], a, fmaT(M.m[1][1], b, M.m[1][2] * c));
    Z[i] = fmaT(M.m[2][0], a, fmaT(M.m[2][1], b, M.m[2][2] * c));
  }
  const T U = X[2] * Y[1] - Y[2] * X[1];
  const T V = X[0] * Y[2] - Y[0] * X[2];
  const T W = X[1] * Y[0] - Y[1] * X[0];
  const T inf = std::numeric_limits<T>::infinity();
  if ((U < T(0) || V < T(0) || W < T(0)) && (U > T(0) || V > T(0) || W > T(0))) return inf;
  const T det = U + V + W;
  if (det == T(0)) return inf;
  const T Tn = fmaT(U, Z[0], fmaT(V, Z[1], W * Z[2]));
  return Tn / det;
}

template <typename T>
T mesh_hit(const KMesh<T> &K, int last, T px, T py, T pz, T dx, T dy, T dz, T rem, int &bk) {
  T best = std::numeric_limits<T>::infinity();
  bk = -1;
  const KShear<T> M = k_shear(dx, dy, dz);
  for (int k = 0; k < (int)K.tri.size(); ++k) {
    if (k == last) continue;
    const auto &r = K.tri[k];
    const T dn = fmaT(r.n[0], dx, fmaT(r.n[1], dy, r.n[2] * dz));
    if (!(dn > T(0))) continue;  // crossings from inside to outside only
    const T np = fmaT(r.n[0], px, fmaT(r.n[1], py, r.n[2] * pz));
    const T dist = r.w - np;
    if (!(dist > -K.slack)) continue;
    if (!(dist < rem * dn)) continue;  // the plane lies beyond the path
    const T s = k_watertight(M, px, py, pz, r.v);
    if (s < rem && s < best) {
      best = s;
      bk = k;
    }
  }
  return best;
}

template <typename T>
void mesh_walk_one(const KMesh<T> &K, double D, const orc_sequence *seqs, int nseq,
                   const orc_params &p, double gamma, int64_t w, WalkOut &out, TraceRow *tr,
                   bool &escaped) {
  const double dt = p.timestep;
  Stream st{p.seed, (uint64_t)(w + p.walker_offset), 1u};
  auto U = [](Stream &s) { return (T)s.uniform(); };
  T x = 0, y = 0, z = 0;
  bool ok = false;
  for (int t = 0; t < 100000 && !ok; ++t) {
    x = fmaT(U(st), K.hi[0] - K.lo[0], K.lo[0]);
    y = fmaT(U(st), K.hi[1] - K.lo[1], K.lo[1]);
    z = fmaT(U(st), K.hi[2] - K.lo[2], K.lo[2]);
    ok = mesh_side(K, x, y, z) == 1;
  }
  if (tr) {
    tr->init_pos[0] = (double)x;
    tr->init_pos[1] = (double)y;
    tr->init_pos[2] = (double)z;
  }
  for (int j = 0; j < nseq; ++j)
    out.phase[j] = gamma * dot(gfunc(seqs[j], 0.0), V3{(double)x, (double)y, (double)z}) * dt;
  const double sp = std::sqrt(6.0 * D / dt);
  const T L = (T)(sp * dt);
  for (int i = 1; i < p.steps; ++i) {
    const T u1 = U(st), u2 = U(st);
    T dx, dy, dz;
    k_direction(u1, u2, dx, dy, dz);
    T rem = L, sx = x, sy = y, sz = z;
    int last = -1, nh = 0;
    bool capped = false;
    for (;;) {
      int bk;
      const T best = mesh_hit(K, last, sx, sy, sz, dx, dy, dz, rem, bk);
      if (bk < 0) break;
      if (nh == 1024) {
        capped = true;
        break;
      }
      sx = fmaT(best, dx, sx);
      sy = fmaT(best, dy, sy);
      sz = fmaT(best, dz, sz);
      rem = rem - best;
      const auto &r = K.tri[bk];
      const T t = T(-2) * fmaT(dx, r.n[0], fmaT(dy, r.n[1], dz * r.n[2]));
      dx = fmaT(t, r.n[0], dx);
      dy = fmaT(t, r.n[1], dy);
      dz = fmaT(t, r.n[2], dz);
      last = bk;
      ++nh;
    }
    if (capped) {
      x = sx;
      y = sy;
      z = sz;
    } else {
      x = fmaT(rem, dx, sx);
      y = fmaT(rem, dy, sy);
      z = fmaT(rem, dz, sz);
    }
    out.caps += capped ? 1 : 0;
    const V3 pp{(double)x, (double)y, (double)z};
    for (int j = 0; j < nseq; ++j) out.phase[j] += gamma * dot(gfunc(seqs[j], dt * i), pp) * dt;
    if (tr) {
      const size_t o = (size_t)(i - 1);
      tr->pos[o * 3 + 0] = (double)x;
      tr->pos[o * 3 + 1] = (double)y;
      tr->pos[o * 3 + 2] = (double)z;
      tr->region[o] = 0;
      tr->hits[o] = nh;
      tr->words[o] = (int32_t)st.word;
    }
  }
  escaped = ok && mesh_side(K, x, y, z) == 0;
}

extern "C" {

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
  philox(c, key[0], key[1]);
  std::memcpy(out, c, 16);
}

void orc_stream_words(uint64_t seed, uint64_t walker, int n, uint32_t *out) {
  Stream s{seed, walker, 0u};
  for (int i = 0; i < n; ++i) out[i] = s.next_word();
}

void orc_sincos_2pi_f32(float u, float *s, float *c) { k_sincos_2pi<float>(u, *s, *c); }

double orc_bvalue(const orc_sequence *q, double gamma) {
  const double G = q->G, d = q->duration, sp = q->spacing, n = (double)q->num_periods;
  if (gamma <= 0.0) gamma = kGAMMA;
  switch (q->kind) {
    case 0: return G * G * d * d * gamma * gamma * ((2.0 / 3.0) * d + sp);
    case 1: return gamma * gamma * (1.0 / 4.0) * G * G * d * d * d / (kPI * kPI * n * n);
    case 2: return gamma * gamma * (3.0 / 4.0) * G * G * d * d * d / (kPI * kPI * n * n);
    case 3:
      return gamma * gamma * (1.0 / 4.0) * G * G * d * d * d / (kPI * kPI * n * n) *
             (1.0 - 1.0 / (8.0 * n));
    case 4: {
      const double nu = n / d;
      const double a1 = (1. - std::pow(-1., 2. * n) + 4. * d * nu) / (4. * nu);
      return G * G * gamma * gamma * (d / (6. * nu * nu) + sp * (d - a1) * (d - a1));
    }
  }
  return 0.0;
}

void orc_gradient(const orc_sequence *q, double t, double out[3]) {
  const V3 g = gfunc(*q, t);
  out[0] = g.x;
  out[1] = g.y;
  out[2] = g.z;
}

int orc_walk(const orc_lattice *lat, const orc_basis *basis, int nbasis, const orc_sequence *seqs,
             int nseq, const orc_params *p, int mode, int nthreads, double *sums, orc_trace *trace,
             int64_t *cap_hits) {
  if (!p || p->num_walkers < 1 || p->steps < 1 || !(p->timestep > 0.0)) return -1;
  if (nbasis < 0 || (nbasis > 0 && !basis) || (nseq > 0 && (!seqs || !sums))) return -1;
  if (!lat && nbasis < 1) return -1;
  if (mode < 0 || mode > 2) return -1;
  // a plane is no pore and has no inside to start walkers in
  if (!lat && basis[0].type == 2) return -1;
  if (lat && p->init_mode == 2 && p->init_arg >= 0 && p->init_arg < nbasis &&
      basis[p->init_arg].type == 2)
    return -1;
  WalkIn in{lat, basis, nbasis, seqs, nseq, p, p->gamma > 0.0 ? p->gamma : kGAMMA,
            lat == nullptr, false, false, (p->flags & 4u) != 0};
  in.relax = !in.single && (p->flags & 1u);
  in.perm = !in.single && (p->flags & 2u);
  in.pick = in.single && (p->flags & 32u);
  RefLattice L{};
  if (!in.single) {
    L.a = lat->a;
    L.b = lat->b;
    L.c = lat->c;
    L.D = lat->D;
    L.T2 = lat->T2;
    for (int k = 0; k < nbasis; ++k) L.B.push_back(RefBasis{&basis[k]});
  }
  KGeom<double> G64;
  KGeom<float> G32;
  if (mode == ORC_KERN64) k_build(lat, basis, nbasis, p->timestep, in.relax, in.single, G64);
  if (mode == ORC_KERN32) k_build(lat, basis, nbasis, p->timestep, in.relax, in.single, G32);
  const int64_t N = p->num_walkers;
  if (nthreads < 1) nthreads = 1;
  if ((int64_t)nthreads > N) nthreads = (int)N;
  // flag 64 (compartment sums): rows nseq..2nseq-1 sum the walkers that start
  // inside a basis
  const int rows = (!in.single && (p->flags & 64u)) ? 2 * nseq : nseq;
  std::vector<std::vector<double>> part(nthreads, std::vector<double>((size_t)rows * 5, 0.0));
  std::vector<int64_t> caps(nthreads, 0);
  auto work = [&](int t) {
    const int64_t w0 = N * t / nthreads, w1 = N * (t + 1) / nthreads;
    WalkOut out;
    out.phase.assign(nseq, 0.0);
    for (int64_t w = w0; w < w1; ++w) {
      TraceRow row, *tr = nullptr;
      if (trace && w < trace->ntrace) {
        const size_t o = (size_t)w * (size_t)(p->steps - 1);
        row = {trace->init_pos + w * 3, trace->pos + o * 3, trace->region + o, trace->hits + o,
               trace->words + o};
        tr = &row;
      }
      out.caps = 0;
      if (mode == ORC_REF64) walk_ref(in, L, w, out, tr);
      else if (mode == ORC_KERN64) walk_kern<double>(in, G64, w, out, tr);
      else walk_kern<float>(in, G32, w, out, tr);
      caps[t] += out.caps;
      // transformAndSumTwoVectors / transformAndSum (cudaVector.cu:143-172):
      // cos(phase) * exp(-T2factor) and sin(phase) * exp(-T2factor)
      const double wgt = in.relax ? std::exp(-out.t2factor) : 1.0;
      for (int j = 0; j < nseq; ++j) {
        const double xv = std::cos(out.phase[j]) * wgt, yv = std::sin(out.phase[j]) * wgt;
        double *s = &part[t][(size_t)j * 5];
        s[0] += xv;
        s[1] += yv;
        s[2] += xv * xv;
        s[3] += yv * yv;
        s[4] += xv * yv;
        if (rows > nseq && out.start_in) {
          double *q = &part[t][(size_t)(nseq + j) * 5];
          q[0] += xv;
          q[1] += yv;
          q[2] += xv * xv;
          q[3] += yv * yv;
          q[4] += xv * yv;
        }
      }
    }
  };
  if (nthreads == 1) {
    work(0);
  } else {
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; ++t) th.emplace_back(work, t);
    for (auto &x : th) x.join();
  }
  for (int j = 0; j < rows * 5; ++j) {
    double s = 0.0;
    for (int t = 0; t < nthreads; ++t) s += part[t][j];
    sums[j] = s;
  }
  if (cap_hits) {
    int64_t c = 0;
    for (auto v : caps) c += v;
    *cap_hits = c;
  }
  return 0;
}

int orc_step(const orc_lattice *lat, const orc_basis *basis, int nbasis, const orc_params *p,
             int mode, int64_t walker, int i, const double r_in[3], int32_t word, double r_out[3],
             int32_t *region, int32_t *hits, int32_t *word_out) {
  if (!p || !lat || i < 1 || mode < 0 || mode > 2) return -1;
  // A walk of two "steps" whose start is the given state: reuse the walkers
  // above with a patched stream and start position.
  const double dt = p->timestep;
  const bool relax = (p->flags & 1u) != 0, perm = (p->flags & 2u) != 0,
             reject = (p->flags & 4u) != 0;
  Stream st{p->seed, (uint64_t)(walker + p->walker_offset), (uint32_t)word};
  int h = 0;
  if (mode == ORC_REF64) {
    RefLattice L{};
    L.a = lat->a;
    L.b = lat->b;
    L.c = lat->c;
    L.D = lat->D;
    L.T2 = lat->T2;
    for (int k = 0; k < nbasis; ++k) L.B.push_back(RefBasis{&basis[k]});
    V3 r{r_in[0], r_in[1], r_in[2]};
    V3 ri = r;
    const double speed = std::sqrt(6.0 * L.getD(r) / dt);
    const double phi = 2.0 * kPI * st.uniform();
    const double theta = std::acos(2.0 * st.uniform() - 1);
    r = r + V3{speed * dt * std::sin(theta) * std::cos(phi), speed * dt * std::sin(theta) * std::sin(phi),
               speed * dt * std::cos(theta)};
    if (reject) {
      if (L.region(ri) != L.region(r)) r = ri;
    } else {
      double v = 0.0, acc = 0.0, pm = 0.0;
      V3 n{0, 0, 0}, rc = ri;
      bool transmitted = false;
      const double cur = std::sqrt(6.0 * L.getD(ri) / dt);
      while (L.check(rc, r, v, n, pm) && transmitted == false) {
        ++h;
        const double trs = std::sqrt(6.0 * L.getD(r) / dt);
        r = (r - rc) * v + rc;
        const V3 I = r - rc;
        const double Im = mag(I);
        acc += Im / (perm ? cur : speed);
        if (perm && !(st.uniform() > pm * 4.0 / cur)) {
          r = r + ((I / Im) * trs) * (dt - acc);
          transmitted = true;
        } else {
          rc = r;
          r = r + ((I - (n * 2.0) * dot(n, I)) * ((perm ? cur : speed) / Im)) * (dt - acc);
        }
      }
    }
    L.correct(r);
    r_out[0] = r.x;
    r_out[1] = r.y;
    r_out[2] = r.z;
    *region = L.first_inside(r);
  } else {
    auto run = [&](auto tag) {
      using T = decltype(tag);
      KGeom<T> G;
      k_build(lat, basis, nbasis, dt, relax, false, G);
      T x = (T)r_in[0], y = (T)r_in[1], z = (T)r_in[2];
      const int slot = G.inst.empty() ? G.ecs : k_lookup(G, x, y, z);
      const T v = G.speed[slot], Ls = G.step[slot];
      const T u1 = (T)st.uniform(), u2 = (T)st.uniform();
      T dx, dy, dz;
      k_direction(u1, u2, dx, dy, dz);
      T fx, fy, fz;
      if (G.inst.empty() || reject) {
        fx = fmaT(Ls, dx, x);
        fy = fmaT(Ls, dy, y);
        fz = fmaT(Ls, dz, z);
        if (reject && !G.inst.empty() && G.region[k_lookup(G, fx, fy, fz)] != G.region[slot]) {
          fx = x;
          fy = y;
          fz = z;
        }
      } else {
        const KMove<T> o = k_boundary(G, x, y, z, dx, dy, dz, Ls, v, perm, st, Ls);
        fx = o.fx;
        fy = o.fy;
        fz = o.fz;
        h = o.hits;
      }
      fx = k_wrap(fx, G.a);
      fy = k_wrap(fy, G.b);
      fz = k_wrap(fz, G.c);
      r_out[0] = (double)fx;
      r_out[1] = (double)fy;
      r_out[2] = (double)fz;
      const int rs = G.inst.empty() ? G.ecs : k_lookup(G, fx, fy, fz);
      *region = rs == G.ecs ? -1 : rs;
    };
    if (mode == ORC_KERN64) run(double(0));
    else run(float(0));
  }
  (void)relax;
  (void)i;
  *hits = h;
  *word_out = (int32_t)st.word;
  return 0;
}

int orc_wc(const orc_basis *pore, int64_t n, int steps, double timestep, double gamma,
           const uint32_t *rng_state, const double *start, const double *grad, double *phase,
           double *sum_cos, double *sum_sin) {
  if (!pore || n < 1 || steps < 0 || !rng_state || !start || !grad || !phase) return -1;
  const bool sph = pore->type == 1;
  // d_sigma = sqrt(2.0f * basis->getD() * pars->timestep)
  const double sigma = std::sqrt(2.0f * pore->D * timestep);
  double sc = 0.0, ss = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    uint32_t st = rng_state[i];
    auto uni = [&]() {  // rng_uni (:13-23)
      uint32_t x = st;
      x = x ^ (x >> 13);
      x = x ^ (x << 17);
      x = x ^ (x >> 5);
      st = x;
      return ((double)x + 1.0) / 4294967296.0f;
    };
    double x1 = start[3 * i], y1 = start[3 * i + 1], z1 = start[3 * i + 2];
    double ph = 0.0, kc = 0.0;
    for (int t = 0; t < steps; ++t) {
      double r = std::sqrt(-2.0f * std::log(uni()));
      double phi = 2.0f * kPI * (-0.5f + uni());
      const double dx = r * std::cos(phi), dy = r * std::sin(phi);
      r = std::sqrt(-2.0f * std::log(uni()));
      phi = 2.0f * kPI * (-0.5f + uni());
      const double dz = r * std::cos(phi);
      double x2 = x1 + dx * sigma, y2 = y1 + dy * sigma, z2 = z1 + dz * sigma;
      // Cylinder_XY / Sphere::inside(x, y, z) (cylinderXY.cuh:76-80, Sphere.cuh:96-100)
      double q = (x2 - pore->cx) * (x2 - pore->cx) + (y2 - pore->cy) * (y2 - pore->cy);
      if (sph) q = q + (z2 - pore->cz) * (z2 - pore->cz);
      if (!(q < pore->radius * pore->radius)) {
        x2 = x1;
        y2 = y1;
        z2 = z1;
      }
      const double ky = grad[3 * t] * x2 + grad[3 * t + 1] * y2 + grad[3 * t + 2] * z2 - kc;
      const double kt = ph + ky;
      kc = (kt - ph) - ky;
      ph = kt;
      x1 = x2;
      y1 = y2;
      z1 = z2;
    }
    phase[i] = ph * gamma * timestep;
    sc += (double)std::cos((float)phase[i]);
    ss += (double)std::sin((float)phase[i]);
  }
  if (sum_cos) *sum_cos = sc;
  if (sum_sin) *sum_sin = ss;
  return 0;
}

int orc_mesh_walk(const double *vertices, int nvert, const int32_t *triangles, int ntri, double D,
                  const orc_sequence *seqs, int nseq, const orc_params *p, int mode, int nthreads,
                  double *sums, orc_trace *trace, int64_t *escaped) {
  if (!vertices || !triangles || nvert < 4 || ntri < 4 || !p || p->num_walkers < 1 ||
      p->steps < 1 || !(p->timestep > 0.0) || !(D > 0.0) || (nseq > 0 && (!seqs || !sums)))
    return -1;
  if (mode != ORC_KERN64 && mode != ORC_KERN32) return -1;
  KMesh<double> K64;
  KMesh<float> K32;
  if ((mode == ORC_KERN64 ? mesh_build(vertices, nvert, triangles, ntri, K64)
                          : mesh_build(vertices, nvert, triangles, ntri, K32)) != 0)
    return -1;
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300}, cmax = 0.0;
  for (int t = 0; t < ntri; ++t)
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 3; ++k) {
        const double c = vertices[3 * triangles[3 * t + j] + k];
        lo[k] = std::min(lo[k], c);
        hi[k] = std::max(hi[k], c);
      }
  for (int k = 0; k < 3; ++k) cmax = std::max(cmax, std::max(std::fabs(lo[k]), std::fabs(hi[k])));
  K64.slack = 4e-6 * cmax;
  K32.slack = (float)(4e-6 * cmax);
  const double gamma = p->gamma > 0.0 ? p->gamma : kGAMMA;
  const int64_t N = p->num_walkers;
  if (nthreads < 1) nthreads = 1;
  if ((int64_t)nthreads > N) nthreads = (int)N;
  std::vector<std::vector<double>> part(nthreads, std::vector<double>((size_t)nseq * 5, 0.0));
  std::vector<int64_t> esc(nthreads, 0);
  auto work = [&](int t) {
    WalkOut out;
    out.phase.assign(nseq, 0.0);
    for (int64_t w = N * t / nthreads; w < N * (t + 1) / nthreads; ++w) {
      TraceRow row, *tr = nullptr;
      if (trace && w < trace->ntrace) {
        const size_t o = (size_t)w * (size_t)(p->steps - 1);
        row = {trace->init_pos + w * 3, trace->pos + o * 3, trace->region + o, trace->hits + o,
               trace->words + o};
        tr = &row;
      }
      bool e = false;
      if (mode == ORC_KERN64) mesh_walk_one(K64, D, seqs, nseq, *p, gamma, w, out, tr, e);
      else mesh_walk_one(K32, D, seqs, nseq, *p, gamma, w, out, tr, e);
      esc[t] += e ? 1 : 0;
      for (int j = 0; j < nseq; ++j) {
        const double xv = std::cos(out.phase[j]), yv = std::sin(out.phase[j]);
        double *s = &part[t][(size_t)j * 5];
        s[0] += xv;
        s[1] += yv;
        s[2] += xv * xv;
        s[3] += yv * yv;
        s[4] += xv * yv;
      }
    }
  };
  if (nthreads == 1) {
    work(0);
  } else {
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; ++t) th.emplace_back(work, t);
    for (auto &x : th) x.join();
  }
  for (int j = 0; j < nseq * 5; ++j) {
    double s = 0.0;
    for (int t = 0; t < nthreads; ++t) s += part[t][j];
    sums[j] = s;
  }
  if (escaped) {
    int64_t c = 0;
    for (auto v : esc) c += v;
    *escaped = c;
  }
  return 0;
}

int orc_volume_fraction(const orc_lattice *lat, const orc_basis *basis, int nbasis,
                        int64_t points, uint64_t seed, int mode, int nthreads, int64_t *inside) {
  if (!lat || nbasis < 0 || (nbasis > 0 && !basis) || points < 1 || !inside) return -1;
  if (mode != ORC_REF64 && mode != ORC_KERN32) return -1;
  RefLattice L{};
  L.a = lat->a;
  L.b = lat->b;
  L.c = lat->c;
  for (int k = 0; k < nbasis; ++k) L.B.push_back(RefBasis{&basis[k]});
  KGeom<float> G;
  if (mode == ORC_KERN32) k_build(lat, basis, nbasis, 1e-12, false, false, G);
  if (nthreads < 1) nthreads = 1;
  if ((int64_t)nthreads > points) nthreads = (int)points;
  std::vector<int64_t> cnt(nthreads, 0);
  auto work = [&](int t) {
    for (int64_t i = points * t / nthreads; i < points * (t + 1) / nthreads; ++i) {
      Stream st{seed, (uint64_t)i, 1u};
      if (mode == ORC_REF64) {
        V3 r;
        r.x = st.uniform() * L.a;
        r.y = st.uniform() * L.b;
        r.z = st.uniform() * L.c;
        cnt[t] += L.region(r) > 0 ? 1 : 0;
      } else {
        const float x = (float)st.uniform() * G.a, y = (float)st.uniform() * G.b,
                    z = (float)st.uniform() * G.c;
        cnt[t] += G.region[k_lookup(G, x, y, z)] > 0 ? 1 : 0;
      }
    }
  };
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; ++t) th.emplace_back(work, t);
  for (auto &x : th) x.join();
  int64_t c = 0;
  for (auto v : cnt) c += v;
  *inside = c;
  return 0;
}

void orc_bfield(const orc_field *f, double gamma, const double r[3], double t, double out[3]) {
  const V3 b = bfield(*f, gamma, V3{r[0], r[1], r[2]}, t);
  out[0] = b.x;
  out[1] = b.y;
  out[2] = b.z;
}

void orc_mag_along(const orc_field *f, int nf, const orc_mag_params *p, const double *pos,
                   double *m_out) {
  for (int j = 0; j < nf; ++j) {
    V3 M{p->m0[0], p->m0[1], p->m0[2]};
    for (int i = 0; i < p->steps; ++i)
      M = mag_update(f[j], *p, V3{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]}, M, i);
    m_out[3 * j] = M.x;
    m_out[3 * j + 1] = M.y;
    m_out[3 * j + 2] = M.z;
  }
}

int orc_mag_walk(const orc_basis *pore, const orc_field *f, int nf, const orc_mag_params *p,
                 int nthreads, double *sums, double *m_walk, orc_trace *trace) {
  if (!pore || !p || p->num_walkers < 1 || p->steps < 1 || !(p->timestep > 0.0)) return -1;
  if (nf < 1 || !f || !sums || p->integrator < 0 || p->integrator > 3) return -1;
  if (p->integrator == 3 && p->dorp_levels > 12) return -1;
  for (int j = 0; j < nf; ++j) {
    if (f[j].kind < 0 || f[j].kind > 7) return -1;
    if (p->integrator == 2 && f[j].kind != 1 && f[j].kind != 7) return -2;  // no getStepTimeMin
  }
  orc_params wp{p->num_walkers, p->steps, 0, 0, p->flags & 4u, p->seed, p->timestep, p->gamma,
                p->walker_offset};
  WalkIn in{nullptr, pore, 1, nullptr, 0, &wp, p->gamma, true, false, false, (p->flags & 4u) != 0};
  RefLattice L{};
  const int64_t N = p->num_walkers;
  if (nthreads < 1) nthreads = 1;
  if ((int64_t)nthreads > N) nthreads = (int)N;
  std::vector<std::vector<double>> part(nthreads, std::vector<double>((size_t)nf * 3, 0.0));
  auto work = [&](int t) {
    const int64_t w0 = N * t / nthreads, w1 = N * (t + 1) / nthreads;
    WalkOut out;
    std::vector<V3> M(nf);
    const std::function<void(int, const V3 &)> cb = [&](int i, const V3 &r) {
      for (int j = 0; j < nf; ++j) M[j] = mag_update(f[j], *p, r, M[j], i);
    };
    for (int64_t w = w0; w < w1; ++w) {
      TraceRow row, *tr = nullptr;
      if (trace && w < trace->ntrace) {
        const size_t o = (size_t)w * (size_t)(p->steps - 1);
        row = {trace->init_pos + w * 3, trace->pos + o * 3, trace->region + o, trace->hits + o,
               trace->words + o};
        tr = &row;
      }
      for (int j = 0; j < nf; ++j) M[j] = V3{p->m0[0], p->m0[1], p->m0[2]};
      walk_ref(in, L, w, out, tr, &cb);
      for (int j = 0; j < nf; ++j) {
        double *s = &part[t][(size_t)j * 3];
        s[0] += M[j].x;
        s[1] += M[j].y;
        s[2] += M[j].z;
        if (m_walk && trace && w < trace->ntrace) {
          double *o = m_walk + ((size_t)w * nf + j) * 3;
          o[0] = M[j].x;
          o[1] = M[j].y;
          o[2] = M[j].z;
        }
      }
    }
  };
  if (nthreads == 1) {
    work(0);
  } else {
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; ++t) th.emplace_back(work, t);
    for (auto &x : th) x.join();
  }
  for (int j = 0; j < nf * 3; ++j) {
    double s = 0.0;
    for (int t = 0; t < nthreads; ++t) s += part[t][j];
    sums[j] = s;
  }
  return 0;
}

}  // extern "C\"
