// walk_kernel.cuh -- the FP32 random-walker kernel for GB300 (sm_103a).
//
// One thread owns one walker at a time; its position, unbounded position,
// Philox stream, T2 sum and K phase-channel accumulators (value + Kahan
// compensation) live in registers for the whole walk.  A warp walks 32
// walkers; warps stride over walker tasks (32 walkers each) so the grid can
// be sized to the GPU's resident capacity.  After the walk the warp turns its
// walkers into the reference's signal terms in FP64
//   x = cos(phi_m) exp(-T2factor), y = sin(phi_m) exp(-T2factor)
// and reduces (x, y, x^2, y^2, xy) per sequence with shuffles into
// shared-memory per-warp sums; each block writes one FP64 partial per
// (sequence, statistic) and reduce_partials() sums them in a fixed order.
//
// What the kernel computes, per walker (reference: updateWalkersLatticePhase,
// src/kernels/kernelLattice.cuh:1-104, and updateWalkersPhase,
// src/kernels/kernelPhase.cuh:4-66):
//  1. start position from the stream (Lattice::initializeUniformly,
//     lattice.cuh:31-37; initializeInRegion :46-58; Basis::randUnif;
//     single pore: Basis::unifRand on a copy of the stream);
//  2. phase channel c starts at s_c(0) (p_c . r);
//  3. moves i = 1..steps-1: v, L from the region at r (Lattice::getD,
//     lattice.cuh:118-132); direction from two uniforms; boundary handling
//     (boundaryCheckImpermeable / boundaryCheckPermeable / boundaryNormal,
//     boundaryCheck.cuh:2-113, or simple rejection, kernelLattice.cuh:73-77);
//     r_unb += r - ri; channel c += s_c(i) (p_c . r_unb) with Kahan
//     compensation; T2 sum += dt/T2(region) (kernelLattice.cuh:87-96, with
//     the reference's permeable weighting that always sees accumtime = 0);
//     periodic wrap (Lattice::correctBoundary, lattice.cuh:60-88).
//
// Geometry of one boundary test (the reference's Cylinder_XY::intersect /
// Sphere::intersect, cylinderXY.cuh:82-122, Sphere.cuh:102-139, in the
// distance parameter s = v * |dr| along the unit direction d):
//   p = start - centre, c0 = |p|^2 - R^2, bh = p . d, a = |d|^2 (xy only for
//   cylinders).  The smallest root in (0, rem) with s >= eps is the hit.  The
//   instance hit last is tested with c0 = 0 (the walker sits on it), which is
//   the reference's rule in exact arithmetic (its root 0 fails the eps test).
//   Centre-relative differences keep FP32 accurate to the step scale where the
//   reference's expanded quadratic would lose the boundary distance.
// Periodicity: every basis and each periodic ghost that can be reached from
// the cell within one step is an instance; all tests of one move use the
// instance list of the grid cell that holds the move's start.
//
// Specialisation: the walk mode (KM: lattice specular impermeable / permeable
// / rejection, single pore specular / rejection), the geometry class and the
// channel capacity are template parameters, so a move carries no runtime mode
// branches; padded channels carry zero waveforms and coefficients.
#pragma once
#include <cuda_runtime.h>
#include "axx_rng.cuh"
#include "axx_walk.h"

namespace axx {

#define AXX_INF __int_as_float(0x7f800000)

// Geometry, slot tables and cell lists, staged in shared memory.
struct SmemView {
  const float4 *geo;
  const float4 *aux;
  const float4 *slot;
  const uint32_t *cstart;
  const int *region;
  const uint16_t *clist;
};

// Grid cell of an in-cell point: floor(x*inv) as round-to-nearest of
// x*inv - 1/2, done by adding 1.5*2^23 (where the FP32 spacing is 1) and
// reading the integer from the mantissa.  A point within rounding of a grid
// line may land in either neighbouring cell, which is safe because every
// cell list covers the cell dilated by one step.
__device__ __forceinline__ int cell_index(float x, float inv, int n) {
  const float t = fma_f(x, inv, -0.5f);
  const float f = t + 12582912.0f;
  const int i = __float_as_int(f) - 0x4B400000;
  return min(max(i, 0), n - 1);
}

template <int GEOM>
__device__ __forceinline__ int cell_of(const WalkParams &P, float x, float y, float z) {
  if (P.ncell == 1) return 0;
  const int ix = cell_index(x, P.inv_hx, P.gx);
  const int iy = cell_index(y, P.inv_hy, P.gy);
  if (GEOM == AXX_GEOM_CYL) return iy * P.gx + ix;
  const int iz = cell_index(z, P.inv_hz, P.gz);
  return (iz * P.gy + iy) * P.gx + ix;
}

__device__ __forceinline__ int aux_slot(const float4 &a) { return __float_as_int(a.z); }
__device__ __forceinline__ int aux_type(const float4 &a) { return __float_as_int(a.w); }

template <int GEOM>
__device__ __forceinline__ bool is_sphere(const float4 &aux) {
  if (GEOM == AXX_GEOM_SPH) return true;
  if (GEOM == AXX_GEOM_CYL) return false;
  return aux_type(aux) == 1;
}

// Planes (type 2) occur only in the mixed-type kernels.
template <int GEOM>
__device__ __forceinline__ bool is_plane(const float4 &aux) {
  if (GEOM != AXX_GEOM_MIX) return false;
  return aux_type(aux) == 2;
}

// |p|^2 - R^2 for the point (x, y, z) against one instance.
__device__ __forceinline__ float c0_of(const float4 &g, bool sph, float x, float y, float z) {
  const float px = x - g.x, py = y - g.y;
  if (sph) {
    const float pz = z - g.z;
    return fma_f(px, px, fma_f(py, py, fma_f(pz, pz, g.w)));
  }
  return fma_f(px, px, fma_f(py, py, g.w));
}

// Whether an instance contains the point; a plane contains none (it has no
// inside: Lattice::inRegion never reports it).
template <int GEOM>
__device__ __forceinline__ bool contains(const float4 &g, const float4 &aux, float x, float y,
                                         float z) {
  if (is_plane<GEOM>(aux)) return false;
  return c0_of(g, is_sphere<GEOM>(aux), x, y, z) < 0.0f;
}

// First instance (ascending basis order) of list [b, e) that contains the
// point; its slot, or the extracellular slot.
template <int GEOM>
__device__ __forceinline__ int lookup_list(const SmemView &S, uint32_t b, uint32_t e, int ecs,
                                           float x, float y, float z) {
  for (uint32_t j = b; j < e; ++j) {
    const int k = S.clist[j];
    const float4 aux = S.aux[k];
    if (contains<GEOM>(S.geo[k], aux, x, y, z)) return aux_slot(aux);
  }
  return ecs;
}

// Distance along the unit direction d from the start s to a plane
// g = (n, n.c), if in (0, rem) and >= eps, or +inf (Plane::intersect,
// plane.cuh:19-28: v = n.(c - ri) / n.dr on the segment, with the segment
// length folded in; the plane just reflected from is skipped, as its
// doub_equal test drops the zero root).  A direction parallel to the plane
// divides by zero and fails the range test.
__device__ __forceinline__ float plane_hit(const float4 &g, float eps, bool on_surface,
                                           float sx, float sy, float sz, float dx, float dy,
                                           float dz, float rem) {
  if (on_surface) return AXX_INF;
  const float np = fma_f(g.x, sx, fma_f(g.y, sy, g.z * sz));
  const float dn = fma_f(g.x, dx, fma_f(g.y, dy, g.z * dz));
  const float s = div_f(g.w - np, dn);
  if (!(s > 0.0f && s < rem && s >= eps)) return AXX_INF;
  return s;
}

// The annulus test of a cylinder list: whether a segment whose midpoint is
// (mx, my), of length at most the plan's longest step, can come near the
// cylinder's surface.  Cylinder-lattice plans store (R + h)^2 in geo.z, with
// h half the longest step plus a slack (1 % of it and 1e-6 of the cell)
// far above the FP32 rounding of positions; h2x2 = 2 h^2.  The segment lies
// within the ball of its half length around the midpoint, so a centre
// distance D with D > R + h (outside) or D < R - h (inside, (R - h)^2 =
// 2 R^2 + 2 h^2 - (R + h)^2) means no root of the exact test.
__device__ __forceinline__ bool annulus_keeps(const float4 &g, float mx, float my, float h2x2) {
  const float ex = mx - g.x, ey = my - g.y;
  const float d2 = fma_f(ex, ex, ey * ey);
  return !(d2 > g.z || d2 < fma_f(-2.0f, g.w, h2x2 - g.z));
}

// The quadratic of one instance along the segment start + s*d, s in
// [0, rem]: half the linear coefficient bh = p.d and |p|^2 - R^2 at both
// ends (c0 at the start, c1 at s = rem), p = start - centre.
__device__ __forceinline__ void seg_coef(const float4 &g, bool sph, float sx, float sy, float sz,
                                         float dx, float dy, float dz, float rem, float &bh,
                                         float &c0, float &c1) {
  const float px = sx - g.x, py = sy - g.y;
  const float pz = sph ? (sz - g.z) : 0.0f;
  const float ex = fma_f(rem, dx, px), ey = fma_f(rem, dy, py);
  if (sph) {
    const float ez = fma_f(rem, dz, pz);
    bh = fma_f(px, dx, fma_f(py, dy, pz * dz));
    c0 = fma_f(px, px, fma_f(py, py, fma_f(pz, pz, g.w)));
    c1 = fma_f(ex, ex, fma_f(ey, ey, fma_f(ez, ez, g.w)));
  } else {
    bh = fma_f(px, dx, py * dy);
    c0 = fma_f(px, px, fma_f(py, py, g.w));
    c1 = fma_f(ex, ex, fma_f(ey, ey, g.w));
  }
}

// The segment can meet the instance (the rejections the hit test applies
// first fail), given its quadratic.
__device__ __forceinline__ bool seg_may(float bh, float c0, float c1, float aa, float rem) {
  return !((c0 < 0.0f && c1 < 0.0f) ||
           (c0 >= 0.0f && (bh >= 0.0f || (c0 > 0.0f && c1 > 0.0f && fma_f(aa, rem, bh) <= 0.0f))));
}

// seg_may, and for a start outside also the discriminant test of seg_root's
// entry root (the same operation on the same operands): a line that passes
// beside the instance is rejected before the nearest-hit loop.
__device__ __forceinline__ bool seg_may_disc(float bh, float c0, float c1, float aa, float rem) {
  return seg_may(bh, c0, c1, aa, rem) && !(c0 > 0.0f && !(fma_f(bh, bh, -(aa * c0)) > 0.0f));
}

// Distance to the first boundary of one instance along the segment
// start + s*d, 0 < s < rem, or +inf, given its quadratic (c0 = 0 for a start
// on the instance's surface).
__device__ __forceinline__ float seg_root(float bh, float c0, float c1, float eps, float aa,
                                          float rem) {
  // cheap rejections: both ends inside; outside or on the surface and moving
  // away; outside with the closest approach beyond the end
  if (c0 < 0.0f && c1 < 0.0f) return AXX_INF;
  if (c0 >= 0.0f && (bh >= 0.0f || (c0 > 0.0f && c1 > 0.0f && fma_f(aa, rem, bh) <= 0.0f)))
    return AXX_INF;
  float s;
  if (c0 < 0.0f) {  // inside: the exit root
    const float sq = sqrt_f(fma_f(bh, bh, -(aa * c0)));
    s = (bh <= 0.0f) ? div_f(sq - bh, aa) : div_f(-c0, bh + sq);
  } else if (c0 > 0.0f) {  // outside: the entry root
    const float disc = fma_f(bh, bh, -(aa * c0));
    if (disc <= 0.0f) return AXX_INF;
    s = div_f(c0, sqrt_f(disc) - bh);
  } else {  // on the surface: the far root
    if (fma_f(rem, aa, 2.0f * bh) < 0.0f) return AXX_INF;  // beyond rem (see surface_hit)
    s = div_f(-2.0f * bh, aa);
  }
  if (!(s > 0.0f && s < rem && s >= eps)) return AXX_INF;
  return s;
}

__device__ __forceinline__ float seg_hit(const float4 &g, float eps, bool sph, bool on_surface,
                                         float sx, float sy, float sz, float dx, float dy,
                                         float dz, float aa, float rem) {
  float bh, c0, c1;
  seg_coef(g, sph, sx, sy, sz, dx, dy, dz, rem, bh, c0, c1);
  if (on_surface) c0 = 0.0f;
  return seg_root(bh, c0, c1, eps, aa, rem);
}

// seg_hit for a start on the instance's surface (c0 = 0), which needs only
// bh: moving away (bh >= 0) misses, else the far root -2 bh / aa.
__device__ __forceinline__ float surface_hit(const float4 &g, float eps, bool sph, float sx,
                                             float sy, float sz, float dx, float dy, float dz,
                                             float aa, float rem) {
  const float px = sx - g.x, py = sy - g.y;
  const float pz = sph ? (sz - g.z) : 0.0f;
  const float bh = sph ? fma_f(px, dx, fma_f(py, dy, pz * dz)) : fma_f(px, dx, py * dy);
  if (bh >= 0.0f) return AXX_INF;
  // The far root -2 bh / aa is at least rem when rem aa + 2 bh < 0: a
  // correctly rounded fma keeps the sign of the exact value (2 bh is exact),
  // and rounding is monotone, so the rounded quotient then fails s < rem
  // exactly as below; the usual case (a chord across the pore far longer than
  // the step) skips the division.
  if (fma_f(rem, aa, 2.0f * bh) < 0.0f) return AXX_INF;
  const float s = div_f(-2.0f * bh, aa);
  if (!(s > 0.0f && s < rem && s >= eps)) return AXX_INF;
  return s;
}

struct MoveOut {
  float fx, fy, fz;
  int hits;
  bool capped;
  bool crossed;  // transmitted through a permeable wall
};

__device__ __forceinline__ void kahan_add(float &s, float &c, float y) {
  const float yy = y - c;
  const float t = s + yy;
  c = (t - s) - yy;
  s = t;
}

// Start position.  Returns false if a rejection loop ran out of tries.
template <int GEOM, int KM>
__device__ __forceinline__ bool init_position(const WalkParams &P, const SmemView &S,
                                              DevStream &st, float &x, float &y, float &z) {
  constexpr bool single = KM >= AXX_KM_SINGLE;
  if (single) {
    // Basis::unifRand (cylinderXY.cuh:45-55, Sphere.cuh:55-63).  The sphere's
    // box is centred on the sphere (the reference omits the centre, which
    // only agrees for a sphere at the origin); its retries draw z, y, x, the
    // order in which the compiled reference evaluates the three draws passed
    // as Vector3 constructor arguments.
    const float4 g = S.geo[P.init_inst];
    const bool sph = P.init_sph != 0;
    x = fma_f(fma_f(2.0f, st.next(P), -1.0f), P.init_R, P.init_cx);
    y = fma_f(fma_f(2.0f, st.next(P), -1.0f), P.init_R, P.init_cy);
    z = sph ? fma_f(fma_f(2.0f, st.next(P), -1.0f), P.init_R, P.init_cz)
            : (2.0f * P.init_R) * st.next(P);
    for (int t = 0; t < AXX_INIT_TRIES; ++t) {
      if (c0_of(g, sph, x, y, z) < 0.0f) return true;
      if (sph) {
        z = fma_f(fma_f(2.0f, st.next(P), -1.0f), P.init_R, P.init_cz);
        y = fma_f(fma_f(2.0f, st.next(P), -1.0f), P.init_R, P.init_cy);
        x = fma_f(fma_f(2.0f, st.next(P), -1.0f), P.init_R, P.init_cx);
      } else {
        x = fma_f(fma_f(2.0f, st.next(P), -1.0f), P.init_R, P.init_cx);
        y = fma_f(fma_f(2.0f, st.next(P), -1.0f), P.init_R, P.init_cy);
        z = (2.0f * P.init_R) * st.next(P);
      }
    }
    return false;
  } else {
    if (P.init_mode == 2) {
      // Basis::randUnif (cylinderXY.cuh:176-183, Sphere.cuh:384-391): the
      // three draws are Vector3 constructor arguments, consumed z, y, x; a
      // cylinder's centre has z = 0.
      const float4 g = S.geo[P.init_inst];
      const bool sph = P.init_sph != 0;
      for (int t = 0; t < AXX_INIT_TRIES; ++t) {
        const float tz = fma_f(2.0f, st.next(P), -1.0f);
        y = fma_f(fma_f(2.0f, st.next(P), -1.0f), P.init_R, P.init_cy);
        x = fma_f(fma_f(2.0f, st.next(P), -1.0f), P.init_R, P.init_cx);
        z = sph ? fma_f(tz, P.init_R, P.init_cz) : tz * P.init_R;
        if (c0_of(g, sph, x, y, z) < 0.0f) return true;
      }
      return false;
    }
    for (int t = 0; t < AXX_INIT_TRIES; ++t) {
      x = st.next(P) * P.a;
      y = st.next(P) * P.b;
      z = st.next(P) * P.c;
      if (P.init_mode == 0) return true;
      // Lattice::initializeInRegion: region id of the first containing basis
      int slot = P.ecs_slot;
      if (GEOM != AXX_GEOM_FREE) {
        const int cell = cell_of<GEOM>(P, x, y, z);
        slot = lookup_list<GEOM>(S, S.cstart[cell], S.cstart[cell + 1], P.ecs_slot, x, y, z);
      }
      if (S.region[slot] == P.init_arg) return true;
    }
    return false;
  }
}

struct WalkResult {
  unsigned caps, hits;
  bool init_fail, aborted;
};

// State of one walker between moves.
template <int KMAX>
struct Walker {
  float x, y, z;     // wrapped position (bounded position for the single pore)
  float ux, uy, uz;  // unbounded position
  int slot;          // slot of the region at (x, y, z)
  float acc[KMAX], cmp[KMAX];
  float part[KMAX];  // phase of the current block of moves (DEFER)
  float t2s, t2c;
  int nin;  // ONE: moves weighted by the instance's region (T2 by counts)
  // speed, step and dt/T2 of the walker's slot, held while the slot holds
  // (walks behind specular or permeable walls, whose slot changes only at a
  // wrap or a transmission)
  float v0, L0, t2z;
};

// The instances and the list a move may test: either the cell list of the
// move's start (general substrates) or instance 0 held in registers (ONE:
// substrates of a single instance -- a one-basis cell without reachable
// ghosts, or any single pore).
template <int GEOM, bool ONE>
struct Cands {
  const SmemView &S;
  float4 g0, a0;
  uint32_t b, e;
  __device__ __forceinline__ int lookup(int ecs, float x, float y, float z) const {
    if (ONE) return contains<GEOM>(g0, a0, x, y, z) ? aux_slot(a0) : ecs;
    return lookup_list<GEOM>(S, b, e, ecs, x, y, z);
  }
};

// The pre-filter of a move: whether any candidate may meet the segment
// (maybe), and for lists the candidates that may (mmask: bit j for the
// list's j-th candidate; candidates past the 32nd are always tested).  ONE:
// the quadratic of the first pass (bh1, c01, c11), which the nearest-hit
// loop's first pass reuses.
template <int GEOM, bool PERM, bool ONE>
__device__ __forceinline__ bool prefilter(const WalkParams &P, const Cands<GEOM, ONE> &C, float sx,
                                          float sy, float sz, float dx, float dy, float dz,
                                          float L, uint32_t &mmask, float &bh1, float &c01,
                                          float &c11) {
  bool maybe = false;
  mmask = 0u;
  {
    const float aa_c = fma_f(dx, dx, dy * dy);
    const float aa_s = fma_f(dx, dx, fma_f(dy, dy, dz * dz));
    auto may = [&](const float4 &g, const float4 &aux) {
      // a plane: the test of the nearest-hit loop's first pass itself
      if (is_plane<GEOM>(aux))
        return plane_hit(g, aux.y, false, sx, sy, sz, dx, dy, dz, L) < AXX_INF;
      const bool sph = is_sphere<GEOM>(aux);
      float bh, c0, c1;
      seg_coef(g, sph, sx, sy, sz, dx, dy, dz, L, bh, c0, c1);
      // the same rejections seg_root applies first (c0 is exact here: no
      // instance has been hit yet in this move), its discriminant test
      // included
      return seg_may_disc(bh, c0, c1, sph ? aa_s : aa_c, L);
    };
    if (ONE) {
      if (is_plane<GEOM>(C.a0)) {
        maybe = may(C.g0, C.a0);
      } else {
        const bool sph = is_sphere<GEOM>(C.a0);
        seg_coef(C.g0, sph, sx, sy, sz, dx, dy, dz, L, bh1, c01, c11);
        maybe = seg_may_disc(bh1, c01, c11, sph ? aa_s : aa_c, L);
      }
    } else if constexpr (GEOM == AXX_GEOM_CYL && PERM) {
      // lists of permeable cylinders: the annulus test first (the segment lies within
      // L/2 of its midpoint; a cylinder whose surface is farther than that,
      // plus a slack far above FP32 rounding, cannot be met), then the exact
      // test on the candidates it keeps
      const float hl = 0.5f * L;
      const float mx = fma_f(hl, dx, sx), my = fma_f(hl, dy, sy);
      uint32_t keep = 0u;
      bool far = false;  // a candidate past the 32nd kept (always tested)
#pragma unroll 2
      for (uint32_t j = C.b; j < C.e; ++j) {
        const uint32_t bit = j - C.b;
        const bool k = annulus_keeps(C.S.geo[C.S.clist[j]], mx, my, P.ann_h2x2);
        keep |= (k && bit < 32u) ? (1u << bit) : 0u;
        far |= k && bit >= 32u;
      }
      while (keep) {
        const uint32_t bit = (uint32_t)(__ffs(keep) - 1);
        keep &= keep - 1u;
        const int k = C.S.clist[C.b + bit];
        const bool m = may(C.S.geo[k], C.S.aux[k]);
        mmask |= m ? (1u << bit) : 0u;
      }
      maybe = mmask != 0u || far;
    } else {
      for (uint32_t j = C.b; j < C.e; ++j) {
        const int k = C.S.clist[j];
        const bool m = may(C.S.geo[k], C.S.aux[k]);
        maybe |= m;
        const uint32_t bit = j - C.b;
        mmask |= (m || bit >= 32u) ? (1u << (bit & 31u)) : 0u;
      }
    }
  }
  return maybe;
}

// The nearest-hit loop of a move whose pre-filter passed: reflections,
// transmissions and the end point.
template <int GEOM, bool PERM, bool ONE>
__device__ __forceinline__ MoveOut hit_loop(const WalkParams &P, const Cands<GEOM, ONE> &C,
                                            float sx, float sy, float sz, float dx, float dy,
                                            float dz, float L, float v, DevStream &st, float Lb,
                                            uint32_t mmask, float bh1, float c01, float c11) {
  MoveOut o;
  o.hits = 0;
  o.capped = false;
  o.crossed = false;
  float rem = L;
  int last = -1;
  while (true) {
    const float aa_c = fma_f(dx, dx, dy * dy);
    const float aa_s = fma_f(dx, dx, fma_f(dy, dy, dz * dz));
    float best = AXX_INF;
    int bk = -1;
    float4 bg, ba;
    if (ONE) {
      // the only instance: the first pass reuses the pre-filter's quadratic;
      // after a hit the start is on its surface
      const bool sph = is_sphere<GEOM>(C.a0);
      const float aa = sph ? aa_s : aa_c;
      if (is_plane<GEOM>(C.a0))
        best = plane_hit(C.g0, C.a0.y, last == 0, sx, sy, sz, dx, dy, dz, rem);
      else if (last < 0)
        best = seg_root(bh1, c01, c11, C.a0.y, aa, rem);
      else
        best = surface_hit(C.g0, C.a0.y, sph, sx, sy, sz, dx, dy, dz, aa, rem);
      if (best < AXX_INF) bk = 0;
      bg = C.g0;
      ba = C.a0;
    } else {
      // after a hit: the annulus test of the remaining segment (cylinder
      // lists; the instance just hit is tested from its surface)
      const float hl = 0.5f * rem;
      const float mx = fma_f(hl, dx, sx), my = fma_f(hl, dy, sy);
      auto test = [&](uint32_t j) {
        const int k = C.S.clist[j];
        if (GEOM == AXX_GEOM_CYL && PERM && last >= 0 && k != last &&
            !annulus_keeps(C.S.geo[k], mx, my, P.ann_h2x2))
          return;
        const float4 aux = C.S.aux[k];
        const bool sph = is_sphere<GEOM>(aux);
        const float s =
            is_plane<GEOM>(aux)
                ? plane_hit(C.S.geo[k], aux.y, k == last, sx, sy, sz, dx, dy, dz, rem)
                : seg_hit(C.S.geo[k], aux.y, sph, k == last, sx, sy, sz, dx, dy, dz,
                          sph ? aa_s : aa_c, rem);
        if (s < best) {
          best = s;
          bk = k;
        }
      };
      if (last < 0) {
        // first pass: the candidates the pre-filter kept, in list order (the
        // others would be rejected the same way), then any past the 32nd
        for (uint32_t m = mmask; m != 0u; m &= m - 1u) test(C.b + (uint32_t)(__ffs(m) - 1));
        for (uint32_t j = C.b + 32u; j < C.e; ++j) test(j);
      } else {
        for (uint32_t j = C.b; j < C.e; ++j) test(j);
      }
      if (bk >= 0) {
        bg = C.S.geo[bk];
        ba = C.S.aux[bk];
      }
    }
    if (bk < 0) break;
    if (o.hits == AXX_REFL_CAP) {
      o.capped = true;
      o.fx = sx;
      o.fy = sy;
      o.fz = sz;
      return o;
    }
    const float hx = fma_f(best, dx, sx), hy = fma_f(best, dy, sy), hz = fma_f(best, dz, sz);
    const float rem_before = rem;
    rem = (o.hits == 0 ? Lb : rem) - best;
    ++o.hits;
    if (PERM) {
      const float u = st.next(P);
      const float ptr = div_f(C.S.slot[aux_slot(ba)].w, v);
      if (!(u > ptr)) {  // transmitted: continue with the speed of the far side
        const float tx = fma_f(rem_before, dx, sx), ty = fma_f(rem_before, dy, sy),
                    tz = fma_f(rem_before, dz, sz);
        const int ts = C.lookup(P.ecs_slot, tx, ty, tz);
        const float vn = C.S.slot[ts].x;
        const float remt = div_f(rem * vn, v);
        o.fx = fma_f(remt, dx, hx);
        o.fy = fma_f(remt, dy, hy);
        o.fz = fma_f(remt, dz, hz);
        o.crossed = true;
        return o;
      }
    }
    // unit normal: radial for cylinders and spheres, the stored normal of a
    // plane (Plane::getNormal)
    const bool pl = is_plane<GEOM>(ba);
    const bool n3 = is_sphere<GEOM>(ba) || pl;
    float nx, ny, nz;
    if (pl) {
      nx = bg.x;
      ny = bg.y;
      nz = bg.z;
    } else {
      nx = (hx - bg.x) * ba.x;
      ny = (hy - bg.y) * ba.x;
      nz = n3 ? (hz - bg.z) * ba.x : 0.0f;
    }
    const float dn = n3 ? fma_f(dx, nx, fma_f(dy, ny, dz * nz)) : fma_f(dx, nx, dy * ny);
    const float t = -2.0f * dn;
    dx = fma_f(t, nx, dx);
    dy = fma_f(t, ny, dy);
    if (n3) dz = fma_f(t, nz, dz);
    sx = hx;
    sy = hy;
    sz = hz;
    last = bk;
  }
  o.fx = fma_f(rem, dx, sx);
  o.fy = fma_f(rem, dy, sy);
  o.fz = fma_f(rem, dz, sz);
  return o;
}

// The move's end without a wall met.
__device__ __forceinline__ MoveOut free_move(float sx, float sy, float sz, float dx, float dy,
                                             float dz, float L) {
  MoveOut o;
  o.hits = 0;
  o.capped = false;
  o.crossed = false;
  o.fx = fma_f(L, dx, sx);
  o.fy = fma_f(L, dy, sy);
  o.fz = fma_f(L, dz, sz);
  return o;
}

// Specular boundary handling of one move, general substrates and single
// instances alike.  A cheap test decides for every candidate whether the
// segment can meet it at all; the warp votes, and only lanes that may hit
// run the full nearest-hit loop.
// L is the move's segment length, Lb its path budget, which replaces L at the
// first hit (lattice picking: a sqrt(3) L diagonal segment, budget L).
template <int GEOM, bool PERM, bool ONE>
__device__ __forceinline__ MoveOut boundary(const WalkParams &P, const Cands<GEOM, ONE> &C,
                                            float sx, float sy, float sz, float dx, float dy,
                                            float dz, float L, float v, DevStream &st,
                                            float Lb) {
  uint32_t mmask;
  float bh1 = 0.0f, c01 = 0.0f, c11 = 0.0f;
  const bool maybe =
      prefilter<GEOM, PERM, ONE>(P, C, sx, sy, sz, dx, dy, dz, L, mmask, bh1, c01, c11);
  if (!__any_sync(__activemask(), maybe) || !maybe) return free_move(sx, sy, sz, dx, dy, dz, L);
  return hit_loop<GEOM, PERM, ONE>(P, C, sx, sy, sz, dx, dy, dz, L, v, st, Lb, mmask, bh1, c01,
                                   c11);
}

// PAX value of the axis-channel instantiations (channel 3w + a is waveform w
// along axis a; every axis carries phase: bits x, y, z set, and bit 3)
#define AXX_PAX_AXES 15

// A channel's projection p . r, fma(p_z, z, fma(p_y, y, p_x x)), over the
// axes in PAX: a term of a zero coefficient adds a zero, so leaving it out
// gives the same value (up to the sign of a zero sum).
template <int PAX>
__device__ __forceinline__ float project(const float p[3], float x, float y, float z) {
  float d;
  if ((PAX & 3) == 3)
    d = fma_f(p[1], y, p[0] * x);
  else if (PAX & 1)
    d = p[0] * x;
  else if (PAX & 2)
    d = p[1] * y;
  else
    d = 0.0f;
  return (PAX & 4) ? fma_f(p[2], z, d) : d;
}

// seg_root for a segment that passes its first rejections (seg_may holds),
// with selects in place of the early returns: the same operations on the
// same operands, so the same value, and one square root and one division
// whatever the case.
__device__ __forceinline__ float seg_root_may(float bh, float c0, float eps, float aa,
                                              float rem) {
  const bool in = c0 < 0.0f, out = c0 > 0.0f, lo = bh <= 0.0f;
  const float disc = fma_f(bh, bh, -(aa * c0));  // > 0 inside (aa > 0)
  const float sq = sqrt_f(disc > 0.0f ? disc : 0.0f);
  const float num = in ? (lo ? sq - bh : -c0) : (out ? c0 : -2.0f * bh);
  const float den = in ? (lo ? aa : bh + sq) : (out ? sq - bh : aa);
  const float s = div_f(num, den);
  const bool ok = !(out && disc <= 0.0f) && s > 0.0f && s < rem && s >= eps;
  return ok ? s : AXX_INF;
}

// boundary() for a single cylinder or sphere held in registers: the same
// passes, the first from the pre-filter's quadratic (seg_root_may), the later
// ones from the surface (surface_hit), with the loop test on the pass's result.
template <int GEOM, bool PERM>
__device__ __forceinline__ MoveOut boundary_one(const WalkParams &P, const Cands<GEOM, true> &C,
                                                float sx, float sy, float sz, float dx, float dy,
                                                float dz, float L, float v, DevStream &st,
                                                float Lb) {
  static_assert(GEOM == AXX_GEOM_CYL || GEOM == AXX_GEOM_SPH, "one cylinder or sphere");
  constexpr bool sph = GEOM == AXX_GEOM_SPH;
  const float4 g = C.g0, a = C.a0;
  float aa = sph ? fma_f(dx, dx, fma_f(dy, dy, dz * dz)) : fma_f(dx, dx, dy * dy);
  float bh, c0, c1;
  seg_coef(g, sph, sx, sy, sz, dx, dy, dz, L, bh, c0, c1);
  const bool maybe = seg_may_disc(bh, c0, c1, aa, L);
  MoveOut o;
  o.hits = 0;
  o.capped = false;
  o.crossed = false;
  o.fx = fma_f(L, dx, sx);
  o.fy = fma_f(L, dy, sy);
  o.fz = fma_f(L, dz, sz);
  if (!__any_sync(__activemask(), maybe) || !maybe) return o;
  float rem = L;
  float best = seg_root_may(bh, c0, a.y, aa, rem);
  while (best < AXX_INF) {
    if (o.hits == AXX_REFL_CAP) {
      o.capped = true;
      o.fx = sx;
      o.fy = sy;
      o.fz = sz;
      return o;
    }
    const float hx = fma_f(best, dx, sx), hy = fma_f(best, dy, sy), hz = fma_f(best, dz, sz);
    const float rem_before = rem;
    rem = (o.hits == 0 ? Lb : rem) - best;
    ++o.hits;
    if (PERM) {
      const float u = st.next(P);
      const float ptr = div_f(C.S.slot[aux_slot(a)].w, v);
      if (!(u > ptr)) {  // transmitted: continue with the speed of the far side
        const float tx = fma_f(rem_before, dx, sx), ty = fma_f(rem_before, dy, sy),
                    tz = fma_f(rem_before, dz, sz);
        const int ts = C.lookup(P.ecs_slot, tx, ty, tz);
        const float vn = C.S.slot[ts].x;
        const float remt = div_f(rem * vn, v);
        o.fx = fma_f(remt, dx, hx);
        o.fy = fma_f(remt, dy, hy);
        o.fz = fma_f(remt, dz, hz);
        o.crossed = true;
        return o;
      }
    }
    const float nx = (hx - g.x) * a.x, ny = (hy - g.y) * a.x;
    const float nz = sph ? (hz - g.z) * a.x : 0.0f;
    const float dn = sph ? fma_f(dx, nx, fma_f(dy, ny, dz * nz)) : fma_f(dx, nx, dy * ny);
    const float t = -2.0f * dn;
    dx = fma_f(t, nx, dx);
    dy = fma_f(t, ny, dy);
    if (sph) dz = fma_f(t, nz, dz);
    sx = hx;
    sy = hy;
    sz = hz;
    aa = sph ? fma_f(dx, dx, fma_f(dy, dy, dz * dz)) : fma_f(dx, dx, dy * dy);
    best = surface_hit(g, a.y, sph, sx, sy, sz, dx, dy, dz, aa, rem);
  }
  o.fx = fma_f(rem, dx, sx);
  o.fy = fma_f(rem, dy, sy);
  o.fz = fma_f(rem, dz, sz);
  return o;
}

// Branch-free periodic wrap (Lattice::lmod for a displacement below one cell).
__device__ __forceinline__ float wrap_sel(float x, float a) {
  const float hi = x - a, lo = x + a;
  return (x > a) ? hi : ((x < 0.0f) ? lo : x);
}

// The end of move i of walker W: the position after the boundary handling
// (fx, fy, fz), its boundary hits and whether it crossed a permeable wall;
// the wrap, the phase terms, the region and T2 bookkeeping and the trace.
// s4 holds the slot values the move started with (speed, step, dt/T2).
template <int GEOM, int KMAX, int KM, bool TRACE, bool ONE, bool DEFER, int PAX>
__device__ __forceinline__ void move_tail(const WalkParams &P, const SmemView &S,
                                          const TraceParams &T, long long wid, int i,
                                          const DevStream &st, Walker<KMAX> &W,
                                          const Cands<GEOM, ONE> &C, const float4 &s4, float fx,
                                          float fy, float fz, int hits, bool crossed) {
  constexpr bool single = KM >= AXX_KM_SINGLE;
  constexpr bool perm = KM == AXX_KM_LAT_PERM;
  constexpr bool tracked = KM == AXX_KM_LAT_IMP || KM == AXX_KM_LAT_PERM;
  constexpr bool PX = PAX & 1, PY = PAX & 2, NOZ = !(PAX & 4);
  const float4 g0 = C.g0, a0 = C.a0;
  float px, py, pz;  // position seen by the phase
  bool wrapped = false;
  if (single) {
    px = fx;
    py = fy;
    pz = fz;
  } else {
    if (PX) W.ux = W.ux + (fx - W.x);
    if (PY) W.uy = W.uy + (fy - W.y);
    if (!NOZ) W.uz = W.uz + (fz - W.z);
    px = W.ux;
    py = W.uy;
    pz = W.uz;
    const float ox = fx, oy = fy, oz = fz;
    fx = wrap_sel(fx, P.a);
    fy = wrap_sel(fy, P.b);
    if (!NOZ) fz = wrap_sel(fz, P.c);
    wrapped = (fx != ox) || (fy != oy) || (fz != oz);
  }
  // phase channels: s_c(i) is wave_il[i*KMAX + c]; padded channels carry
  // zero waveforms and zero projections
  const float *wrow = P.wave_il + (size_t)i * KMAX;
  float wv[KMAX];
  if constexpr (PAX == AXX_PAX_AXES) {
    // channel 3w + a: waveform w along axis a; the projection is the
    // coordinate itself (the same value: fma(0, y, 1 * x) = x)
    static_assert(KMAX == 12, "axis channels: four waveforms along three axes");
    const float4 w4 = __ldg(P.wave4 + i);
    const float wq[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
    for (int c = 0; c < KMAX; ++c) {
      const float d = (c % 3 == 0) ? px : ((c % 3 == 1) ? py : pz);
      kahan_add(W.acc[c], W.cmp[c], wq[c / 3] * d);
    }
  } else if (KMAX % 4 == 0) {
    // rows of 4k floats start on 16-byte boundaries (the table is 256-aligned)
#pragma unroll
    for (int q = 0; q < KMAX / 4; ++q) {
      const float4 w4 = __ldg(reinterpret_cast<const float4 *>(wrow) + q);
      wv[4 * q] = w4.x;
      wv[4 * q + 1] = w4.y;
      wv[4 * q + 2] = w4.z;
      wv[4 * q + 3] = w4.w;
    }
  } else {
#pragma unroll
    for (int c = 0; c < KMAX; ++c) wv[c] = __ldg(&wrow[c]);
  }
  if constexpr (PAX == AXX_PAX_AXES) {
  } else if (KMAX > 1 && P.one_dir) {
    // every channel projects on the same direction (padded channels carry
    // zero waveforms): one projection serves all, the same bits as each
    const float d = project<PAX>(P.ch_p[0], px, py, pz);
#pragma unroll
    for (int c = 0; c < KMAX; ++c) {
      if (DEFER)
        W.part[c] = fma_f(wv[c], d, W.part[c]);
      else
        kahan_add(W.acc[c], W.cmp[c], wv[c] * d);
    }
  } else {
#pragma unroll
    for (int c = 0; c < KMAX; ++c) {
      const float d = project<PAX>(P.ch_p[c], px, py, pz);
      if (DEFER)
        W.part[c] = fma_f(wv[c], d, W.part[c]);
      else
        kahan_add(W.acc[c], W.cmp[c], wv[c] * d);
    }
  }
  // Behind specular walls a walker stays in its region: it is looked up
  // again only when the move wraps across the cell edge (into another listed
  // image, whose region id may differ) or crosses a permeable wall.  With a
  // single instance (no reachable ghost) a wrap never changes the region: an
  // impermeable walk then looks up nothing and forms its T2 sum at the end.
  // (The FP32 lookup of a position a rounding error from a wall could name
  // the other side; the FP64 reference's hardly ever does.)  Rejection walks
  // look the region up after every move.
  if (!single && tracked && !(ONE && !perm)) {
    // dt/T2 of the move's region (0 without relaxation); the permeable walk
    // weights the region after the move (accumtime is always 0)
    if (!perm) kahan_add(W.t2s, W.t2c, s4.z);
    if (GEOM != AXX_GEOM_FREE && (ONE ? crossed : (wrapped || crossed))) {
      if (ONE) {
        W.slot = C.lookup(P.ecs_slot, fx, fy, fz);
      } else {
        const int cell = cell_of<GEOM>(P, fx, fy, fz);
        W.slot =
            lookup_list<GEOM>(S, S.cstart[cell], S.cstart[cell + 1], P.ecs_slot, fx, fy, fz);
      }
      if (perm) {
        const float4 ns = S.slot[W.slot];
        W.v0 = ns.x;
        W.L0 = ns.y;
        W.t2z = ns.z;
      }
    }
    if (perm) {
      if (ONE)
        W.nin += (W.slot != P.ecs_slot) ? 1 : 0;
      else
        kahan_add(W.t2s, W.t2c, W.t2z);
    }
  }
  if (!single && !tracked) {  // rejection walks
    int new_slot = P.ecs_slot;
    if (GEOM != AXX_GEOM_FREE) {
      if (ONE) {
        new_slot = C.lookup(P.ecs_slot, fx, fy, fz);
      } else {
        const int cell = cell_of<GEOM>(P, fx, fy, fz);
        new_slot =
            lookup_list<GEOM>(S, S.cstart[cell], S.cstart[cell + 1], P.ecs_slot, fx, fy, fz);
      }
    }
    // dt/T2 of the move's region (0 without relaxation).  With one instance
    // there are two regions: count the moves in the instance's and form the
    // sum at the end.
    if (ONE)
      W.nin += (W.slot != P.ecs_slot) ? 1 : 0;
    else
      kahan_add(W.t2s, W.t2c, s4.z);
    W.slot = new_slot;
  }
  W.x = fx;
  W.y = fy;
  W.z = fz;
  if (TRACE && wid < T.ntrace) {
    const long long o = wid * (long long)(P.steps - 1) + (i - 1);
    T.pos[o * 3 + 0] = W.x;
    T.pos[o * 3 + 1] = W.y;
    T.pos[o * 3 + 2] = W.z;
    int rs = W.slot;
    if (single) rs = (c0_of(g0, is_sphere<GEOM>(a0), W.x, W.y, W.z) < 0.0f) ? 0 : -1;
    T.region[o] = (!single && rs == P.ecs_slot) ? -1 : rs;
    T.hits[o] = hits;
    T.words[o] = (int32_t)st.words_used();
  }}

// One move i of walker W with the uniforms (u1, u2); `words` is the stream
// position after the move's draws (for traces).
// PICK (single pore, LATTICE_PICKING, kernelPhase.cuh:31-35): the move is
// +-L along every axis, the signs in bits 0..2 of `signs` (x, y, z): a
// sqrt(3) L segment along a cube diagonal with path budget L.
// DEFER: the move's phase terms go to W.part (FP32 sums over a block of
// moves, folded into the compensated sums by the caller) instead of the
// compensated sums directly.
// PAX: the axes some channel projects on (bits x, y, z); the unbounded
// coordinate of any other axis feeds nothing and is not kept.  Without z
// (cylinders along z only) z enters neither a boundary test, a region lookup
// nor a phase term, so the walk keeps no z at all.
template <int GEOM, int KMAX, int KM, bool TRACE, bool ONE, bool PICK = false, bool DEFER = false,
          int PAX = 7>
__device__ __forceinline__ void do_move(const WalkParams &P, const SmemView &S,
                                        const TraceParams &T, long long wid, int i, float u1,
                                        float u2, DevStream &st, Walker<KMAX> &W,
                                        WalkResult &res, const float4 &g0, const float4 &a0,
                                        uint32_t signs = 0u) {
  constexpr bool single = KM >= AXX_KM_SINGLE;
  constexpr bool perm = KM == AXX_KM_LAT_PERM;
  constexpr bool reject = KM == AXX_KM_LAT_REJ || KM == AXX_KM_SINGLE_REJ;
  constexpr bool NOZ = !(PAX & 4);
  // a single pore, or one instance behind impermeable walls: the walker's
  // slot never changes, and its speed and step stay in registers (the T2
  // term, .z, is then not read per move)
  constexpr bool fixed_slot = ONE && (single || KM == AXX_KM_LAT_IMP);
  // permeable walks hold their slot's values in registers (reloaded when the
  // slot changes); impermeable list walks read them per move (the registers
  // would spill there)
  constexpr bool cached = fixed_slot || perm;
  const float4 s4 = cached ? make_float4(W.v0, W.L0, W.t2z, 0.0f) : S.slot[W.slot];
  const float v = s4.x, Lb = s4.y;
  float dx, dy, dz, L = Lb;
  if (PICK) {
    const float k = 0.57735026918962576451f;
    dx = (signs & 1u) ? k : -k;
    dy = (signs & 2u) ? k : -k;
    dz = (signs & 4u) ? k : -k;
    L = Lb * 1.7320508075688772935f;
  } else {
    direction(u1, u2, dx, dy, dz);
  }
  Cands<GEOM, ONE> C{S, g0, a0, 0u, 0u};
  if (GEOM != AXX_GEOM_FREE && !ONE) {
    const int cell = single ? 0 : cell_of<GEOM>(P, W.x, W.y, W.z);
    C.b = S.cstart[cell];
    C.e = S.cstart[cell + 1];
  }
  float fx, fy, fz;
  int hits = 0;
  bool crossed = false;
  if (GEOM == AXX_GEOM_FREE) {
    fx = fma_f(L, dx, W.x);
    fy = fma_f(L, dy, W.y);
    fz = fma_f(L, dz, W.z);
  } else if (reject) {
    fx = fma_f(L, dx, W.x);
    fy = fma_f(L, dy, W.y);
    fz = fma_f(L, dz, W.z);
    bool back;
    if (single) {
      back = !(c0_of(g0, is_sphere<GEOM>(a0), fx, fy, fz) < 0.0f);
    } else {
      const int s_new = C.lookup(P.ecs_slot, fx, fy, fz);
      back = S.region[s_new] != S.region[W.slot];
    }
    fx = back ? W.x : fx;
    fy = back ? W.y : fy;
    fz = back ? W.z : fz;
  } else {
    MoveOut o;
    if constexpr (ONE && (GEOM == AXX_GEOM_CYL || GEOM == AXX_GEOM_SPH))
      o = boundary_one<GEOM, perm>(P, C, W.x, W.y, W.z, dx, dy, dz, L, v, st, Lb);
    else
      o = boundary<GEOM, perm, ONE>(P, C, W.x, W.y, W.z, dx, dy, dz, L, v, st, Lb);
    fx = o.fx;
    fy = o.fy;
    fz = NOZ ? W.z : o.fz;
    hits = o.hits;
    crossed = o.crossed;
    res.hits += (unsigned)o.hits;
    res.caps += o.capped ? 1u : 0u;
  }
  move_tail<GEOM, KMAX, KM, TRACE, ONE, DEFER, PAX>(P, S, T, wid, i, st, W, C, s4, fx, fy, fz,
                                                    hits, crossed);
}

// One walker.  On return W holds the channel sums (value, Kahan
// compensation) and the T2 sum.  TRACE records every move of the walker when
// wid < ntrace.
template <int GEOM, int KMAX, int KM, bool TRACE, bool ONE, int PAX = 7>
__device__ __forceinline__ WalkResult walk_one(const WalkParams &P, const SmemView &S,
                                               const TraceParams &T, long long wid,
                                               Walker<KMAX> &W) {
  constexpr bool single = KM >= AXX_KM_SINGLE;
  constexpr bool perm = KM == AXX_KM_LAT_PERM;
  WalkResult res{0u, 0u, false, false};
  const float4 g0 = S.geo[0], a0 = S.aux[0];
  DevStream st;
  st.init(P, (uint64_t)(wid + P.walker_offset), 1u);
  float x = 0.0f, y = 0.0f, z = 0.0f;
  bool ok;
  if (single && P.init_quirk) {
    DevStream cp = st;  // the reference passes its curandState by value
    ok = init_position<GEOM, KM>(P, S, cp, x, y, z);
  } else {
    ok = init_position<GEOM, KM>(P, S, st, x, y, z);
  }
  res.init_fail = !ok;
  if (TRACE && wid < T.ntrace) {
    T.init_pos[wid * 3 + 0] = x;
    T.init_pos[wid * 3 + 1] = y;
    T.init_pos[wid * 3 + 2] = z;
  }
  W.x = W.ux = x;
  W.y = W.uy = y;
  W.z = W.uz = z;
#pragma unroll
  for (int c = 0; c < KMAX; ++c) {
    const float d = fma_f(P.ch_p[c][2], z, fma_f(P.ch_p[c][1], y, P.ch_p[c][0] * x));
    W.acc[c] = __ldg(&P.wave_il[c]) * d;
    W.cmp[c] = 0.0f;
  }
  W.t2s = 0.0f;
  W.t2c = 0.0f;
  W.nin = 0;
  W.slot = single ? 0 : P.ecs_slot;
  if (!single && GEOM != AXX_GEOM_FREE) {
    if (ONE) {
      W.slot = contains<GEOM>(g0, a0, x, y, z) ? aux_slot(a0) : P.ecs_slot;
    } else {
      const int cell = cell_of<GEOM>(P, x, y, z);
      W.slot = lookup_list<GEOM>(S, S.cstart[cell], S.cstart[cell + 1], P.ecs_slot, x, y, z);
    }
  }
  {
    const float4 s = S.slot[W.slot];
    W.v0 = s.x;
    W.L0 = s.y;
    W.t2z = s.z;
  }
  int i = 1;
  if constexpr (single) {
    if (P.picking) {
      // LATTICE_PICKING: three raw words per move, their low bits the signs
      // (randomSign, kernelSetup.cuh:13-15), drawn z, y, x as the compiled
      // reference evaluates the three Vector3 constructor arguments
      for (; i < P.steps; ++i) {
        if ((i & 1023) == 0 && P.abort_flag != nullptr && *P.abort_flag) {
          res.aborted = true;
          break;
        }
        const uint32_t wz = st.next_word(P), wy = st.next_word(P), wx = st.next_word(P);
        const uint32_t signs = (wx & 1u) | ((wy & 1u) << 1) | ((wz & 1u) << 2);
        do_move<GEOM, KMAX, KM, TRACE, ONE, true>(P, S, T, wid, i, 0.f, 0.f, st, W, res, g0, a0,
                                                  signs);
      }
      return res;
    }
  }
  // Two moves per Philox block when every walker of the warp has its stream
  // at a block boundary and moves draw nothing else (the lattice walk from a
  // uniform start); otherwise the general stream.  With up to 4 channels the
  // phase terms of up to 32 moves are summed in FP32 and then added to the
  // compensated sums (more channels keep per-move compensation: the block
  // sums would cost registers the list walk needs).
  constexpr bool defer = KMAX <= 4;
  if (!defer && !perm && __all_sync(__activemask(), st.pos == 4)) {
    for (; i + 1 < P.steps; i += 2) {
      if (((i + 1) & 1023) == 0 && P.abort_flag != nullptr && *P.abort_flag) {
        res.aborted = true;
        return res;
      }
      ++st.blk;
      st.load(P);
      const uint32_t w0 = st.b0, w1 = st.b1, w2 = st.b2, w3 = st.b3;
      st.pos = 2;
      do_move<GEOM, KMAX, KM, TRACE, ONE, false, false, PAX>(
          P, S, T, wid, i, word_to_uniform(w0), word_to_uniform(w1), st, W, res, g0, a0);
      st.pos = 4;
      do_move<GEOM, KMAX, KM, TRACE, ONE, false, false, PAX>(
          P, S, T, wid, i + 1, word_to_uniform(w2), word_to_uniform(w3), st, W, res, g0, a0);
    }
  }
  if (defer && !perm && __all_sync(__activemask(), st.pos == 4)) {
    while (i + 1 < P.steps) {
      if (((i - 1) & 1023) == 0 && P.abort_flag != nullptr && *P.abort_flag) {
        res.aborted = true;
        return res;
      }
#pragma unroll
      for (int c = 0; c < KMAX; ++c) W.part[c] = 0.0f;
      const int stop = min(i + 32, P.steps - 1);  // 16 pairs, or up to the last pair
      for (; i < stop; i += 2) {
        ++st.blk;
        st.load(P);
        const uint32_t w0 = st.b0, w1 = st.b1, w2 = st.b2, w3 = st.b3;
        st.pos = 2;
        do_move<GEOM, KMAX, KM, TRACE, ONE, false, defer, PAX>(
            P, S, T, wid, i, word_to_uniform(w0), word_to_uniform(w1), st, W, res, g0, a0);
        st.pos = 4;
        do_move<GEOM, KMAX, KM, TRACE, ONE, false, defer, PAX>(
            P, S, T, wid, i + 1, word_to_uniform(w2), word_to_uniform(w3), st, W, res, g0, a0);
      }
#pragma unroll
      for (int c = 0; c < KMAX; ++c) kahan_add(W.acc[c], W.cmp[c], W.part[c]);
    }
  }
  for (; i < P.steps; ++i) {
    if ((i & 1023) == 0 && P.abort_flag != nullptr && *P.abort_flag) {
      res.aborted = true;
      break;
    }
    float u1, u2;
    if (perm)
      st.next2_eager(P, u1, u2);
    else
      st.next2(P, u1, u2);
    do_move<GEOM, KMAX, KM, TRACE, ONE, false, false, PAX>(P, S, T, wid, i, u1, u2, st, W, res,
                                                          g0, a0);
  }

  if (!single && KM == AXX_KM_LAT_IMP && ONE) {  // the T2 sum of the walker's one region
    const double t = (double)(i - 1) * (double)S.slot[W.slot].z;
    W.t2s = (float)t;
    W.t2c = (float)((double)W.t2s - t);
  } else if (ONE && !single) {  // the T2 sum from the move counts of the two regions
    const float tin = S.slot[aux_slot(a0)].z, tout = S.slot[P.ecs_slot].z;
    const double t = (double)W.nin * (double)tin + (double)(i - 1 - W.nin) * (double)tout;
    W.t2s = (float)t;
    W.t2c = (float)((double)W.t2s - t);
  }
  return res;
}

// Whether the lattice walker `wid` starts inside a basis (region != 0): its
// start drawn again from the head of its stream, so the walk itself keeps
// no register for it.
template <int GEOM, int KM>
__device__ __forceinline__ bool starts_inside(const WalkParams &P, const SmemView &S,
                                           long long wid) {
  if (GEOM == AXX_GEOM_FREE) return false;
  DevStream st;
  st.init(P, (uint64_t)(wid + P.walker_offset), 1u);
  float x, y, z;
  init_position<GEOM, KM>(P, S, st, x, y, z);
  const int cell = cell_of<GEOM>(P, x, y, z);
  return S.region[lookup_list<GEOM>(S, S.cstart[cell], S.cstart[cell + 1], P.ecs_slot, x, y,
                                    z)] != 0;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// The walk kernel.  Dynamic shared memory: [warps][M][5] FP64 sums (none with
// per-warp rows in global memory), then the instances, cell starts and cell
// lists.
// ONEONLY: compiled for substrates of a single instance only (the host checks
// n_inst == 1 and ncell == 1); the list path is left out, which frees
// registers for one more resident block per SM.
// GT: the substrate tables stay in global memory (too large to stage in
// shared memory); a compile-time choice, so that the staged kernels keep
// their shared-memory loads.
// PAX: the axes the channels project on (bits x, y, z; the host checks that
// no channel has a component on another axis); an instantiation without z
// serves single-instance walks of a cylinder along z, which then walk no z.
template <int GEOM, int KMAX, int KM, bool TRACE, bool ONEONLY = false, bool GT = false,
          int PAX = 7>
__global__ void __launch_bounds__(AXX_BLOCK, ONEONLY && KMAX <= 4 ? AXX_MIN_BLOCKS + 1
                                                                 : AXX_MIN_BLOCKS_FOR(KMAX))
    walk_kernel(const __grid_constant__ WalkParams P, const __grid_constant__ TraceParams T) {
  static_assert(PAX == 7 || (GEOM == AXX_GEOM_CYL && ONEONLY && !TRACE) ||
                    (PAX == AXX_PAX_AXES && KMAX == 12 && !ONEONLY && !TRACE),
                "axes are dropped only from single-cylinder walks without traces");
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int warps = AXX_BLOCK / 32;
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double *wsum = reinterpret_cast<double *>(smem);
  const int M = P.M;
  // rows of sums: all walkers, then those starting inside a basis (the
  // compartment sums run in the general instantiations only)
  const int Mo = (!ONEONLY && P.compart) ? 2 * M : M;
  const long long gwarp = (long long)blockIdx.x * warps + wib;
  // the sums of this warp: per-warp rows in shared memory, folded into one
  // partial per block at the end, or (warp_rows) the warp's own row of the
  // partials in global memory (the row's address is formed where it is used,
  // so that it holds no register during the walk)
  auto warp_row = [&]() {
    return P.warp_rows ? P.partials + (size_t)gwarp * Mo * 5 : wsum + (size_t)wib * Mo * 5;
  };
  if (P.warp_rows) {
    double *wrow = warp_row();
    for (int j = lane; j < Mo * 5; j += 32) wrow[j] = 0.0;
  } else {
    for (int j = threadIdx.x; j < warps * Mo * 5; j += blockDim.x) wsum[j] = 0.0;
  }

  SmemView S;
  if constexpr (GT) {
    // tables beyond the shared-memory budget (thousands of bases): read in
    // place, through L1
    S.geo = P.inst_geo;
    S.aux = P.inst_aux;
    S.slot = P.slot_tab;
    S.cstart = P.cell_start;
    S.region = P.slot_region;
    S.clist = P.cell_list;
  } else {
    // stage the substrate tables (layout fixed by the host planner); the slot
    // tables, read when a walker's slot changes, stay in global memory
    float4 *sg = reinterpret_cast<float4 *>(smem + (P.warp_rows ? 0 : (size_t)warps * Mo * 5 *
                                                                          sizeof(double)));
    float4 *sa = sg + P.n_inst;
    uint32_t *sc = reinterpret_cast<uint32_t *>(sa + P.n_inst);
    uint16_t *sl = reinterpret_cast<uint16_t *>(sc + P.ncell + 1);
    for (int j = threadIdx.x; j < P.n_inst; j += blockDim.x) {
      sg[j] = P.inst_geo[j];
      sa[j] = P.inst_aux[j];
    }
    for (int j = threadIdx.x; j <= P.ncell; j += blockDim.x) sc[j] = P.cell_start[j];
    for (int j = threadIdx.x; j < P.n_list; j += blockDim.x) sl[j] = P.cell_list[j];
    S.geo = sg;
    S.aux = sa;
    S.slot = P.slot_tab;
    S.cstart = sc;
    S.region = P.slot_region;
    S.clist = sl;
  }
  __syncthreads();

  const long long ntask = (P.n_walkers + 31) / 32;
  const long long nwarp = (long long)gridDim.x * warps;
  unsigned caps = 0, hits = 0, init_fail = 0, aborted = 0, start_in = 0;
  // a single instance (one basis without reachable ghosts, or a single pore)
  // is held in registers instead of walking a list
  const bool one = (GEOM != AXX_GEOM_FREE) && P.n_inst == 1 && P.ncell == 1;
  for (long long task = gwarp; task < ntask; task += nwarp) {
    const long long wid = task * 32 + lane;
    const bool active = wid < P.n_walkers;
    Walker<KMAX> W;
#pragma unroll
    for (int c = 0; c < KMAX; ++c) W.acc[c] = W.cmp[c] = 0.0f;
    W.t2s = W.t2c = 0.0f;
    bool in0 = false;
    if (active) {
      WalkResult r;
      if constexpr (ONEONLY)
        r = walk_one<GEOM, KMAX, KM, TRACE, true, PAX>(P, S, T, wid, W);
      else if constexpr (KMAX > 4)  // (the list path serves one instance too)
        r = walk_one<GEOM, KMAX, KM, TRACE, false, PAX>(P, S, T, wid, W);
      else
        r = one ? walk_one<GEOM, KMAX, KM, TRACE, true>(P, S, T, wid, W)
                : walk_one<GEOM, KMAX, KM, TRACE, false>(P, S, T, wid, W);
      caps += r.caps;
      hits += r.hits;
      init_fail += r.init_fail ? 1u : 0u;
      aborted += r.aborted ? 1u : 0u;
      if constexpr (KM < AXX_KM_SINGLE && !ONEONLY) {
        if (P.compart) in0 = starts_inside<GEOM, KM>(P, S, wid);
        start_in += in0 ? 1u : 0u;
      }
    }
    // FP64 epilogue (reference: transformAndSumTwoVectors with
    // COS/SIN_EXP_BINARY, src/util/cudaVector.cu:165-171, src/util/misc.cuh:29-39)
    double ph[KMAX];
#pragma unroll
    for (int c = 0; c < KMAX; ++c) ph[c] = (double)W.acc[c] - (double)W.cmp[c];
    const double w = exp(-((double)W.t2s - (double)W.t2c));
    double *wrow = warp_row();
    for (int m = 0; m < M; ++m) {
      double ang = 0.0;
#pragma unroll
      for (int c = 0; c < KMAX; ++c) ang = fma(__ldg(&P.coef[m * KMAX + c]), ph[c], ang);
      double sn, cs;
      sincos(ang, &sn, &cs);
      const double xv = active ? cs * w : 0.0, yv = active ? sn * w : 0.0;
      const double s0 = warp_sum(xv), s1 = warp_sum(yv), s2 = warp_sum(xv * xv),
                   s3 = warp_sum(yv * yv), s4 = warp_sum(xv * yv);
      if (lane == 0) {
        double *d = wrow + (size_t)m * 5;
        d[0] += s0;
        d[1] += s1;
        d[2] += s2;
        d[3] += s3;
        d[4] += s4;
      }
      if (!ONEONLY && P.compart) {  // the same over the walkers that started inside a basis
        // (x and y only: the rows' other entries stay 0)
        const double t0 = warp_sum(in0 ? xv : 0.0), t1 = warp_sum(in0 ? yv : 0.0);
        if (lane == 0) {
          double *d = wrow + (size_t)(M + m) * 5;
          d[0] += t0;
          d[1] += t1;
        }
      }
    }
  }
  if (caps) atomicAdd(&P.counters[AXX_CNT_CAP], (unsigned long long)caps);
  if (hits) atomicAdd(&P.counters[AXX_CNT_HITS], (unsigned long long)hits);
  if (init_fail) atomicAdd(&P.counters[AXX_CNT_INIT_FAIL], (unsigned long long)init_fail);
  if (aborted) atomicAdd(&P.counters[AXX_CNT_ABORTED], (unsigned long long)aborted);
  if (!ONEONLY && start_in)
    atomicAdd(&P.counters[AXX_CNT_START_IN], (unsigned long long)start_in);
  if (P.warp_rows) return;  // each warp's row is its partial
  __syncthreads();
  for (int j = threadIdx.x; j < Mo * 5; j += blockDim.x) {
    double s = 0.0;
    for (int q = 0; q < warps; ++q) s += wsum[(size_t)q * Mo * 5 + j];
    P.partials[(size_t)blockIdx.x * Mo * 5 + j] = s;
  }
}

}  // namespace axx
