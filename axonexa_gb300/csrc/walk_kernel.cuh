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
//  2. phase channel c starts at s_w(0) (p_c . r);
//  3. moves i = 1..steps-1: v, L from the region at r (Lattice::getD,
//     lattice.cuh:118-132); direction from two uniforms; boundary handling
//     (boundaryCheckImpermeable / boundaryCheckPermeable / boundaryNormal,
//     boundaryCheck.cuh:2-113, or simple rejection, kernelLattice.cuh:73-77);
//     r_unb += r - ri; channel c += s_w(i) (p_c . r_unb) with Kahan
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
#pragma once
#include <cuda_runtime.h>
#include <math_constants.h>
#include "axx_rng.cuh"
#include "axx_walk.h"

namespace axx {

#define AXX_INF __int_as_float(0x7f800000)

struct GeoView {
  const float4 *geo;
  const float4 *aux;
  const uint32_t *cstart;
  const uint16_t *clist;
};

__device__ __forceinline__ int cell_of(const WalkParams &P, float x, float y, float z) {
  int ix = (int)(x * P.inv_hx);
  int iy = (int)(y * P.inv_hy);
  int iz = (int)(z * P.inv_hz);
  ix = min(max(ix, 0), P.gx - 1);
  iy = min(max(iy, 0), P.gy - 1);
  iz = min(max(iz, 0), P.gz - 1);
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

// |p|^2 - R^2 for the point (x, y, z) against one instance.
__device__ __forceinline__ float c0_of(const float4 &g, bool sph, float x, float y, float z) {
  const float px = x - g.x, py = y - g.y;
  if (sph) {
    const float pz = z - g.z;
    return fma_f(px, px, fma_f(py, py, fma_f(pz, pz, g.w)));
  }
  return fma_f(px, px, fma_f(py, py, g.w));
}

// First instance (ascending basis order) of list [b, e) that contains the
// point; its slot, or the extracellular slot.
template <int GEOM>
__device__ __forceinline__ int lookup_list(const GeoView &G, uint32_t b, uint32_t e, int ecs,
                                           float x, float y, float z) {
  for (uint32_t j = b; j < e; ++j) {
    const int k = G.clist[j];
    const float4 aux = G.aux[k];
    if (c0_of(G.geo[k], is_sphere<GEOM>(aux), x, y, z) < 0.0f) return aux_slot(aux);
  }
  return ecs;
}

template <int GEOM>
__device__ __forceinline__ int lookup_slot(const WalkParams &P, const GeoView &G, float x,
                                           float y, float z) {
  if (GEOM == AXX_GEOM_FREE) return P.ecs_slot;
  const int cell = cell_of(P, x, y, z);
  return lookup_list<GEOM>(G, G.cstart[cell], G.cstart[cell + 1], P.ecs_slot, x, y, z);
}

// Distance to the first boundary of one instance along the segment
// start + s*d, 0 < s < rem, or +inf.
__device__ __forceinline__ float seg_hit(const float4 &g, float eps, bool sph, bool on_surface,
                                         float sx, float sy, float sz, float dx, float dy,
                                         float dz, float aa, float rem) {
  const float px = sx - g.x, py = sy - g.y;
  const float pz = sph ? (sz - g.z) : 0.0f;
  float bh, c0, c1;
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
  if (on_surface) c0 = 0.0f;
  float s;
  if (c0 < 0.0f) {  // inside: the exit root
    if (c1 < 0.0f) return AXX_INF;
    const float disc = fma_f(bh, bh, -(aa * c0));
    const float sq = sqrt_f(disc);
    s = (bh <= 0.0f) ? div_f(sq - bh, aa) : div_f(-c0, bh + sq);
  } else if (c0 > 0.0f) {  // outside: the entry root
    if (bh >= 0.0f) return AXX_INF;
    if (c1 > 0.0f && fma_f(aa, rem, bh) <= 0.0f) return AXX_INF;
    const float disc = fma_f(bh, bh, -(aa * c0));
    if (disc <= 0.0f) return AXX_INF;
    const float sq = sqrt_f(disc);
    s = div_f(c0, sq - bh);
  } else {  // on the surface: the far root
    if (bh >= 0.0f) return AXX_INF;
    s = div_f(-2.0f * bh, aa);
  }
  if (!(s > 0.0f && s < rem && s >= eps)) return AXX_INF;
  return s;
}

struct MoveOut {
  float fx, fy, fz;
  int hits;
  bool capped;
};

// Specular boundary handling of one move from (sx, sy, sz) with unit
// direction d and length L, using the instance list [b, e).
template <int GEOM>
__device__ __forceinline__ MoveOut boundary_move(const WalkParams &P, const GeoView &G,
                                                 uint32_t b, uint32_t e, float sx, float sy,
                                                 float sz, float dx, float dy, float dz, float L,
                                                 float v, bool perm, Stream &st) {
  MoveOut o;
  o.hits = 0;
  o.capped = false;
  float rem = L;
  int last = -1;
  while (true) {
    const float aa_c = fma_f(dx, dx, dy * dy);
    const float aa_s = fma_f(dx, dx, fma_f(dy, dy, dz * dz));
    float best = AXX_INF;
    int bk = -1;
    for (uint32_t j = b; j < e; ++j) {
      const int k = G.clist[j];
      const float4 aux = G.aux[k];
      const bool sph = is_sphere<GEOM>(aux);
      const float s = seg_hit(G.geo[k], aux.y, sph, k == last, sx, sy, sz, dx, dy, dz,
                              sph ? aa_s : aa_c, rem);
      if (s < best) {
        best = s;
        bk = k;
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
    ++o.hits;
    const float hx = fma_f(best, dx, sx), hy = fma_f(best, dy, sy), hz = fma_f(best, dz, sz);
    const float rem_before = rem;
    rem = rem - best;
    const float4 aux = G.aux[bk];
    if (perm) {
      const float u = st.next();
      const float ptr = div_f(P.slot_tab[aux_slot(aux)].w, v);
      if (!(u > ptr)) {  // transmitted: continue with the speed of the far side
        const float tx = fma_f(rem_before, dx, sx), ty = fma_f(rem_before, dy, sy),
                    tz = fma_f(rem_before, dz, sz);
        const int ts = lookup_list<GEOM>(G, b, e, P.ecs_slot, tx, ty, tz);
        const float vn = P.slot_tab[ts].x;
        const float remt = div_f(rem * vn, v);
        o.fx = fma_f(remt, dx, hx);
        o.fy = fma_f(remt, dy, hy);
        o.fz = fma_f(remt, dz, hz);
        return o;
      }
    }
    const float4 g = G.geo[bk];
    const bool sph = is_sphere<GEOM>(aux);
    const float nx = (hx - g.x) * aux.x, ny = (hy - g.y) * aux.x;
    const float nz = sph ? (hz - g.z) * aux.x : 0.0f;
    const float dn = sph ? fma_f(dx, nx, fma_f(dy, ny, dz * nz)) : fma_f(dx, nx, dy * ny);
    const float t = -2.0f * dn;
    dx = fma_f(t, nx, dx);
    dy = fma_f(t, ny, dy);
    if (sph) dz = fma_f(t, nz, dz);
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

__device__ __forceinline__ void kahan_add(float &s, float &c, float y) {
  const float yy = y - c;
  const float t = s + yy;
  c = (t - s) - yy;
  s = t;
}

__device__ __forceinline__ float wrap1(float x, float a) {
  if (x > a) return x - a;
  if (x < 0.0f) return x + a;
  return x;
}

// Start position.  Returns false if a rejection loop ran out of tries.
template <int GEOM>
__device__ __forceinline__ bool init_position(const WalkParams &P, const GeoView &G,
                                              Stream &st, float &x, float &y, float &z) {
  if (P.mode == AXX_MODE_SINGLE) {
    // Basis::unifRand (cylinderXY.cuh:45-55, Sphere.cuh:55-63).  The sphere's
    // box is centred on the sphere (the reference omits the centre, which
    // only agrees for a sphere at the origin); its retries draw z, y, x, the
    // order in which the compiled reference evaluates the three draws passed
    // as Vector3 constructor arguments.
    const float4 g = G.geo[P.init_inst];
    const bool sph = P.init_sph != 0;
    x = fma_f(fma_f(2.0f, st.next(), -1.0f), P.init_R, P.init_cx);
    y = fma_f(fma_f(2.0f, st.next(), -1.0f), P.init_R, P.init_cy);
    z = sph ? fma_f(fma_f(2.0f, st.next(), -1.0f), P.init_R, P.init_cz)
            : (2.0f * P.init_R) * st.next();
    for (int t = 0; t < AXX_INIT_TRIES; ++t) {
      if (c0_of(g, sph, x, y, z) < 0.0f) return true;
      if (sph) {
        z = fma_f(fma_f(2.0f, st.next(), -1.0f), P.init_R, P.init_cz);
        y = fma_f(fma_f(2.0f, st.next(), -1.0f), P.init_R, P.init_cy);
        x = fma_f(fma_f(2.0f, st.next(), -1.0f), P.init_R, P.init_cx);
      } else {
        x = fma_f(fma_f(2.0f, st.next(), -1.0f), P.init_R, P.init_cx);
        y = fma_f(fma_f(2.0f, st.next(), -1.0f), P.init_R, P.init_cy);
        z = (2.0f * P.init_R) * st.next();
      }
    }
    return false;
  }
  if (P.init_mode == 2) {
    // Basis::randUnif (cylinderXY.cuh:176-183, Sphere.cuh:384-391): the three
    // draws are Vector3 constructor arguments, consumed z, y, x; a cylinder's
    // centre has z = 0.
    const float4 g = G.geo[P.init_inst];
    const bool sph = P.init_sph != 0;
    for (int t = 0; t < AXX_INIT_TRIES; ++t) {
      const float tz = fma_f(2.0f, st.next(), -1.0f);
      y = fma_f(fma_f(2.0f, st.next(), -1.0f), P.init_R, P.init_cy);
      x = fma_f(fma_f(2.0f, st.next(), -1.0f), P.init_R, P.init_cx);
      z = sph ? fma_f(tz, P.init_R, P.init_cz) : tz * P.init_R;
      if (c0_of(g, sph, x, y, z) < 0.0f) return true;
    }
    return false;
  }
  for (int t = 0; t < AXX_INIT_TRIES; ++t) {
    x = st.next() * P.a;
    y = st.next() * P.b;
    z = st.next() * P.c;
    if (P.init_mode == 0) return true;
    // Lattice::initializeInRegion: region id of the first containing basis
    if (P.slot_region[lookup_slot<GEOM>(P, G, x, y, z)] == P.init_arg) return true;
  }
  return false;
}

// One walker: returns the channel sums (value - compensation) in phi[] and
// the T2 sum.  TRACE records every move of the first ntrace walkers.
template <int GEOM, int KMAX, bool TRACE>
__device__ __forceinline__ void walk_one(const WalkParams &P, const GeoView &G,
                                         const TraceParams &T, long long wid, float *phi,
                                         float &t2sum, bool &aborted) {
  const bool single = (P.mode == AXX_MODE_SINGLE);
  const bool relax = !single && (P.flags & 1u);
  const bool perm = !single && (P.flags & 2u);
  const bool reject = (P.flags & 4u) != 0;
  const uint64_t seed = ((uint64_t)P.seed_hi << 32) | P.seed_lo;
  const uint64_t gwid = (uint64_t)(wid + P.walker_offset);
  Stream st;
  st.init(seed, gwid, 1u);
  float x = 0.0f, y = 0.0f, z = 0.0f;
  bool ok;
  if (single && P.init_quirk) {
    Stream cp = st;  // the reference passes its curandState by value
    ok = init_position<GEOM>(P, G, cp, x, y, z);
  } else {
    ok = init_position<GEOM>(P, G, st, x, y, z);
  }
  if (!ok) atomicAdd(&P.counters[AXX_CNT_INIT_FAIL], 1ull);
  const long long tw = wid;  // trace index
  if (TRACE && tw < T.ntrace) {
    T.init_pos[tw * 3 + 0] = x;
    T.init_pos[tw * 3 + 1] = y;
    T.init_pos[tw * 3 + 2] = z;
  }
  float ux = x, uy = y, uz = z;  // unbounded position
  float acc[KMAX], cmp[KMAX];
#pragma unroll
  for (int c = 0; c < KMAX; ++c) {
    acc[c] = 0.0f;
    cmp[c] = 0.0f;
    if (c < P.K) {
      const float sw = __ldg(&P.wave[P.ch_wave[c] * P.steps]);
      const float d = fma_f(P.ch_p[c][2], z, fma_f(P.ch_p[c][1], y, P.ch_p[c][0] * x));
      acc[c] = sw * d;
    }
  }
  float t2s = 0.0f, t2c = 0.0f;
  int slot = single ? 0 : lookup_slot<GEOM>(P, G, x, y, z);
  unsigned long long caps = 0, nhits = 0;
  for (int i = 1; i < P.steps; ++i) {
    if ((i & 1023) == 0 && P.abort_flag != nullptr) {
      int f = 0;
      if ((threadIdx.x & 31) == 0) f = *P.abort_flag;
      f = __shfl_sync(__activemask(), f, 0);
      if (f) {
        aborted = true;
        break;
      }
    }
    float v, L;
    if (single) {
      v = P.single_speed;
      L = P.single_step;
    } else {
      const float4 s4 = P.slot_tab[slot];
      v = s4.x;
      L = s4.y;
    }
    float u1, u2;
    st.next2(u1, u2);
    float dx, dy, dz;
    direction(u1, u2, dx, dy, dz);
    float fx, fy, fz;
    int hits = 0;
    if (GEOM == AXX_GEOM_FREE) {
      fx = fma_f(L, dx, x);
      fy = fma_f(L, dy, y);
      fz = fma_f(L, dz, z);
    } else {
      const int cell = cell_of(P, x, y, z);
      const uint32_t b = G.cstart[cell], e = G.cstart[cell + 1];
      if (reject) {
        fx = fma_f(L, dx, x);
        fy = fma_f(L, dy, y);
        fz = fma_f(L, dz, z);
        int s_new;
        if (single) {
          s_new = (c0_of(G.geo[0], is_sphere<GEOM>(G.aux[0]), fx, fy, fz) < 0.0f) ? 0 : -1;
          if (s_new != 0) {
            fx = x;
            fy = y;
            fz = z;
          }
        } else {
          s_new = lookup_list<GEOM>(G, b, e, P.ecs_slot, fx, fy, fz);
          if (P.slot_region[s_new] != P.slot_region[slot]) {
            fx = x;
            fy = y;
            fz = z;
          }
        }
      } else {
        const MoveOut o = boundary_move<GEOM>(P, G, b, e, x, y, z, dx, dy, dz, L, v, perm, st);
        fx = o.fx;
        fy = o.fy;
        fz = o.fz;
        hits = o.hits;
        nhits += (unsigned long long)o.hits;
        caps += o.capped ? 1ull : 0ull;
      }
    }
    float px, py, pz;  // position seen by the phase
    if (single) {
      px = fx;
      py = fy;
      pz = fz;
    } else {
      ux = ux + (fx - x);
      uy = uy + (fy - y);
      uz = uz + (fz - z);
      px = ux;
      py = uy;
      pz = uz;
      fx = wrap1(fx, P.a);
      fy = wrap1(fy, P.b);
      fz = wrap1(fz, P.c);
    }
#pragma unroll
    for (int c = 0; c < KMAX; ++c) {
      if (c < P.K) {
        const float sw = __ldg(&P.wave[P.ch_wave[c] * P.steps + i]);
        const float d = fma_f(P.ch_p[c][2], pz, fma_f(P.ch_p[c][1], py, P.ch_p[c][0] * px));
        kahan_add(acc[c], cmp[c], sw * d);
      }
    }
    int new_slot = slot;
    if (!single && GEOM != AXX_GEOM_FREE) new_slot = lookup_slot<GEOM>(P, G, fx, fy, fz);
    if (relax) kahan_add(t2s, t2c, P.slot_tab[perm ? new_slot : slot].z);
    x = fx;
    y = fy;
    z = fz;
    slot = new_slot;
    if (TRACE && tw < T.ntrace) {
      const long long o = tw * (long long)(P.steps - 1) + (i - 1);
      T.pos[o * 3 + 0] = x;
      T.pos[o * 3 + 1] = y;
      T.pos[o * 3 + 2] = z;
      int rs = slot;
      if (single) rs = (c0_of(G.geo[0], is_sphere<GEOM>(G.aux[0]), x, y, z) < 0.0f) ? 0 : -1;
      T.region[o] = (rs == P.ecs_slot && !single) ? -1 : rs;
      T.hits[o] = hits;
      T.words[o] = (int32_t)st.words_used();
    }
  }
  if (caps) atomicAdd(&P.counters[AXX_CNT_CAP], caps);
  if (nhits) atomicAdd(&P.counters[AXX_CNT_HITS], nhits);
#pragma unroll
  for (int c = 0; c < KMAX; ++c) phi[2 * c] = acc[c], phi[2 * c + 1] = cmp[c];
  t2sum = t2s;
  (void)t2c;
  phi[2 * KMAX] = t2c;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// The walk kernel.  Dynamic shared memory: [warps][M][5] FP64 sums, then
// (if smem_geom) the instance arrays and the cell lists.
template <int GEOM, int KMAX, bool TRACE>
__global__ void __launch_bounds__(AXX_BLOCK) walk_kernel(const __grid_constant__ WalkParams P,
                                                         const __grid_constant__ TraceParams T) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int warps = AXX_BLOCK / 32;
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double *wsum = reinterpret_cast<double *>(smem);
  const int M = P.M;
  for (int j = threadIdx.x; j < warps * M * 5; j += blockDim.x) wsum[j] = 0.0;

  GeoView G;
  G.geo = P.inst_geo;
  G.aux = P.inst_aux;
  G.cstart = P.cell_start;
  G.clist = P.cell_list;
  if (P.smem_geom) {
    unsigned char *p = smem + (size_t)warps * M * 5 * sizeof(double);
    float4 *sg = reinterpret_cast<float4 *>(p);
    float4 *sa = sg + P.n_inst;
    uint32_t *sc = reinterpret_cast<uint32_t *>(sa + P.n_inst);
    uint16_t *sl = reinterpret_cast<uint16_t *>(sc + P.ncell + 1);
    for (int j = threadIdx.x; j < P.n_inst; j += blockDim.x) {
      sg[j] = P.inst_geo[j];
      sa[j] = P.inst_aux[j];
    }
    for (int j = threadIdx.x; j <= P.ncell; j += blockDim.x) sc[j] = P.cell_start[j];
    for (int j = threadIdx.x; j < P.n_list; j += blockDim.x) sl[j] = P.cell_list[j];
    G.geo = sg;
    G.aux = sa;
    G.cstart = sc;
    G.clist = sl;
  }
  __syncthreads();

  const long long ntask = (P.n_walkers + 31) / 32;
  const long long gwarp = (long long)blockIdx.x * warps + wib;
  const long long nwarp = (long long)gridDim.x * warps;
  const bool single = (P.mode == AXX_MODE_SINGLE);
  const bool relax = !single && (P.flags & 1u);
  bool aborted = false;
  for (long long task = gwarp; task < ntask; task += nwarp) {
    const long long wid = task * 32 + lane;
    const bool active = wid < P.n_walkers;
    float phi[2 * KMAX + 1];
    float t2 = 0.0f;
#pragma unroll
    for (int c = 0; c < 2 * KMAX + 1; ++c) phi[c] = 0.0f;
    if (active) walk_one<GEOM, KMAX, TRACE>(P, G, T, wid, phi, t2, aborted);
    // FP64 epilogue (reference: transformAndSumTwoVectors with COS/SIN_EXP_BINARY,
    // src/util/cudaVector.cu:165-171, src/util/misc.cuh:29-39)
    double ph[KMAX];
#pragma unroll
    for (int c = 0; c < KMAX; ++c) ph[c] = (double)phi[2 * c] - (double)phi[2 * c + 1];
    const double w = relax ? exp(-((double)t2 - (double)phi[2 * KMAX])) : 1.0;
    for (int m = 0; m < M; ++m) {
      double ang = 0.0;
#pragma unroll
      for (int c = 0; c < KMAX; ++c)
        if (c < P.K) ang = fma(__ldg(&P.coef[m * P.K + c]), ph[c], ang);
      double sn, cs;
      sincos(ang, &sn, &cs);
      const double xv = active ? cs * w : 0.0, yv = active ? sn * w : 0.0;
      const double s0 = warp_sum(xv), s1 = warp_sum(yv), s2 = warp_sum(xv * xv),
                   s3 = warp_sum(yv * yv), s4 = warp_sum(xv * yv);
      if (lane == 0) {
        double *d = wsum + ((size_t)wib * M + m) * 5;
        d[0] += s0;
        d[1] += s1;
        d[2] += s2;
        d[3] += s3;
        d[4] += s4;
      }
    }
  }
  if (aborted) atomicAdd(&P.counters[AXX_CNT_ABORTED], 1ull);
  __syncthreads();
  for (int j = threadIdx.x; j < M * 5; j += blockDim.x) {
    double s = 0.0;
    for (int q = 0; q < warps; ++q) s += wsum[(size_t)q * M * 5 + j];
    P.partials[(size_t)blockIdx.x * M * 5 + j] = s;
  }
}

}  // namespace axx
