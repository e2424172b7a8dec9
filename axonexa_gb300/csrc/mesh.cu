// mesh.cu -- a closed triangle mesh as a single pore.
//
// Reference: Mesh (src/primitives/mesh.cuh:1-75) and Triangle
// (src/primitives/triangle.cuh:1-59), drafts that do not compile (members
// that are never declared), meant for the single-pore walk of
// updateWalkersPhase (src/kernels/kernelPhase.cuh:4-66) with
// boundaryNormal (src/kernels/boundaryCheck.cuh:2-32):
//   * Triangle::intersect: the crossing of the segment with the triangle's
//     plane, v = n.(v0 - ri) / n.dr in (0, 1) and not within doub_equal of 0,
//     then Triangle::inside: barycentric coordinates (s, t) of the crossing,
//     s > 0, t > 0, s + t < 1;
//   * Mesh::intersect: the nearest triangle crossing and its normal;
//   * Mesh::inside: the parity of the triangles crossed by a ray from the
//     point along z.
// A walker's reflection off a face sits on that face's plane; in FP32 the
// draft's rule (any crossing not within 1e-14 of the start) re-hits the same
// plane through a coplanar neighbour and can ping-pong the walker out of the
// mesh, and a start rounded to just beyond a face would miss it.  Here the
// host orients every triangle outward (consistent winding across edges,
// positive volume per component) and a move counts only crossings from
// inside to outside (n.d > 0), from a start at most a rounding slack
// (4e-6 of the largest coordinate) beyond the face.
//
// GB300 formulation:
//  * per triangle: its vertices (FP32, the same values for every triangle
//    that shares them) and the unit outward normal n with n.v0; the hit test
//    is watertight (Woop, Benthin and Wald 2013): the ray's shear frame, then
//    edge functions that are exactly opposite for the two triangles of a
//    shared edge, so a ray through an edge or vertex cannot slip between
//    triangles (a barycentric test of the plane crossing leaves such gaps in
//    FP32, and walkers leaked through them at grazing incidence);
//  * a 3-D grid over the mesh's bounding box lists, per cell, the triangles
//    whose bounding box meets the cell dilated by one step: a move (at most
//    one step of path, reflections included) tests only its start cell's
//    list; cells away from the surface have empty lists;
//  * a 2-D (x, y) grid lists the triangles for the vertical-ray parity test
//    of the start (and the end-of-walk leak check), watertight as well: a
//    line through an edge or vertex counts for exactly one of its triangles
//    (a top-left rule); rays up and down must agree, else the point is
//    redrawn;
//  * the triangle tables are read through the read-only cache (a mesh of a
//    few thousand triangles fits in L1); the walker, its direction and its
//    phase channels stay in registers; FP64 sums per block as in the lattice
//    walk.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <string>
#include <vector>

#include "../../include/axx.h"
#include "ctx_internal.h"
#include "host_plan.h"
#include "plan_layout.h"
#include "walk_kernel.cuh"
#include "walk_launch.h"

namespace axx {

struct MeshArgs {
  const float4 *tri;   // [ntri][4]: v0, v1, v2 (outward winding), (n, n.v0)
  const uint32_t *c3s, *c3l;  // 3-D grid: cell starts, triangle lists
  const float4 *c3n;          // per list entry: the triangle's (n, n.v0), read in list order
  const uint32_t *c2s, *c2l;  // 2-D grid
  float lo[3], hi[3];  // bounding box
  float inv3[3];
  int g3[3];
  float inv2[2];
  int g2[2];
  float slack;
  unsigned long long *escaped;
};

// Whether the vertical line through (px, py) crosses the projection of the
// triangle (a, b, c) on (x, y), counting a line through an edge or vertex
// for exactly one of the triangles that share it: edge functions from the
// vertices relative to the point (exactly opposite for the two triangles of
// an edge), a zero edge function counting only for "top-left" edges
// (direction dy > 0, or dy = 0 and dx < 0, after orienting the projection
// counter-clockwise).
__device__ __forceinline__ bool covers_xy(float px, float py, const float4 &a, const float4 &b,
                                          const float4 &c) {
  const float ax = a.x - px, ay = a.y - py, bx = b.x - px, by = b.y - py;
  const float cx = c.x - px, cy = c.y - py;
  float e0 = bx * cy - by * cx;  // edge b -> c
  float e1 = cx * ay - cy * ax;  // edge c -> a
  float e2 = ax * by - ay * bx;  // edge a -> b
  const float area = e0 + e1 + e2;
  if (area == 0.0f) return false;
  const float sg = area > 0.0f ? 1.0f : -1.0f;
  e0 *= sg;
  e1 *= sg;
  e2 *= sg;
  auto tl = [&](float ux, float uy, float vx, float vy) {  // edge u -> v, oriented
    const float dx = (vx - ux) * sg, dy = (vy - uy) * sg;
    return dy > 0.0f || (dy == 0.0f && dx < 0.0f);
  };
  return (e0 > 0.0f || (e0 == 0.0f && tl(b.x, b.y, c.x, c.y))) &&
         (e1 > 0.0f || (e1 == 0.0f && tl(c.x, c.y, a.x, a.y))) &&
         (e2 > 0.0f || (e2 == 0.0f && tl(a.x, a.y, b.x, b.y)));
}

// Which side of the mesh (x, y, z) is on by vertical-ray parity
// (Mesh::inside): 1 inside, 0 outside, -1 when the rays up and down disagree
// (the point lies on the surface).
__device__ __forceinline__ int mesh_side(const MeshArgs &Q, float x, float y, float z) {
  const int ix = cell_index(x - Q.lo[0], Q.inv2[0], Q.g2[0]);
  const int iy = cell_index(y - Q.lo[1], Q.inv2[1], Q.g2[1]);
  const int cell = iy * Q.g2[0] + ix;
  int up = 0, down = 0;
  for (uint32_t j = __ldg(&Q.c2s[cell]), e = __ldg(&Q.c2s[cell + 1]); j < e; ++j) {
    const uint32_t k = __ldg(&Q.c2l[j]);
    const float4 a = __ldg(&Q.tri[4 * k]), b = __ldg(&Q.tri[4 * k + 1]),
                 c = __ldg(&Q.tri[4 * k + 2]), n = __ldg(&Q.tri[4 * k + 3]);
    if (!covers_xy(x, y, a, b, c)) continue;
    // the plane's height over (x, y)
    const float zh = div_f(n.w - fma_f(n.x, x, n.y * y), n.z);
    up += zh > z ? 1 : 0;
    down += zh < z ? 1 : 0;
  }
  if ((up & 1) != (down & 1)) return -1;
  return up & 1;
}

// The ray's shear frame (Woop, Benthin and Wald, "Watertight ray/triangle
// intersection", JCGT 2013): rows m0, m1 map a point relative to the ray's
// origin to 2-D coordinates in which the ray is the origin, m2 to its
// distance along the ray.  kz is the direction's largest component.
struct Shear {
  float m0x, m0y, m0z, m1x, m1y, m1z, m2x, m2y, m2z;
};

__device__ __forceinline__ Shear make_shear(float dx, float dy, float dz) {
  const float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
  const int kz = (ax > ay) ? ((ax > az) ? 0 : 2) : ((ay > az) ? 1 : 2);
  int kx = kz == 2 ? 0 : kz + 1, ky = kx == 2 ? 0 : kx + 1;
  const float dkz = kz == 0 ? dx : (kz == 1 ? dy : dz);
  if (dkz < 0.0f) {  // keep the winding
    const int t = kx;
    kx = ky;
    ky = t;
  }
  const float dkx = kx == 0 ? dx : (kx == 1 ? dy : dz);
  const float dky = ky == 0 ? dx : (ky == 1 ? dy : dz);
  const float sx = div_f(dkx, dkz), sy = div_f(dky, dkz), sz = div_f(1.0f, dkz);
  auto row = [&](int k, float sk, float &cx, float &cy, float &cz) {
    cx = k == 0 ? 1.0f : (kz == 0 ? -sk : 0.0f);
    cy = k == 1 ? 1.0f : (kz == 1 ? -sk : 0.0f);
    cz = k == 2 ? 1.0f : (kz == 2 ? -sk : 0.0f);
  };
  Shear M;
  row(kx, sx, M.m0x, M.m0y, M.m0z);
  row(ky, sy, M.m1x, M.m1y, M.m1z);
  M.m2x = kz == 0 ? sz : 0.0f;
  M.m2y = kz == 1 ? sz : 0.0f;
  M.m2z = kz == 2 ? sz : 0.0f;
  return M;
}

// Distance along the ray to the triangle (a, b, c), or +inf on a miss.  A
// vertex's sheared coordinates depend only on the vertex and the ray, and an
// edge function is a difference of two products: the two triangles of a
// shared edge get exactly opposite values, so no ray slips between them.
// Zero edge functions count as hits (a ray through an edge meets both).
__device__ __forceinline__ float watertight_hit(const Shear &M, float px, float py, float pz,
                                                const float4 &a, const float4 &b,
                                                const float4 &c) {
  const float ax = a.x - px, ay = a.y - py, az = a.z - pz;
  const float bx = b.x - px, by = b.y - py, bz = b.z - pz;
  const float cx = c.x - px, cy = c.y - py, cz = c.z - pz;
  const float Ax = fma_f(M.m0x, ax, fma_f(M.m0y, ay, M.m0z * az));
  const float Ay = fma_f(M.m1x, ax, fma_f(M.m1y, ay, M.m1z * az));
  const float Bx = fma_f(M.m0x, bx, fma_f(M.m0y, by, M.m0z * bz));
  const float By = fma_f(M.m1x, bx, fma_f(M.m1y, by, M.m1z * bz));
  const float Cx = fma_f(M.m0x, cx, fma_f(M.m0y, cy, M.m0z * cz));
  const float Cy = fma_f(M.m1x, cx, fma_f(M.m1y, cy, M.m1z * cz));
  const float U = Cx * By - Cy * Bx;
  const float V = Ax * Cy - Ay * Cx;
  const float W = Bx * Ay - By * Ax;
  if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return AXX_INF;
  const float det = U + V + W;
  if (det == 0.0f) return AXX_INF;
  const float Az = fma_f(M.m2x, ax, fma_f(M.m2y, ay, M.m2z * az));
  const float Bz = fma_f(M.m2x, bx, fma_f(M.m2y, by, M.m2z * bz));
  const float Cz = fma_f(M.m2x, cx, fma_f(M.m2y, cy, M.m2z * cz));
  const float T = fma_f(U, Az, fma_f(V, Bz, W * Cz));
  return div_f(T, det);
}

// Nearest triangle crossing along start + s*d, s < rem, of the triangles
// whose outward normal the direction leaves through (so the face just
// reflected from, and the faces coplanar with it, never count again), the
// triangle `last` excluded: its distance, or +inf.  The start may lie up to
// `slack` beyond a face's plane (the FP32 rounding of a point on the face,
// a few ulps of the coordinates): it then meets the face at s <= 0.
__device__ __forceinline__ float mesh_hit(const MeshArgs &Q, uint32_t b, uint32_t e, int last,
                                          float px, float py, float pz, float dx, float dy,
                                          float dz, float rem, int &bk) {
  float best = AXX_INF;
  bk = -1;
  if (b == e) return best;
  const Shear M = make_shear(dx, dy, dz);
  for (uint32_t j = b; j < e; ++j) {
    // the normal comes with the list entry (consecutive entries share cache
    // lines); the vertices only for candidates that pass the plane tests
    const float4 n = __ldg(&Q.c3n[j]);
    const float dn = fma_f(n.x, dx, fma_f(n.y, dy, n.z * dz));
    if (!(dn > 0.0f)) continue;  // only crossings from inside to outside
    const float np = fma_f(n.x, px, fma_f(n.y, py, n.z * pz));
    const float dist = n.w - np;
    if (!(dist > -Q.slack)) continue;        // not beyond the face's plane
    if (!(dist < rem * dn)) continue;        // the plane lies beyond the path
    const int k = (int)__ldg(&Q.c3l[j]);
    if (k == last) continue;
    const float s = watertight_hit(M, px, py, pz, __ldg(&Q.tri[4 * k]),
                                   __ldg(&Q.tri[4 * k + 1]), __ldg(&Q.tri[4 * k + 2]));
    if (s < rem && s < best) {
      best = s;
      bk = k;
    }
  }
  return best;
}

template <int KMAX, bool TRACE>
__global__ void __launch_bounds__(AXX_BLOCK, AXX_MIN_BLOCKS_FOR(KMAX))
    mesh_kernel(const __grid_constant__ WalkParams P, const __grid_constant__ MeshArgs Q,
                const __grid_constant__ TraceParams T) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int warps = AXX_BLOCK / 32;
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double *wsum = reinterpret_cast<double *>(smem);
  const int M = P.M;
  for (int j = threadIdx.x; j < warps * M * 5; j += blockDim.x) wsum[j] = 0.0;
  __syncthreads();
  const long long ntask = (P.n_walkers + 31) / 32;
  const long long gwarp = (long long)blockIdx.x * warps + wib;
  const long long nwarp = (long long)gridDim.x * warps;
  const float4 s4 = __ldg(&P.slot_tab[0]);
  const float L = s4.y;  // speed * dt
  unsigned caps = 0, hits_all = 0, init_fail = 0, aborted = 0, escaped = 0;
  for (long long task = gwarp; task < ntask; task += nwarp) {
    const long long wid = task * 32 + lane;
    const bool active = wid < P.n_walkers;
    float acc[KMAX], cmp[KMAX];
#pragma unroll
    for (int c = 0; c < KMAX; ++c) acc[c] = cmp[c] = 0.0f;
    if (active) {
      DevStream st;
      st.init(P, (uint64_t)(wid + P.walker_offset), 1u);
      // start: uniform in the bounding box, redrawn until inside
      float x = 0.f, y = 0.f, z = 0.f;
      bool ok = false;
      for (int t = 0; t < AXX_INIT_TRIES && !ok; ++t) {
        x = fma_f(st.next(P), Q.hi[0] - Q.lo[0], Q.lo[0]);
        y = fma_f(st.next(P), Q.hi[1] - Q.lo[1], Q.lo[1]);
        z = fma_f(st.next(P), Q.hi[2] - Q.lo[2], Q.lo[2]);
        ok = mesh_side(Q, x, y, z) == 1;
      }
      init_fail += ok ? 0u : 1u;
      if (TRACE && wid < T.ntrace) {
        T.init_pos[wid * 3 + 0] = x;
        T.init_pos[wid * 3 + 1] = y;
        T.init_pos[wid * 3 + 2] = z;
      }
#pragma unroll
      for (int c = 0; c < KMAX; ++c) {
        const float d = fma_f(P.ch_p[c][2], z, fma_f(P.ch_p[c][1], y, P.ch_p[c][0] * x));
        acc[c] = __ldg(&P.wave_il[c]) * d;
      }
      for (int i = 1; i < P.steps; ++i) {
        if ((i & 1023) == 0 && P.abort_flag != nullptr && *P.abort_flag) {
          aborted += 1u;
          break;
        }
        float u1, u2, dx, dy, dz;
        st.next2(P, u1, u2);
        direction(u1, u2, dx, dy, dz);
        // the start cell's list covers every point within one step
        const int cx = cell_index(x - Q.lo[0], Q.inv3[0], Q.g3[0]);
        const int cy = cell_index(y - Q.lo[1], Q.inv3[1], Q.g3[1]);
        const int cz = cell_index(z - Q.lo[2], Q.inv3[2], Q.g3[2]);
        const int cell = (cz * Q.g3[1] + cy) * Q.g3[0] + cx;
        const uint32_t b = __ldg(&Q.c3s[cell]), e = __ldg(&Q.c3s[cell + 1]);
        float rem = L, sx = x, sy = y, sz = z;
        int last = -1, nh = 0;
        bool capped = false;
        while (true) {
          int bk;
          const float best = mesh_hit(Q, b, e, last, sx, sy, sz, dx, dy, dz, rem, bk);
          if (bk < 0) break;
          if (nh == AXX_REFL_CAP) {
            capped = true;
            break;
          }
          // boundaryNormal: to the hit, reflect, the rest of the path
          sx = fma_f(best, dx, sx);
          sy = fma_f(best, dy, sy);
          sz = fma_f(best, dz, sz);
          rem = rem - best;
          const float4 n = __ldg(&Q.tri[4 * bk + 3]);
          const float t = -2.0f * fma_f(dx, n.x, fma_f(dy, n.y, dz * n.z));
          dx = fma_f(t, n.x, dx);
          dy = fma_f(t, n.y, dy);
          dz = fma_f(t, n.z, dz);
          last = bk;
          ++nh;
        }
        if (capped) {
          x = sx;
          y = sy;
          z = sz;
        } else {
          x = fma_f(rem, dx, sx);
          y = fma_f(rem, dy, sy);
          z = fma_f(rem, dz, sz);
        }
        caps += capped ? 1u : 0u;
        hits_all += (unsigned)nh;
        const float *wrow = P.wave_il + (size_t)i * KMAX;
#pragma unroll
        for (int c = 0; c < KMAX; ++c) {
          const float d = fma_f(P.ch_p[c][2], z, fma_f(P.ch_p[c][1], y, P.ch_p[c][0] * x));
          kahan_add(acc[c], cmp[c], __ldg(&wrow[c]) * d);
        }
        if (TRACE && wid < T.ntrace) {
          const long long o = wid * (long long)(P.steps - 1) + (i - 1);
          T.pos[o * 3 + 0] = x;
          T.pos[o * 3 + 1] = y;
          T.pos[o * 3 + 2] = z;
          T.hits[o] = nh;
          T.words[o] = (int32_t)st.words_used();
        }
      }
      escaped += (ok && mesh_side(Q, x, y, z) == 0) ? 1u : 0u;
    }
    // FP64 epilogue: cos and sin of each sequence's phase
    double ph[KMAX];
#pragma unroll
    for (int c = 0; c < KMAX; ++c) ph[c] = (double)acc[c] - (double)cmp[c];
    for (int m = 0; m < M; ++m) {
      double ang = 0.0;
#pragma unroll
      for (int c = 0; c < KMAX; ++c) ang = fma(__ldg(&P.coef[m * KMAX + c]), ph[c], ang);
      double sn, cs;
      sincos(ang, &sn, &cs);
      const double xv = active ? cs : 0.0, yv = active ? sn : 0.0;
      const double s0 = warp_sum(xv), s1 = warp_sum(yv), s2 = warp_sum(xv * xv),
                   s3 = warp_sum(yv * yv), s4v = warp_sum(xv * yv);
      if (lane == 0) {
        double *d = wsum + ((size_t)wib * M + m) * 5;
        d[0] += s0;
        d[1] += s1;
        d[2] += s2;
        d[3] += s3;
        d[4] += s4v;
      }
    }
  }
  if (caps) atomicAdd(&P.counters[AXX_CNT_CAP], (unsigned long long)caps);
  if (hits_all) atomicAdd(&P.counters[AXX_CNT_HITS], (unsigned long long)hits_all);
  if (init_fail) atomicAdd(&P.counters[AXX_CNT_INIT_FAIL], (unsigned long long)init_fail);
  if (aborted) atomicAdd(&P.counters[AXX_CNT_ABORTED], (unsigned long long)aborted);
  if (escaped) atomicAdd(Q.escaped, (unsigned long long)escaped);
  __syncthreads();
  for (int j = threadIdx.x; j < M * 5; j += blockDim.x) {
    double s = 0.0;
    for (int q = 0; q < warps; ++q) s += wsum[(size_t)q * M * 5 + j];
    P.partials[(size_t)blockIdx.x * M * 5 + j] = s;
  }
}

namespace {

template <int KMAX, bool TRACE>
cudaError_t go_mesh(const WalkParams &P, const MeshArgs &Q, const TraceParams &T, int grid,
                    size_t smem, cudaStream_t s) {
  auto fn = mesh_kernel<KMAX, TRACE>;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  fn<<<grid, AXX_BLOCK, smem, s>>>(P, Q, T);
  return cudaGetLastError();
}

cudaError_t launch_mesh(int kmax, bool trace, const WalkParams &P, const MeshArgs &Q,
                        const TraceParams &T, int grid, size_t smem, cudaStream_t s) {
  if (trace) return go_mesh<1, true>(P, Q, T, grid, smem, s);
  switch (kmax) {
    case 1: return go_mesh<1, false>(P, Q, T, grid, smem, s);
    case 2: return go_mesh<2, false>(P, Q, T, grid, smem, s);
    case 4: return go_mesh<4, false>(P, Q, T, grid, smem, s);
    case 8: return go_mesh<8, false>(P, Q, T, grid, smem, s);
    case 16: return go_mesh<16, false>(P, Q, T, grid, smem, s);
  }
  return cudaErrorInvalidValue;
}

template <int KMAX>
int occ_mesh(size_t smem) {
  int n = 0;
  cudaFuncSetAttribute(mesh_kernel<KMAX, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, mesh_kernel<KMAX, false>, AXX_BLOCK,
                                                    smem) != cudaSuccess)
    return 0;
  return n;
}

int occupancy_mesh(int kmax, size_t smem) {
  switch (kmax) {
    case 1: return occ_mesh<1>(smem);
    case 2: return occ_mesh<2>(smem);
    case 4: return occ_mesh<4>(smem);
    case 8: return occ_mesh<8>(smem);
    case 16: return occ_mesh<16>(smem);
  }
  return 0;
}

struct DevBuf {
  void *p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

// Host tables of a mesh: per-triangle records and the two grids.
struct MeshPlan {
  std::vector<float4> tri;
  std::vector<uint8_t> vertical;  // |n_z| tiny: no transversal crossing with a vertical line
  std::vector<uint32_t> c3s, c3l, c2s, c2l;
  std::vector<float4> c3n;  // (n, n.v0) of each 3-D list entry
  double lo[3], hi[3];
  int g3[3], g2[2];
  float inv3[3], inv2[2];
};

// Orients every triangle outward: across each edge the two triangles must
// traverse it in opposite directions (flipping (b, c) where they do not), and
// each connected component's signed volume must be positive (else the whole
// component flips).  Fails unless every edge has exactly two triangles (a
// closed surface).
std::string orient_mesh(const axx_mesh &m, std::vector<int32_t> &tris) {
  const int nt = m.ntri;
  tris.assign(m.triangles, m.triangles + 3 * (size_t)nt);
  std::map<std::pair<int, int>, std::vector<int>> edges;
  for (int t = 0; t < nt; ++t)
    for (int j = 0; j < 3; ++j) {
      const int a = tris[3 * t + j], b = tris[3 * t + (j + 1) % 3];
      if (a == b) return "degenerate triangle " + std::to_string(t);
      edges[{std::min(a, b), std::max(a, b)}].push_back(t);
    }
  for (auto &kv : edges)
    if (kv.second.size() != 2)
      return "the mesh is not a closed surface (an edge has " +
             std::to_string(kv.second.size()) + " triangles)";
  auto dir = [&](int t, int a, int b) {  // +1 if t traverses a -> b, -1 if b -> a
    for (int j = 0; j < 3; ++j) {
      const int u = tris[3 * t + j], v = tris[3 * t + (j + 1) % 3];
      if (u == a && v == b) return 1;
      if (u == b && v == a) return -1;
    }
    return 0;
  };
  std::vector<int> comp(nt, -1);
  int ncomp = 0;
  for (int s0 = 0; s0 < nt; ++s0) {
    if (comp[s0] >= 0) continue;
    std::vector<int> queue{s0};
    comp[s0] = ncomp;
    for (size_t qi = 0; qi < queue.size(); ++qi) {
      const int t = queue[qi];
      for (int j = 0; j < 3; ++j) {
        const int a = tris[3 * t + j], b = tris[3 * t + (j + 1) % 3];
        for (int u : edges[{std::min(a, b), std::max(a, b)}]) {
          if (u == t) continue;
          if (comp[u] >= 0) {
            if (dir(u, a, b) == dir(t, a, b)) return "the mesh is not orientable";
            continue;
          }
          if (dir(u, a, b) == dir(t, a, b)) std::swap(tris[3 * u + 1], tris[3 * u + 2]);
          comp[u] = ncomp;
          queue.push_back(u);
        }
      }
    }
    ++ncomp;
  }
  std::vector<double> vol(ncomp, 0.0);
  for (int t = 0; t < nt; ++t) {
    const double *p0 = &m.vertices[3 * tris[3 * t]];
    const double *p1 = &m.vertices[3 * tris[3 * t + 1]];
    const double *p2 = &m.vertices[3 * tris[3 * t + 2]];
    vol[comp[t]] += p0[0] * (p1[1] * p2[2] - p1[2] * p2[1]) -
                    p0[1] * (p1[0] * p2[2] - p1[2] * p2[0]) +
                    p0[2] * (p1[0] * p2[1] - p1[1] * p2[0]);
  }
  for (int t = 0; t < nt; ++t)
    if (vol[comp[t]] < 0.0) std::swap(tris[3 * t + 1], tris[3 * t + 2]);
  return "";
}

std::string plan_mesh(const axx_mesh &m, double step, MeshPlan &o) {
  if (!m.vertices || !m.triangles || m.nvert < 4 || m.ntri < 4)
    return "a closed mesh needs at least 4 vertices and 4 triangles";
  if (m.ntri > (1 << 22)) return "at most 4,194,304 triangles";
  if (!(m.D > 0.0) || !std::isfinite(m.D)) return "mesh D must be > 0";
  for (int k = 0; k < 3; ++k) {
    o.lo[k] = 1e300;
    o.hi[k] = -1e300;
  }
  for (int v = 0; v < m.nvert; ++v)
    for (int k = 0; k < 3; ++k) {
      const double c = m.vertices[3 * v + k];
      if (!std::isfinite(c)) return "mesh vertices must be finite";
    }
  for (int t = 0; t < m.ntri; ++t)
    for (int j = 0; j < 3; ++j) {
      const int v = m.triangles[3 * t + j];
      if (v < 0 || v >= m.nvert) return "triangle vertex index out of range";
    }
  std::vector<int32_t> tris;
  std::string oerr = orient_mesh(m, tris);
  if (!oerr.empty()) return oerr;
  for (int t = 0; t < m.ntri; ++t)
    for (int j = 0; j < 3; ++j) {
      const int v = tris[3 * t + j];
      for (int k = 0; k < 3; ++k) {
        o.lo[k] = std::min(o.lo[k], m.vertices[3 * v + k]);
        o.hi[k] = std::max(o.hi[k], m.vertices[3 * v + k]);
      }
    }
  double ext[3], scale = 0.0;
  for (int k = 0; k < 3; ++k) {
    ext[k] = o.hi[k] - o.lo[k];
    scale = std::max(scale, ext[k]);
    if (!(ext[k] > 0.0)) return "the mesh must enclose a volume (flat bounding box)";
  }
  if (2.0 * step >= std::min(ext[0], std::min(ext[1], ext[2])))
    return "the step length must be below half the mesh's smallest extent";
  // per-triangle records (FP64 -> FP32)
  o.tri.resize((size_t)m.ntri * 4);
  o.vertical.assign(m.ntri, 0);
  std::vector<double> box((size_t)m.ntri * 6);
  for (int t = 0; t < m.ntri; ++t) {
    const double *p0 = &m.vertices[3 * tris[3 * t]];
    const double *p1 = &m.vertices[3 * tris[3 * t + 1]];
    const double *p2 = &m.vertices[3 * tris[3 * t + 2]];
    const double u[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
    const double v[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
    double n[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2],
                   u[0] * v[1] - u[1] * v[0]};
    const double nm = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (!(nm > 1e-12 * scale * scale)) return "degenerate triangle " + std::to_string(t);
    for (double &c : n) c /= nm;
    const double w = n[0] * p0[0] + n[1] * p0[1] + n[2] * p0[2];
    float4 *r = &o.tri[(size_t)t * 4];
    r[0] = make_float4((float)p0[0], (float)p0[1], (float)p0[2], 0.f);
    r[1] = make_float4((float)p1[0], (float)p1[1], (float)p1[2], 0.f);
    r[2] = make_float4((float)p2[0], (float)p2[1], (float)p2[2], 0.f);
    r[3] = make_float4((float)n[0], (float)n[1], (float)n[2], (float)w);
    o.vertical[t] = std::fabs(n[2]) < 1e-9 ? 1 : 0;
    for (int k = 0; k < 3; ++k) {
      box[(size_t)t * 6 + k] = std::min(p0[k], std::min(p1[k], p2[k]));
      box[(size_t)t * 6 + 3 + k] = std::max(p0[k], std::max(p1[k], p2[k]));
    }
  }
  // 3-D grid: cells about the size of a triangle (surface area / count), at
  // most four steps, so that cells away from the surface have empty lists
  const double area = 2.0 * (ext[0] * ext[1] + ext[1] * ext[2] + ext[2] * ext[0]);
  const double h = std::max(2.0 * step, std::min(std::sqrt(area / m.ntri), 4.0 * step));
  for (int k = 0; k < 3; ++k) {
    o.g3[k] = (int)std::min(64.0, std::max(1.0, std::floor(ext[k] / h)));
    o.inv3[k] = (float)(o.g3[k] / ext[k]);
  }
  const double dil = step * 1.01 + 1e-7 * scale;
  const size_t nc3 = (size_t)o.g3[0] * o.g3[1] * o.g3[2];
  o.c3s.assign(nc3 + 1, 0);
  std::vector<std::vector<uint32_t>> lists(nc3);
  for (int t = 0; t < m.ntri; ++t) {
    int c0[3], c1[3];
    for (int k = 0; k < 3; ++k) {
      const double cw = ext[k] / o.g3[k], slack = 1e-5 * cw;
      c0[k] = std::max(0, (int)std::floor((box[(size_t)t * 6 + k] - dil - slack - o.lo[k]) / cw));
      c1[k] = std::min(o.g3[k] - 1,
                       (int)std::floor((box[(size_t)t * 6 + 3 + k] + dil + slack - o.lo[k]) / cw));
    }
    for (int iz = c0[2]; iz <= c1[2]; ++iz)
      for (int iy = c0[1]; iy <= c1[1]; ++iy)
        for (int ix = c0[0]; ix <= c1[0]; ++ix)
          lists[((size_t)iz * o.g3[1] + iy) * o.g3[0] + ix].push_back((uint32_t)t);
  }
  for (size_t c = 0; c < nc3; ++c) {
    o.c3l.insert(o.c3l.end(), lists[c].begin(), lists[c].end());
    o.c3s[c + 1] = (uint32_t)o.c3l.size();
  }
  o.c3n.resize(o.c3l.size());
  for (size_t j = 0; j < o.c3l.size(); ++j) o.c3n[j] = o.tri[(size_t)o.c3l[j] * 4 + 3];
  // 2-D grid for the parity test (points; no dilation)
  const double h2 = std::sqrt(ext[0] * ext[1] / std::max(1, m.ntri / 4));
  for (int k = 0; k < 2; ++k) {
    o.g2[k] = (int)std::min(256.0, std::max(1.0, std::floor(ext[k] / h2)));
    o.inv2[k] = (float)(o.g2[k] / ext[k]);
  }
  const size_t nc2 = (size_t)o.g2[0] * o.g2[1];
  o.c2s.assign(nc2 + 1, 0);
  std::vector<std::vector<uint32_t>> l2(nc2);
  for (int t = 0; t < m.ntri; ++t) {
    if (o.vertical[t]) continue;
    int c0[2], c1[2];
    for (int k = 0; k < 2; ++k) {
      const double cw = ext[k] / o.g2[k], slack = 1e-5 * cw;
      c0[k] = std::max(0, (int)std::floor((box[(size_t)t * 6 + k] - slack - o.lo[k]) / cw));
      c1[k] = std::min(o.g2[k] - 1,
                       (int)std::floor((box[(size_t)t * 6 + 3 + k] + slack - o.lo[k]) / cw));
    }
    for (int iy = c0[1]; iy <= c1[1]; ++iy)
      for (int ix = c0[0]; ix <= c1[0]; ++ix) l2[(size_t)iy * o.g2[0] + ix].push_back((uint32_t)t);
  }
  for (size_t c = 0; c < nc2; ++c) {
    o.c2l.insert(o.c2l.end(), l2[c].begin(), l2[c].end());
    o.c2s[c + 1] = (uint32_t)o.c2l.size();
  }
  if (o.c3l.empty()) {
    o.c3l.push_back(0);
    o.c3n.push_back(make_float4(0.f, 0.f, 0.f, 0.f));
  }
  if (o.c2l.empty()) o.c2l.push_back(0);
  return "";
}

axx_status mesh_fail(axx_ctx *ctx, axx_status s, const std::string &m) {
  ctx->err = m;
  return s;
}

axx_status mesh_run(axx_ctx *ctx, const axx_mesh *mesh, const axx_sequence *seqs, int nseq,
                    const axx_run_params *params, double *mx, double *my, axx_stats *stats,
                    int64_t *escaped, int ntrace, float *init_pos, float *pos, int32_t *hits,
                    int32_t *words) {
  if (!ctx) return AXX_ERR_INVALID_ARG;
  if (!mesh || !params || nseq < 0 || (nseq > 0 && !seqs))
    return mesh_fail(ctx, AXX_ERR_INVALID_ARG, "NULL argument");
  const axx_run_params &p = *params;
  if (p.num_walkers < 1 || p.steps < 1 || !(p.timestep > 0.0) || !std::isfinite(p.timestep) ||
      !std::isfinite(p.gamma) || p.gamma < 0.0 || p.walker_offset < 0)
    return mesh_fail(ctx, AXX_ERR_INVALID_ARG, "invalid run parameters");
  if (p.flags != 0)
    return mesh_fail(ctx, AXX_ERR_UNSUPPORTED,
                     "mesh pores take specular reflection only (flags must be 0)");
  const double dt = p.timestep;
  const double speed = std::sqrt(6.0 * mesh->D / dt);
  MeshPlan mp;
  std::string err = plan_mesh(*mesh, speed * dt, mp);
  if (!err.empty()) return mesh_fail(ctx, AXX_ERR_INVALID_ARG, err);
  const double gamma = p.gamma > 0.0 ? p.gamma : kGammaDefault;
  SeqPlan sq;
  err = plan_sequences(seqs, nseq, p.steps, dt, gamma, sq);
  if (!err.empty()) return mesh_fail(ctx, AXX_ERR_INVALID_ARG, err);
  // the walk tables of a pore without instances: one slot (speed, step)
  GeomPlan g;
  g.geom = AXX_GEOM_FREE;
  g.slot_tab = {make_float4((float)speed, (float)(speed * dt), 0.f, 0.f)};
  g.slot_region = {1};
  g.ecs_slot = 0;
  g.cstart = {0, 0};
  g.lmax = (float)(speed * dt);
  const int M = nseq;
  KernelTables kt;
  err = make_kernel_tables(g, sq, M, p.steps, AXX_MODE_SINGLE, 0u, kt);
  if (!err.empty()) return mesh_fail(ctx, AXX_ERR_UNSUPPORTED, err);
  const bool trace = ntrace > 0;
  const int kmax = trace ? 1 : kt.kmax;
  if (trace && kt.K > 0) return mesh_fail(ctx, AXX_ERR_INVALID_ARG, "traces take no sequences");
  const size_t smem = (size_t)(AXX_BLOCK / 32) * M * 5 * sizeof(double);
  if (smem > AXX_SMEM_MAX) return mesh_fail(ctx, AXX_ERR_UNSUPPORTED, "too many sequences");
  const int occ = occupancy_mesh(kmax, smem);
  if (occ <= 0) return mesh_fail(ctx, AXX_ERR_CUDA, "mesh kernel cannot be resident");
  const long long nw = trace ? std::min<long long>(p.num_walkers, ntrace) : p.num_walkers;
  const long long ntask = (nw + 31) / 32;
  const long long want = (ntask + AXX_BLOCK / 32 - 1) / (AXX_BLOCK / 32);
  const int grid = (int)std::max<long long>(1, std::min<long long>(want, (long long)occ * ctx->nsm));

  const ArenaLayout L = arena_layout(g, kt, M);
  auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
  size_t off = up(L.fixed + L.per_block * grid);
  const size_t o_tri = off;
  off = up(off + mp.tri.size() * 16);
  const size_t o_c3s = off;
  off = up(off + mp.c3s.size() * 4);
  const size_t o_c3l = off;
  off = up(off + mp.c3l.size() * 4);
  const size_t o_c3n = off;
  off = up(off + mp.c3n.size() * 16);
  const size_t o_c2s = off;
  off = up(off + mp.c2s.size() * 4);
  const size_t o_c2l = off;
  off = up(off + mp.c2l.size() * 4);
  const size_t o_esc = off;
  off = up(off + 8);
  const size_t nmv = trace ? (size_t)nw * (size_t)(p.steps - 1) : 0;
  const size_t o_tip = off;
  off = up(off + (size_t)(trace ? nw : 0) * 12);
  const size_t o_tpos = off;
  off = up(off + nmv * 12);
  const size_t o_thit = off;
  off = up(off + nmv * 4);
  const size_t o_twrd = off;
  off = up(off + nmv * 4);
  DevBuf arena;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e == cudaSuccess) e = cudaMalloc(&arena.p, off);
  if (e != cudaSuccess) {
    ctx->err = std::string("cudaMalloc(mesh arena): ") + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? AXX_ERR_OUT_OF_MEMORY : AXX_ERR_CUDA;
  }
  char *base = (char *)arena.p;
  e = upload_tables(base, L, g, kt, ctx->stream);
  auto put = [&](size_t o, const void *src, size_t n) {
    if (e == cudaSuccess && n)
      e = cudaMemcpyAsync(base + o, src, n, cudaMemcpyHostToDevice, ctx->stream);
  };
  put(o_tri, mp.tri.data(), mp.tri.size() * 16);
  put(o_c3s, mp.c3s.data(), mp.c3s.size() * 4);
  put(o_c3l, mp.c3l.data(), mp.c3l.size() * 4);
  put(o_c3n, mp.c3n.data(), mp.c3n.size() * 16);
  put(o_c2s, mp.c2s.data(), mp.c2s.size() * 4);
  put(o_c2l, mp.c2l.data(), mp.c2l.size() * 4);
  if (e == cudaSuccess) e = cudaMemsetAsync(base + o_esc, 0, 8, ctx->stream);
  WalkParams P;
  axx_run_params rp = p;
  rp.num_walkers = nw;
  InitSpec init;
  const double cell[3] = {1.0, 1.0, 1.0};
  fill_walk_params(P, base, L, g, kt, &rp, AXX_MODE_SINGLE, M, init, cell, ctx->abort_dev);
  P.kmax = kmax;
  MeshArgs Q{};
  Q.tri = (const float4 *)(base + o_tri);
  Q.c3s = (const uint32_t *)(base + o_c3s);
  Q.c3l = (const uint32_t *)(base + o_c3l);
  Q.c3n = (const float4 *)(base + o_c3n);
  Q.c2s = (const uint32_t *)(base + o_c2s);
  Q.c2l = (const uint32_t *)(base + o_c2l);
  for (int k = 0; k < 3; ++k) {
    Q.lo[k] = (float)mp.lo[k];
    Q.hi[k] = (float)mp.hi[k];
    Q.inv3[k] = mp.inv3[k];
    Q.g3[k] = mp.g3[k];
  }
  for (int k = 0; k < 2; ++k) {
    Q.inv2[k] = mp.inv2[k];
    Q.g2[k] = mp.g2[k];
  }
  double cmax = 0.0;  // largest coordinate magnitude: FP32 positions round to ulps of it
  for (int k = 0; k < 3; ++k) cmax = std::max(cmax, std::max(std::fabs(mp.lo[k]), std::fabs(mp.hi[k])));
  Q.slack = (float)(4e-6 * cmax);
  Q.escaped = (unsigned long long *)(base + o_esc);
  TraceParams T{};
  if (trace) {
    T.ntrace = (int)nw;
    T.init_pos = (float *)(base + o_tip);
    T.pos = (float *)(base + o_tpos);
    T.hits = (int32_t *)(base + o_thit);
    T.words = (int32_t *)(base + o_twrd);
  }
  *ctx->abort_host = 0;
  if (e == cudaSuccess) e = cudaMemsetAsync(P.counters, 0, AXX_CNT_N * 8, ctx->stream);
  if (e == cudaSuccess) e = launch_mesh(kmax, trace, P, Q, T, grid, smem, ctx->stream);
  double *d_out = (double *)(base + L.o_out);
  if (e == cudaSuccess && M > 0) e = launch_reduce_partials(P.partials, grid, M * 5, d_out, ctx->stream);
  std::vector<double> h((size_t)M * 5);
  unsigned long long cnt[AXX_CNT_N] = {0}, esc = 0;
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e == cudaSuccess && M > 0) e = cudaMemcpy(h.data(), d_out, h.size() * 8, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(cnt, P.counters, sizeof(cnt), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&esc, base + o_esc, 8, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && trace) {
    if (init_pos) e = cudaMemcpy(init_pos, T.init_pos, (size_t)nw * 12, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && pos) e = cudaMemcpy(pos, T.pos, nmv * 12, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && hits) e = cudaMemcpy(hits, T.hits, nmv * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && words) e = cudaMemcpy(words, T.words, nmv * 4, cudaMemcpyDeviceToHost);
  }
  if (e != cudaSuccess) {
    ctx->err = std::string("mesh walk: ") + cudaGetErrorString(e);
    return AXX_ERR_CUDA;
  }
  for (int m = 0; m < M; ++m) {
    if (mx) mx[m] = h[m * 5 + 0];
    if (my) my[m] = h[m * 5 + 1];
    if (stats) {
      if (stats->sxx) stats->sxx[m] = h[m * 5 + 2];
      if (stats->syy) stats->syy[m] = h[m * 5 + 3];
      if (stats->sxy) stats->sxy[m] = h[m * 5 + 4];
    }
  }
  if (stats) {
    stats->reflection_cap_hits = (int64_t)cnt[AXX_CNT_CAP];
    stats->walker_steps = nw * (int64_t)(p.steps - 1);
    stats->boundary_hits = (int64_t)cnt[AXX_CNT_HITS];
  }
  if (escaped) *escaped = (int64_t)esc;
  if (cnt[AXX_CNT_ABORTED]) return mesh_fail(ctx, AXX_ERR_ABORTED, "run aborted by axx_abort");
  if (cnt[AXX_CNT_INIT_FAIL])
    return mesh_fail(ctx, AXX_ERR_INVALID_ARG,
                     "no start point inside the mesh was found (is it closed?)");
  if (cnt[AXX_CNT_CAP])
    return mesh_fail(ctx, AXX_ERR_REFLECTION_CAP, "some moves hit the reflection cap of 1024");
  return AXX_OK;
}

}  // namespace
}  // namespace axx

extern "C" axx_status axx_run_mesh(axx_ctx *ctx, const axx_mesh *mesh, const axx_sequence *seqs,
                                   int nseq, const axx_run_params *params, double *mx, double *my,
                                   axx_stats *stats, int64_t *escaped) {
  return axx::mesh_run(ctx, mesh, seqs, nseq, params, mx, my, stats, escaped, 0, nullptr, nullptr,
                       nullptr, nullptr);
}

extern "C" axx_status axx_trace_mesh(axx_ctx *ctx, const axx_mesh *mesh,
                                     const axx_run_params *params, int ntrace, float *init_pos,
                                     float *pos, int32_t *hits, int32_t *words, int64_t *escaped) {
  if (!ctx) return AXX_ERR_INVALID_ARG;
  if (ntrace < 1) return axx::mesh_fail(ctx, AXX_ERR_INVALID_ARG, "ntrace must be >= 1");
  return axx::mesh_run(ctx, mesh, nullptr, 0, params, nullptr, nullptr, nullptr, escaped, ntrace,
                       init_pos, pos, hits, words);
}
