// mag.cu -- the magnetisation (Bloch) walk of a single pore on GB300.
//
// Reference: magAcquisitionStream<F>::runAcquisition
// (src/acquisition/magAcquisitionStream.cuh:37-90) launching
// updateWalkersMag (src/kernels/kernelMag.cuh:1-141) with B-field functors
// (src/functors/bfunctors.cuh) and the Bloch updates of
// src/bloch/blochdiff.cuh.  Each walker walks in one pore exactly as the
// single-pore phase walk does (start on a copy of the stream, two uniforms
// per move, boundaryNormal or simple rejection); after the start and after
// every move i each field functor j rotates that walker's magnetisation M_j
// about B_j(r, t).
//
// GB300 formulation:
//  * every field functor has the form B(r, t) = (bx(t), by(t), B0) +
//    s(t) A r with a fixed 3x3 matrix A (the gradient coils) and time-only
//    coefficients (s, bx, by) (lobes, ramps, RF pulses).  The host evaluates
//    the coefficients in FP64 with the reference's branch decisions at every
//    time point the walk uses (t = i dt; RK4's half steps; the multi-step
//    sub-steps) and stores them as FP32 tables, read uniformly by a warp;
//  * M_j (3 floats per field) stays in registers for the whole walk; the
//    rotation angle -gamma |B| h is split into -gamma |B0| h, whose sine and
//    cosine the host computes in FP64, and -gamma (|B| - |B0|) h, with
//    |B| - |B0| = (Bx^2 + By^2 + dBz (2 B0 + dBz)) / (|B| + |B0|) free of
//    cancellation: FP32 keeps the gradient's phase even when B0 dominates;
//  * after the walk a warp reduces each walker's M_j in FP64; blocks write
//    partials that reduce_partials_kernel sums in a fixed order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/axx.h"
#include "ctx_internal.h"
#include "host_plan.h"
#include "plan_layout.h"
#include "walk_kernel.cuh"
#include "walk_launch.h"

namespace axx {

constexpr int kMagMax = AXX_MAG_MAX_FIELDS;

struct MagArgs {
  int nf, integ;
  float gamma, h, gh;    // gamma, dt, -gamma dt
  float m0[3];
  float A[kMagMax][9];   // B = (bx, by, B0) + s A r, A row-major
  float B0[kMagMax];
  float c0[kMagMax], s0[kMagMax];  // cos, sin of -gamma |B0| dt
  const float4 *tab;     // [nf][steps] (s, bx, by, 0) at t = i dt
  const float4 *rk4;     // [nf][3] at t = 0, dt/2, dt (the RK4 start)
  const int2 *ms_idx;    // [nf][steps] (first sub-step, count)
  const float4 *ms_rot;  // [nf][steps] (cos, sin of -gamma |B0| hmin, -gamma hmin, 0)
  const float4 *ms_tab;  // sub-steps (s, bx, by, 0)
  double *partials;      // [grid][nf*3]
  float *m_trace;        // [ntrace][nf][3]
  // Dormand-Prince: per field, step, level k (sub-steps dt/2^k) and sub-step
  // m, the six stage times' coefficients (s, bx, by, 0)
  const float4 *dp_tab;  // [nf][steps][6 (2^(K+1) - 1)]
  int dp_K;              // halvings allowed
  float dp_tol;
};

__device__ __forceinline__ void field_at(const MagArgs &Q, int j, const float4 &tc, float x,
                                         float y, float z, float &bx, float &by, float &dbz) {
  const float *A = Q.A[j];
  const float ax = fma_f(A[0], x, fma_f(A[1], y, A[2] * z));
  const float ay = fma_f(A[3], x, fma_f(A[4], y, A[5] * z));
  const float az = fma_f(A[6], x, fma_f(A[7], y, A[8] * z));
  bx = fma_f(tc.x, ax, tc.y);
  by = fma_f(tc.x, ay, tc.z);
  dbz = tc.x * az;
}

// M rotated about B = (bx, by, B0 + dbz) by -gamma |B| h, with (c0, s0) the
// cosine and sine of -gamma |B0| h and gh = -gamma h (updateMag_noT2_rotate,
// blochdiff.cuh:161-172).  |B| = 0 leaves M unchanged.
__device__ __forceinline__ void rotate(float &mx, float &my, float &mz, float bx, float by,
                                       float dbz, float B0, float c0, float s0, float gh) {
  const float bz = B0 + dbz;
  const float bxy = fma_f(bx, bx, by * by);
  const float b2 = fma_f(bz, bz, bxy);
  if (!(b2 > 0.0f)) return;
  const float bm = sqrt_f(b2);
  const float excess = __fdividef(fma_f(dbz, fma_f(2.0f, B0, dbz), bxy), bm + fabsf(B0));
  float sd, cd;
  sincos_2pi(gh * excess * 0.15915494309189535f, sd, cd);
  const float ct = fma_f(c0, cd, -(s0 * sd)), st = fma_f(s0, cd, c0 * sd);
  const float inv = __fdividef(1.0f, bm);
  const float ux_ = bx * inv, uy_ = by * inv, uz_ = bz * inv;
  const float md = fma_f(mx, ux_, fma_f(my, uy_, mz * uz_));
  const float cx = ux_ * md, cy = uy_ * md, cz = uz_ * md;
  const float vx = mx - cx, vy = my - cy, vz = mz - cz;
  const float wx = fma_f(uy_, vz, -(uz_ * vy)), wy = fma_f(uz_, vx, -(ux_ * vz)),
              wz = fma_f(ux_, vy, -(uy_ * vx));
  mx = fma_f(wx, st, fma_f(vx, ct, cx));
  my = fma_f(wy, st, fma_f(vy, ct, cy));
  mz = fma_f(wz, st, fma_f(vz, ct, cz));
}

// updateMagRK4 without relaxation (blochdiff.cuh:29-44) for the t = 0 update:
// k = gamma h (M x B) at t = 0, dt/2, dt/2, dt.
__device__ __forceinline__ void rk4_start(const MagArgs &Q, int j, float x, float y, float z,
                                          float &mx, float &my, float &mz) {
  float B[3][3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float bx, by, dbz;
    field_at(Q, j, Q.rk4[j * 3 + k], x, y, z, bx, by, dbz);
    B[k][0] = bx;
    B[k][1] = by;
    B[k][2] = Q.B0[j] + dbz;
  }
  const float gh = Q.gamma * Q.h;
  auto bl = [&](const float *b, float px, float py, float pz, float &kx, float &ky, float &kz) {
    kx = gh * fma_f(py, b[2], -(pz * b[1]));
    ky = gh * fma_f(pz, b[0], -(px * b[2]));
    kz = gh * fma_f(px, b[1], -(py * b[0]));
  };
  float k1x, k1y, k1z, k2x, k2y, k2z, k3x, k3y, k3z, k4x, k4y, k4z;
  bl(B[0], mx, my, mz, k1x, k1y, k1z);
  bl(B[1], fma_f(0.5f, k1x, mx), fma_f(0.5f, k1y, my), fma_f(0.5f, k1z, mz), k2x, k2y, k2z);
  bl(B[1], fma_f(0.5f, k2x, mx), fma_f(0.5f, k2y, my), fma_f(0.5f, k2z, mz), k3x, k3y, k3z);
  bl(B[2], mx + k3x, my + k3y, mz + k3z, k4x, k4y, k4z);
  const float s6 = 1.0f / 6.0f;
  mx += s6 * fma_f(2.0f, k2x + k3x, k1x + k4x);
  my += s6 * fma_f(2.0f, k2y + k3y, k1y + k4y);
  mz += s6 * fma_f(2.0f, k2z + k3z, k1z + k4z);
}

// gamma (M x B(r, t)) with the field coefficients tc of the stage time
// (blochdiff.cuh:7-10: bloch() = (M % B) GAMMA).
__device__ __forceinline__ void bloch_deriv(const MagArgs &Q, int j, const float4 &tc, float x,
                                            float y, float z, const float m[3], float f[3]) {
  float bx, by, dbz;
  field_at(Q, j, tc, x, y, z, bx, by, dbz);
  const float bz = Q.B0[j] + dbz;
  f[0] = Q.gamma * fma_f(m[1], bz, -(m[2] * by));
  f[1] = Q.gamma * fma_f(m[2], bx, -(m[0] * bz));
  f[2] = Q.gamma * fma_f(m[0], by, -(m[1] * bx));
}

// Adaptive Dormand-Prince 5(4) over [i dt, (i+1) dt] at the walker's
// position, the FP32 twin of the oracle's mag_dorp: tableau of Dormand &
// Prince (1980), the fifth-order solution propagated, the embedded
// fourth-order error scaled per component by tol (1 + max(|M5|, |M|)) and
// taken as an RMS; sub-steps dt/2^k on a dyadic grid, halved while the error
// exceeds 1 (accepted at level K whatever it is), doubled after an error
// below 1/32 when the grid allows.  Every loop is bounded.
__device__ __noinline__ float3 dorp_update(const MagArgs &Q, int steps, int j, int i, float x,
                                           float y, float z, float mx, float my, float mz) {
  constexpr float a10 = (float)(1.0 / 5.0);
  constexpr float a20 = (float)(3.0 / 40.0), a21 = (float)(9.0 / 40.0);
  constexpr float a30 = (float)(44.0 / 45.0), a31 = (float)(-56.0 / 15.0),
                  a32 = (float)(32.0 / 9.0);
  constexpr float a40 = (float)(19372.0 / 6561.0), a41 = (float)(-25360.0 / 2187.0),
                  a42 = (float)(64448.0 / 6561.0), a43 = (float)(-212.0 / 729.0);
  constexpr float a50 = (float)(9017.0 / 3168.0), a51 = (float)(-355.0 / 33.0),
                  a52 = (float)(46732.0 / 5247.0), a53 = (float)(49.0 / 176.0),
                  a54 = (float)(-5103.0 / 18656.0);
  constexpr float b0 = (float)(35.0 / 384.0), b2 = (float)(500.0 / 1113.0),
                  b3 = (float)(125.0 / 192.0), b4 = (float)(-2187.0 / 6784.0),
                  b5 = (float)(11.0 / 84.0);
  constexpr float e0 = (float)(71.0 / 57600.0), e2 = (float)(-71.0 / 16695.0),
                  e3 = (float)(71.0 / 1920.0), e4 = (float)(-17253.0 / 339200.0),
                  e5 = (float)(22.0 / 525.0), e6 = (float)(-1.0 / 40.0);
  const int K = Q.dp_K, full = 1 << K;
  const float4 *T = Q.dp_tab + ((size_t)j * steps + i) * (size_t)(6 * ((2 << K) - 1));
  float M[3] = {mx, my, mz};
  int pos = 0, k = 0;
  for (int guard = 0; pos < full && guard < 64 * full; ++guard) {
    const float h = Q.h * __int_as_float((127 - k) << 23);  // dt / 2^k, exact
    const float4 *tc = T + 6 * ((1 << k) - 1 + (pos >> (K - k)));
    float f0[3], f1[3], f2[3], f3[3], f4[3], f5[3], f6[3], yv[3], y5[3];
    bloch_deriv(Q, j, tc[0], x, y, z, M, f0);
#pragma unroll
    for (int c = 0; c < 3; ++c) yv[c] = fma_f(h, a10 * f0[c], M[c]);
    bloch_deriv(Q, j, tc[1], x, y, z, yv, f1);
#pragma unroll
    for (int c = 0; c < 3; ++c) yv[c] = fma_f(h, fma_f(a21, f1[c], a20 * f0[c]), M[c]);
    bloch_deriv(Q, j, tc[2], x, y, z, yv, f2);
#pragma unroll
    for (int c = 0; c < 3; ++c)
      yv[c] = fma_f(h, fma_f(a32, f2[c], fma_f(a31, f1[c], a30 * f0[c])), M[c]);
    bloch_deriv(Q, j, tc[3], x, y, z, yv, f3);
#pragma unroll
    for (int c = 0; c < 3; ++c)
      yv[c] = fma_f(h, fma_f(a43, f3[c], fma_f(a42, f2[c], fma_f(a41, f1[c], a40 * f0[c]))), M[c]);
    bloch_deriv(Q, j, tc[4], x, y, z, yv, f4);
#pragma unroll
    for (int c = 0; c < 3; ++c)
      yv[c] = fma_f(h, fma_f(a54, f4[c], fma_f(a53, f3[c], fma_f(a52, f2[c],
                                                                   fma_f(a51, f1[c], a50 * f0[c])))),
                    M[c]);
    bloch_deriv(Q, j, tc[5], x, y, z, yv, f5);
#pragma unroll
    for (int c = 0; c < 3; ++c)
      y5[c] = fma_f(h, fma_f(b5, f5[c], fma_f(b4, f4[c], fma_f(b3, f3[c], fma_f(b2, f2[c], b0 * f0[c])))),
                    M[c]);
    bloch_deriv(Q, j, tc[5], x, y, z, y5, f6);
    float en = 0.0f;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float err =
          h * fma_f(e6, f6[c], fma_f(e5, f5[c], fma_f(e4, f4[c], fma_f(e3, f3[c],
                                                                    fma_f(e2, f2[c], e0 * f0[c])))));
      const float r = __fdividef(err, Q.dp_tol * (1.0f + fmaxf(fabsf(y5[c]), fabsf(M[c]))));
      en = fma_f(r, r, en);
    }
    en = sqrt_f(en * (1.0f / 3.0f));
    if (en <= 1.0f || k == K) {
      M[0] = y5[0];
      M[1] = y5[1];
      M[2] = y5[2];
      pos += 1 << (K - k);
      if (en < (1.0f / 32.0f) && k > 0 && (pos & ((1 << (K - k + 1)) - 1)) == 0) --k;
    } else {
      ++k;
    }
  }
  return make_float3(M[0], M[1], M[2]);
}

// The update of field j at time point i (kernelMag.cuh:32-72 for i = 0,
// :96-134 for i >= 1).
__device__ __forceinline__ void mag_update(const MagArgs &Q, int steps, int j, int i, float x,
                                           float y, float z, float &mx, float &my, float &mz) {
  if (Q.integ == AXX_MAG_DORP) {
    // (by value: a reference into the walker's M array would move it to
    // local memory in every instantiation)
    const float3 r = dorp_update(Q, steps, j, i, x, y, z, mx, my, mz);
    mx = r.x;
    my = r.y;
    mz = r.z;
    return;
  }
  if (Q.integ == AXX_MAG_ROTATE_MULTISTEP) {
    const int2 ix = Q.ms_idx[j * steps + i];
    const float4 rt = Q.ms_rot[j * steps + i];
    for (int k = 0; k < ix.y; ++k) {
      float bx, by, dbz;
      field_at(Q, j, Q.ms_tab[ix.x + k], x, y, z, bx, by, dbz);
      rotate(mx, my, mz, bx, by, dbz, Q.B0[j], rt.x, rt.y, rt.z);
    }
    return;
  }
  if (Q.integ == AXX_MAG_RK4 && i == 0) {
    rk4_start(Q, j, x, y, z, mx, my, mz);
    return;
  }
  float bx, by, dbz;
  field_at(Q, j, Q.tab[j * steps + i], x, y, z, bx, by, dbz);
  rotate(mx, my, mz, bx, by, dbz, Q.B0[j], Q.c0[j], Q.s0[j], Q.gh);
}

template <int MMAX>
__device__ __forceinline__ void mag_update_all(const MagArgs &Q, int steps, int i, float x, float y,
                                               float z, float *m) {
#pragma unroll
  for (int j = 0; j < MMAX; ++j)
    if (j < Q.nf) mag_update(Q, steps, j, i, x, y, z, m[3 * j], m[3 * j + 1], m[3 * j + 2]);
}

template <int GEOM, int KM, int MMAX, bool TRACE>
__global__ void __launch_bounds__(AXX_BLOCK)
    mag_kernel(const __grid_constant__ WalkParams P, const __grid_constant__ MagArgs Q,
               const __grid_constant__ TraceParams T) {
  constexpr int warps = AXX_BLOCK / 32;
  constexpr bool reject = KM == AXX_KM_SINGLE_REJ;
  __shared__ double wsum[warps][3 * MMAX];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  for (int k = lane; k < 3 * MMAX; k += 32) wsum[wib][k] = 0.0;
  SmemView S;
  S.geo = P.inst_geo;
  S.aux = P.inst_aux;
  S.slot = P.slot_tab;
  S.cstart = P.cell_start;
  S.region = P.slot_region;
  S.clist = P.cell_list;
  const float4 g0 = P.inst_geo[0], a0 = P.inst_aux[0];
  const bool sph = is_sphere<GEOM>(a0);
  const float4 s4 = P.slot_tab[0];
  const float v = s4.x, L = s4.y;
  const Cands<GEOM, true> C{S, g0, a0, 0u, 0u};
  const long long ntask = (P.n_walkers + 31) / 32;
  const long long gwarp = (long long)blockIdx.x * warps + wib;
  const long long nwarp = (long long)gridDim.x * warps;
  unsigned caps = 0, hits = 0, init_fail = 0, aborted = 0;
  for (long long task = gwarp; task < ntask; task += nwarp) {
    const long long wid = task * 32 + lane;
    const bool active = wid < P.n_walkers;
    float m[3 * MMAX];
#pragma unroll
    for (int j = 0; j < MMAX; ++j) {
      m[3 * j] = Q.m0[0];
      m[3 * j + 1] = Q.m0[1];
      m[3 * j + 2] = Q.m0[2];
    }
    if (active) {
      DevStream st;
      st.init(P, (uint64_t)(wid + P.walker_offset), 1u);
      float x = 0.f, y = 0.f, z = 0.f;
      bool ok;
      if (P.init_quirk) {
        DevStream cp = st;  // Basis::unifRand takes the curandState by value
        ok = init_position<GEOM, KM>(P, S, cp, x, y, z);
      } else {
        ok = init_position<GEOM, KM>(P, S, st, x, y, z);
      }
      init_fail += ok ? 0u : 1u;
      if (TRACE && wid < T.ntrace) {
        T.init_pos[wid * 3 + 0] = x;
        T.init_pos[wid * 3 + 1] = y;
        T.init_pos[wid * 3 + 2] = z;
      }
      mag_update_all<MMAX>(Q, P.steps, 0, x, y, z, m);
      for (int i = 1; i < P.steps; ++i) {
        if ((i & 1023) == 0 && P.abort_flag != nullptr && *P.abort_flag) {
          aborted += 1u;
          break;
        }
        float u1, u2, dx, dy, dz;
        st.next2(P, u1, u2);
        direction(u1, u2, dx, dy, dz);
        int h = 0;
        if (reject) {
          const float ex = fma_f(L, dx, x), ey = fma_f(L, dy, y), ez = fma_f(L, dz, z);
          if (c0_of(g0, sph, ex, ey, ez) < 0.0f) {
            x = ex;
            y = ey;
            z = ez;
          }
        } else {
          const MoveOut o = boundary<GEOM, false, true>(P, C, x, y, z, dx, dy, dz, L, v, st, L);
          x = o.fx;
          y = o.fy;
          z = o.fz;
          h = o.hits;
          caps += o.capped ? 1u : 0u;
        }
        hits += (unsigned)h;
        if (TRACE && wid < T.ntrace) {
          const long long o = wid * (long long)(P.steps - 1) + (i - 1);
          T.pos[o * 3 + 0] = x;
          T.pos[o * 3 + 1] = y;
          T.pos[o * 3 + 2] = z;
          T.hits[o] = h;
          T.words[o] = (int32_t)st.words_used();
        }
        mag_update_all<MMAX>(Q, P.steps, i, x, y, z, m);
      }
      if (TRACE && wid < T.ntrace) {
#pragma unroll
        for (int k = 0; k < 3 * MMAX; ++k)
          if (k < 3 * Q.nf) Q.m_trace[wid * 3 * Q.nf + k] = m[k];
      }
    }
    // FP64 reduction of the final magnetisation (magAcquisitionStream's sums)
#pragma unroll
    for (int k = 0; k < 3 * MMAX; ++k) {
      if (k < 3 * Q.nf) {
        const double s = warp_sum(active ? (double)m[k] : 0.0);
        if (lane == 0) wsum[wib][k] += s;
      }
    }
  }
  if (caps) atomicAdd(&P.counters[AXX_CNT_CAP], (unsigned long long)caps);
  if (hits) atomicAdd(&P.counters[AXX_CNT_HITS], (unsigned long long)hits);
  if (init_fail) atomicAdd(&P.counters[AXX_CNT_INIT_FAIL], (unsigned long long)init_fail);
  if (aborted) atomicAdd(&P.counters[AXX_CNT_ABORTED], (unsigned long long)aborted);
  __syncthreads();
  for (int k = threadIdx.x; k < 3 * Q.nf; k += blockDim.x) {
    double s = 0.0;
    for (int w = 0; w < warps; ++w) s += wsum[w][k];
    Q.partials[(size_t)blockIdx.x * 3 * Q.nf + k] = s;
  }
}

// ------------------------------------------------------------------ host ---
namespace {

axx_status mfail2(axx_ctx *ctx, axx_status s, const std::string &m) {
  if (ctx) ctx->err = m;
  return s;
}
axx_status mcuda2(axx_ctx *ctx, cudaError_t e, const char *where) {
  if (ctx) ctx->err = std::string(where) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? AXX_ERR_OUT_OF_MEMORY : AXX_ERR_CUDA;
}

const double kPiD = 3.1415926535897932384626433832795;

// Time-only coefficients (s, bx, by) of a functor at time t, with the
// reference's expressions and branch order (bfunctors.cuh).
void time_coef(const axx_field &f, double gamma, double time, double c[3]) {
  const double gd = f.duration, gs = f.spacing, G = f.G, B0 = f.B0;
  c[0] = c[1] = c[2] = 0.0;
  const bool lobe1 = time < gd;
  const bool lobe2 = !lobe1 && time >= gs + gd && time < 2.0 * gd + gs;
  switch (f.kind) {
    case AXX_FIELD_QSC_GRE:  // :29-50
      c[0] = lobe1 ? 1.0 : (lobe2 ? -1.0 : 0.0);
      break;
    case AXX_FIELD_QSC_PGSE: {  // :90-118
      const double B1 = kPiD / std::fabs(gamma * f.rf_duration);
      if (lobe1) {
        c[0] = 1.0;
      } else if (time >= f.TE / 2.0 && time < f.TE / 2.0 + f.rf_duration) {
        const double w = gamma * B0;
        c[1] = B1 * std::cos(w * time);
        c[2] = -B1 * std::sin(w * time);
      } else if (time >= gs + gd && time < 2.0 * gd + gs) {
        c[0] = 1.0;
      }
      break;
    }
    case AXX_FIELD_QSC_COS_GRE: {  // :160-191
      const double period = gd / (double)f.num_periods;
      if (lobe1) c[0] = std::cos(2.0 * kPiD * time / period);
      else if (lobe2) c[0] = -std::cos(2.0 * kPiD * (time - gs - gd) / period);
      break;
    }
    case AXX_FIELD_QSC_GRE_TRAP: {  // :224-271 (ramps multiply G r by (G/ramp) t)
      const double r = f.ramp, t1 = r, t2 = r + gd, t3 = 2.0 * t1 + t2, t5 = gs + t3;
      auto m1 = [&](double t) { return (G / r) * t; };
      auto m2 = [&](double t) { return G - (G / r) * t; };
      if (time < t1) c[0] = m1(time);
      else if (time >= t1 && time < t2) c[0] = 1.0;
      else if (time >= t2 && time < t3) c[0] = m2(time - t2);
      else if (time >= t5 && time < t5 + t1) c[0] = m1(time - t5);
      else if (time >= t5 + t1 && time < t5 + t2) c[0] = 1.0;
      else if (time >= t5 + t2 && time < t5 + t3) c[0] = m2(time - t5 - t2);
      break;
    }
    case AXX_FIELD_SIN_GRE:  // :310-328
    case AXX_FIELD_COS_GRE: {  // :376-392
      const double period = f.kind == AXX_FIELD_SIN_GRE ? f.period : gd / (double)f.num_periods;
      auto amp = [&](double t) {
        const double a = 2.0 * kPiD * t / period;
        return f.kind == AXX_FIELD_SIN_GRE ? std::sin(a) : std::cos(a);
      };
      if (lobe1) c[0] = amp(time);
      else if (lobe2) c[0] = -amp(time - gs - gd);
      break;
    }
    case AXX_FIELD_RECT_GRE:  // :417-425
      c[0] = lobe1 ? 1.0 : (lobe2 ? -1.0 : 0.0);
      break;
    default: {  // UCN_lowfield :457-466
      c[0] = 1.0;
      if (time < f.rf_duration) {
        const double B1 = kPiD / (2.0 * std::fabs(gamma * f.rf_duration));
        const double w = gamma * B0;
        c[1] = B1 * std::cos(w * time);
        c[2] = -B1 * std::sin(w * time);
      }
      break;
    }
  }
}

// The fixed matrix A of B = (bx, by, B0) + s A r.
void field_matrix(const axx_field &f, float A[9]) {
  for (int k = 0; k < 9; ++k) A[k] = 0.f;
  switch (f.kind) {
    case AXX_FIELD_QSC_GRE:
    case AXX_FIELD_QSC_PGSE:
    case AXX_FIELD_QSC_COS_GRE:
    case AXX_FIELD_QSC_GRE_TRAP:  // (0, G z, B0 + G y)
      A[5] = (float)f.G;
      A[7] = (float)f.G;
      break;
    case AXX_FIELD_SIN_GRE:
    case AXX_FIELD_COS_GRE:
    case AXX_FIELD_RECT_GRE:  // (0, 0, B0 + g . r)
      A[6] = (float)f.gx;
      A[7] = (float)f.gy;
      A[8] = (float)f.gz;
      break;
    default:  // UCN: (-G x / 2, -G y / 2, B0 + G z)
      A[0] = (float)(-0.5 * f.G);
      A[4] = (float)(-0.5 * f.G);
      A[8] = (float)f.G;
      break;
  }
}

// getStepTimeMin (QSC_PGSE :121-127, UCN_lowfield :469-475)
double step_time_min(const axx_field &f, double t) {
  if (f.kind == AXX_FIELD_QSC_PGSE)
    return (t >= f.TE / 2.0 && t < f.TE / 2.0 + f.rf_duration) ? f.dtmin : f.dtmax;
  return (t <= f.rf_duration) ? f.dtmin : f.dtmax;
}

float4 f4(const double c[3]) { return make_float4((float)c[0], (float)c[1], (float)c[2], 0.f); }

template <int GEOM, int KM, int MMAX, bool TRACE>
cudaError_t launch_mag_t(const WalkParams &P, const MagArgs &Q, const TraceParams &T, int grid,
                         cudaStream_t s) {
  mag_kernel<GEOM, KM, MMAX, TRACE><<<grid, AXX_BLOCK, 0, s>>>(P, Q, T);
  return cudaGetLastError();
}

template <int GEOM, int KM, int MMAX>
int occ_mag_t() {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, mag_kernel<GEOM, KM, MMAX, false>,
                                                    AXX_BLOCK, 0) != cudaSuccess)
    return 0;
  return n;
}

template <int GEOM, int KM>
cudaError_t launch_mag_g(int mmax, bool trace, const WalkParams &P, const MagArgs &Q,
                         const TraceParams &T, int grid, cudaStream_t s) {
  if (mmax <= 4)
    return trace ? launch_mag_t<GEOM, KM, 4, true>(P, Q, T, grid, s)
                 : launch_mag_t<GEOM, KM, 4, false>(P, Q, T, grid, s);
  return trace ? launch_mag_t<GEOM, KM, kMagMax, true>(P, Q, T, grid, s)
               : launch_mag_t<GEOM, KM, kMagMax, false>(P, Q, T, grid, s);
}

cudaError_t launch_mag(int geom, int km, int mmax, bool trace, const WalkParams &P,
                       const MagArgs &Q, const TraceParams &T, int grid, cudaStream_t s) {
  if (geom == AXX_GEOM_SPH)
    return km == AXX_KM_SINGLE_REJ ? launch_mag_g<AXX_GEOM_SPH, AXX_KM_SINGLE_REJ>(mmax, trace, P, Q, T, grid, s)
                                   : launch_mag_g<AXX_GEOM_SPH, AXX_KM_SINGLE>(mmax, trace, P, Q, T, grid, s);
  return km == AXX_KM_SINGLE_REJ ? launch_mag_g<AXX_GEOM_CYL, AXX_KM_SINGLE_REJ>(mmax, trace, P, Q, T, grid, s)
                                 : launch_mag_g<AXX_GEOM_CYL, AXX_KM_SINGLE>(mmax, trace, P, Q, T, grid, s);
}

int occupancy_mag(int geom, int km, int mmax) {
  const bool big = mmax > 4;
  if (geom == AXX_GEOM_SPH) {
    if (km == AXX_KM_SINGLE_REJ)
      return big ? occ_mag_t<AXX_GEOM_SPH, AXX_KM_SINGLE_REJ, kMagMax>() : occ_mag_t<AXX_GEOM_SPH, AXX_KM_SINGLE_REJ, 4>();
    return big ? occ_mag_t<AXX_GEOM_SPH, AXX_KM_SINGLE, kMagMax>() : occ_mag_t<AXX_GEOM_SPH, AXX_KM_SINGLE, 4>();
  }
  if (km == AXX_KM_SINGLE_REJ)
    return big ? occ_mag_t<AXX_GEOM_CYL, AXX_KM_SINGLE_REJ, kMagMax>() : occ_mag_t<AXX_GEOM_CYL, AXX_KM_SINGLE_REJ, 4>();
  return big ? occ_mag_t<AXX_GEOM_CYL, AXX_KM_SINGLE, kMagMax>() : occ_mag_t<AXX_GEOM_CYL, AXX_KM_SINGLE, 4>();
}

struct DevBuf {
  void *p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

axx_status mag_run(axx_ctx *ctx, const axx_basis *pore, const axx_field *fields, int nf,
                   const axx_mag_params *mp, int ntrace, float *init_pos, float *pos,
                   int32_t *hits_out, int32_t *words_out, float *m_final, double *mx, double *my,
                   double *mz) {
  if (!ctx) return AXX_ERR_INVALID_ARG;
  if (!pore || !fields || !mp) return mfail2(ctx, AXX_ERR_INVALID_ARG, "NULL argument");
  if (nf < 1 || nf > kMagMax)
    return mfail2(ctx, AXX_ERR_INVALID_ARG, "nfield must be 1..16");
  if (mp->num_walkers < 1 || mp->steps < 1 || !(mp->timestep > 0.0) ||
      !std::isfinite(mp->timestep) || mp->walker_offset < 0)
    return mfail2(ctx, AXX_ERR_INVALID_ARG, "num_walkers, steps, timestep or walker_offset out of range");
  if (mp->integrator < 0 || mp->integrator > 3)
    return mfail2(ctx, AXX_ERR_INVALID_ARG, "unknown integrator");
  const int dp_K = mp->dorp_levels ? (int)mp->dorp_levels : 3;
  const double dp_tol = mp->dorp_tol > 0.0 ? mp->dorp_tol : 1e-6;
  if (mp->integrator == AXX_MAG_DORP &&
      (mp->dorp_levels > 8 || !(mp->dorp_tol >= 0.0) || !std::isfinite(mp->dorp_tol)))
    return mfail2(ctx, AXX_ERR_INVALID_ARG, "dorp_levels must be 0..8 and dorp_tol >= 0");
  // negative ratios are physical here (helium-3: the reference's magLF
  // examples use GAMMA = -203789): they reverse the precession
  if (!std::isfinite(mp->gamma))
    return mfail2(ctx, AXX_ERR_INVALID_ARG, "gamma must be finite");
  if (mp->flags & ~(uint32_t)(AXX_FLAG_SIMPLE_REJECTION | AXX_FLAG_FIX_INIT_QUIRK))
    return mfail2(ctx, AXX_ERR_INVALID_ARG, "the magnetisation walk takes only the rejection and init-quirk flags");
  const double gamma = mp->gamma != 0.0 ? mp->gamma : kGammaDefault;
  const double dt = mp->timestep;
  const int steps = mp->steps;
  for (int j = 0; j < nf; ++j) {
    const axx_field &f = fields[j];
    if (f.kind < 0 || f.kind > 7) return mfail2(ctx, AXX_ERR_INVALID_ARG, "unknown field kind");
    if ((f.kind == AXX_FIELD_QSC_COS_GRE || f.kind == AXX_FIELD_COS_GRE) && f.num_periods < 1)
      return mfail2(ctx, AXX_ERR_INVALID_ARG, "num_periods must be >= 1");
    if (mp->integrator == AXX_MAG_ROTATE_MULTISTEP) {
      if (f.kind != AXX_FIELD_QSC_PGSE && f.kind != AXX_FIELD_UCN_LOWFIELD)
        return mfail2(ctx, AXX_ERR_UNSUPPORTED,
                      "multi-step rotation needs getStepTimeMin (QSC_PGSE, UCN_lowfield)");
      if (!(f.dtmin > 0.0) || !(f.dtmax > 0.0))
        return mfail2(ctx, AXX_ERR_INVALID_ARG, "dtmin and dtmax must be > 0");
    }
  }
  GeomPlan g;
  float sp = 0.f, stp = 0.f;
  std::string err = plan_single(pore, dt, g, sp, stp);
  if (!err.empty()) return mfail2(ctx, AXX_ERR_INVALID_ARG, err);
  axx_run_params rp{mp->num_walkers, steps, 0, 0, mp->flags, mp->seed, dt, gamma, mp->walker_offset};
  KernelTables kt;
  err = make_kernel_tables(g, SeqPlan(), 0, steps, AXX_MODE_SINGLE, rp.flags, kt);
  if (!err.empty()) return mfail2(ctx, AXX_ERR_UNSUPPORTED, err);
  InitSpec init;
  err = init_spec(g, pore, 1, AXX_MODE_SINGLE, &rp, init);
  if (!err.empty()) return mfail2(ctx, AXX_ERR_INVALID_ARG, err);

  // time tables (FP64 -> FP32)
  MagArgs Q{};
  Q.nf = nf;
  Q.integ = mp->integrator;
  Q.gamma = (float)gamma;
  Q.h = (float)dt;
  Q.gh = (float)(-gamma * dt);
  for (int k = 0; k < 3; ++k) Q.m0[k] = (float)mp->m0[k];
  std::vector<float4> tab, rk4, ms_rot, ms_tab, dp_tab;
  std::vector<int2> ms_idx;
  if (mp->integrator == AXX_MAG_DORP) {
    const size_t per = (size_t)6 * (size_t)((2 << dp_K) - 1);
    if ((size_t)nf * (size_t)steps * per > ((size_t)1 << 27))
      return mfail2(ctx, AXX_ERR_UNSUPPORTED,
                    "Dormand-Prince tables above 2^27 entries: fewer steps or levels");
    dp_tab.reserve((size_t)nf * (size_t)steps * per);
  }
  for (int j = 0; j < nf; ++j) {
    const axx_field &f = fields[j];
    field_matrix(f, Q.A[j]);
    Q.B0[j] = (float)f.B0;
    const double a0 = -gamma * std::fabs(f.B0) * dt;
    Q.c0[j] = (float)std::cos(a0);
    Q.s0[j] = (float)std::sin(a0);
    double c[3];
    if (mp->integrator == AXX_MAG_DORP) {
      // stage times i dt + (m + c_s) dt / 2^k of every level and sub-step
      static const double cs[6] = {0.0, 1.0 / 5.0, 3.0 / 10.0, 4.0 / 5.0, 8.0 / 9.0, 1.0};
      for (int i = 0; i < steps; ++i)
        for (int k = 0; k <= dp_K; ++k) {
          const double h = dt / (double)(1 << k);
          for (int m = 0; m < (1 << k); ++m)
            for (int q = 0; q < 6; ++q) {
              time_coef(f, gamma, i * dt + ((double)m + cs[q]) * h, c);
              dp_tab.push_back(f4(c));
            }
        }
    } else if (mp->integrator == AXX_MAG_ROTATE_MULTISTEP) {
      for (int i = 0; i < steps; ++i) {
        // updateMag_rotate_noT2_multistep (blochdiff.cuh:118-140)
        double acc = 0.0, tk = i * dt;
        const double hmin = step_time_min(f, tk);
        const int first = (int)ms_tab.size();
        do {
          time_coef(f, gamma, tk, c);
          ms_tab.push_back(f4(c));
          acc += hmin;
          tk += hmin;
          if (ms_tab.size() > (size_t)1 << 27)
            return mfail2(ctx, AXX_ERR_UNSUPPORTED, "more than 2^27 multi-step sub-steps");
        } while (acc < dt);
        ms_idx.push_back(make_int2(first, (int)ms_tab.size() - first));
        const double ah = -gamma * std::fabs(f.B0) * hmin;
        ms_rot.push_back(make_float4((float)std::cos(ah), (float)std::sin(ah), (float)(-gamma * hmin), 0.f));
      }
    } else {
      for (int i = 0; i < steps; ++i) {
        time_coef(f, gamma, i * dt, c);
        tab.push_back(f4(c));
      }
      const double tn = 0.0 * dt, h = dt;  // updateMagRK4 at i = 0
      const double ts[3] = {tn, tn + .5 * h, tn + h};
      for (double t : ts) {
        time_coef(f, gamma, t, c);
        rk4.push_back(f4(c));
      }
    }
  }
  const int mmax = nf <= 4 ? 4 : kMagMax;
  const int occ = occupancy_mag(g.geom, kt.km, mmax);
  if (occ <= 0) return mfail2(ctx, AXX_ERR_CUDA, "magnetisation kernel cannot be resident");
  const long long ntask = (mp->num_walkers + 31) / 32;
  const long long want = (ntask + AXX_BLOCK / 32 - 1) / (AXX_BLOCK / 32);
  const int grid = (int)std::max<long long>(1, std::min<long long>(want, (long long)occ * ctx->nsm));

  // one arena: walk tables | field tables | partials | sums
  const ArenaLayout L = arena_layout(g, kt, 0);
  auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
  size_t off = up(L.fixed);
  const size_t o_tab = off;
  off = up(off + tab.size() * 16);
  const size_t o_rk4 = off;
  off = up(off + rk4.size() * 16);
  const size_t o_msi = off;
  off = up(off + ms_idx.size() * 8);
  const size_t o_msr = off;
  off = up(off + ms_rot.size() * 16);
  const size_t o_mst = off;
  off = up(off + ms_tab.size() * 16);
  const size_t o_dp = off;
  off = up(off + dp_tab.size() * 16);
  const size_t o_part = off;
  off = up(off + (size_t)grid * nf * 3 * 8);
  const size_t o_out = off;
  off = up(off + (size_t)nf * 3 * 8);
  const size_t o_mtr = off;
  const int nt = std::max(0, std::min<int>(ntrace, (int)std::min<long long>(mp->num_walkers, 1 << 20)));
  off = up(off + (size_t)nt * nf * 3 * 4);
  const size_t o_tip = off;
  off = up(off + (size_t)nt * 3 * 4);
  const size_t nmv = (size_t)nt * (size_t)(steps - 1);
  const size_t o_tpos = off;
  off = up(off + nmv * 3 * 4);
  const size_t o_thit = off;
  off = up(off + nmv * 4);
  const size_t o_twrd = off;
  off = up(off + nmv * 4);
  DevBuf arena;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e == cudaSuccess) e = cudaMalloc(&arena.p, off);
  if (e != cudaSuccess) return mcuda2(ctx, e, "cudaMalloc(magnetisation arena)");
  char *base = (char *)arena.p;
  e = upload_tables(base, L, g, kt, ctx->stream);
  auto put = [&](size_t o, const void *src, size_t n) {
    if (e == cudaSuccess && n) e = cudaMemcpyAsync(base + o, src, n, cudaMemcpyHostToDevice, ctx->stream);
  };
  put(o_tab, tab.data(), tab.size() * 16);
  put(o_rk4, rk4.data(), rk4.size() * 16);
  put(o_msi, ms_idx.data(), ms_idx.size() * 8);
  put(o_msr, ms_rot.data(), ms_rot.size() * 16);
  put(o_mst, ms_tab.data(), ms_tab.size() * 16);
  put(o_dp, dp_tab.data(), dp_tab.size() * 16);
  if (e != cudaSuccess) return mcuda2(ctx, e, "uploading the magnetisation tables");
  WalkParams P;
  const double cell[3] = {1.0, 1.0, 1.0};
  fill_walk_params(P, base, L, g, kt, &rp, AXX_MODE_SINGLE, 0, init, cell, ctx->abort_dev);
  Q.tab = (const float4 *)(base + o_tab);
  Q.rk4 = (const float4 *)(base + o_rk4);
  Q.ms_idx = (const int2 *)(base + o_msi);
  Q.ms_rot = (const float4 *)(base + o_msr);
  Q.dp_tab = (const float4 *)(base + o_dp);
  Q.dp_K = dp_K;
  Q.dp_tol = (float)dp_tol;
  Q.ms_tab = (const float4 *)(base + o_mst);
  Q.partials = (double *)(base + o_part);
  Q.m_trace = (float *)(base + o_mtr);
  TraceParams T{};
  T.ntrace = nt;
  T.init_pos = (float *)(base + o_tip);
  T.pos = (float *)(base + o_tpos);
  T.hits = (int32_t *)(base + o_thit);
  T.words = (int32_t *)(base + o_twrd);
  double *d_out = (double *)(base + o_out);
  e = cudaMemsetAsync(P.counters, 0, AXX_CNT_N * 8, ctx->stream);
  if (e == cudaSuccess) e = launch_mag(g.geom, kt.km, mmax, nt > 0, P, Q, T, grid, ctx->stream);
  if (e == cudaSuccess) e = launch_reduce_partials(Q.partials, grid, nf * 3, d_out, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return mcuda2(ctx, e, "magnetisation walk");
  std::vector<double> h((size_t)nf * 3);
  unsigned long long cnt[AXX_CNT_N] = {0};
  e = cudaMemcpy(h.data(), d_out, h.size() * 8, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(cnt, P.counters, sizeof(cnt), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && nt > 0) {
    if (init_pos) e = cudaMemcpy(init_pos, T.init_pos, (size_t)nt * 12, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && pos && nmv) e = cudaMemcpy(pos, T.pos, nmv * 12, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && hits_out && nmv) e = cudaMemcpy(hits_out, T.hits, nmv * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && words_out && nmv) e = cudaMemcpy(words_out, T.words, nmv * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && m_final)
      e = cudaMemcpy(m_final, Q.m_trace, (size_t)nt * nf * 12, cudaMemcpyDeviceToHost);
  }
  if (e != cudaSuccess) return mcuda2(ctx, e, "reading the magnetisation");
  for (int j = 0; j < nf; ++j) {
    if (mx) mx[j] = h[3 * j];
    if (my) my[j] = h[3 * j + 1];
    if (mz) mz[j] = h[3 * j + 2];
  }
  if (cnt[AXX_CNT_ABORTED]) return mfail2(ctx, AXX_ERR_ABORTED, "run aborted by axx_abort");
  if (cnt[AXX_CNT_INIT_FAIL])
    return mfail2(ctx, AXX_ERR_INVALID_ARG, "no start position found in the pore");
  for (double v : h)
    if (!std::isfinite(v)) return mfail2(ctx, AXX_ERR_NUMERIC, "non-finite magnetisation");
  if (cnt[AXX_CNT_CAP])
    return mfail2(ctx, AXX_ERR_REFLECTION_CAP, "some moves hit the reflection cap of 1024");
  return AXX_OK;
}

}  // namespace
}  // namespace axx

extern "C" axx_status axx_run_mag(axx_ctx *ctx, const axx_basis *pore, const axx_field *fields,
                                  int nfield, const axx_mag_params *params, double *mx,
                                  double *my, double *mz) {
  return axx::mag_run(ctx, pore, fields, nfield, params, 0, nullptr, nullptr, nullptr, nullptr,
                      nullptr, mx, my, mz);
}

extern "C" axx_status axx_trace_mag(axx_ctx *ctx, const axx_basis *pore, const axx_field *fields,
                                    int nfield, const axx_mag_params *params, int ntrace,
                                    float *init_pos, float *pos, int32_t *hits, int32_t *words,
                                    float *m_final) {
  if (ntrace < 1) return AXX_ERR_INVALID_ARG;
  return axx::mag_run(ctx, pore, fields, nfield, params, ntrace, init_pos, pos, hits, words,
                      m_final, nullptr, nullptr, nullptr);
}
