// pack.cu -- gamma-radius cylinder packings generated on the GPU, many at a
// time (the substrate generator RPSLatticeInitializer,
// src/substrate/RPSinitializer.h:10-314, restated for one thread block per
// packing).
//
// Per packing (block of 256 threads, positions and radii in shared memory):
//  1. n radii from gamma(shape, mean/shape) truncated to (rmin, rmax)
//     (gammaRadialDist :76-101): the Marsaglia-Tsang sampler (ACM TOMS
//     26(3), 2000) on Box-Muller normals, one radius per thread at a time,
//     uniforms from Philox4x32-10 keyed by (seed, packing, radius, trial);
//  2. radii sorted (bitonic sort in shared memory); the cell side L makes the
//     cylinders' area the requested fraction;
//  3. random sequential addition, largest radius first (uniformCenterDist
//     :103-129): 256 candidate centres at a time, one per thread, each tested
//     against every placed cylinder with the periodic (minimum-image) overlap
//     test and a gap of 1 % of the radius sum; the lowest-numbered thread whose
//     candidate fits places the cylinder; up to 2,048 candidates per cylinder;
//  4. when addition jams (its limit is near 0.55 for equal discs), it places
//     the cylinders at a lower fraction and the cell is compressed to the
//     requested one in steps of 0.01, each followed by overlap removal: every
//     pair closer than the minimum separation moves apart along its centre
//     line by half the shortfall, all pairs at once, until no pair overlaps;
//  5. the cylinders, smallest radius first with region = index + 1, then the
//     periodic images of those that cross the cell edge (correctEdges
//     :131-186), in a fixed order.
// The host packer (substrate.cpp) follows the same steps on the CPU with
// SplitMix64 draws, one candidate at a time and in-place (sequential) overlap
// removal; packings agree in distribution, not draw by draw.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/axx.h"
#include "axx_rng.cuh"
#include "ctx_internal.h"

namespace axx {

constexpr int PK_THREADS = 256;
constexpr int PK_MAX_N = 2048;
constexpr double PK_GAP = 1.01;
constexpr int PK_RSA_ROUNDS = 8;       // 8 x 256 candidates per cylinder
constexpr int PK_RELAX_ITERS = 20000;
constexpr int PK_TRIES = 4096;         // gamma draws per radius before giving up

enum { PK_OK = 0, PK_ERR_RADII = 1, PK_ERR_RELAX = 2, PK_ERR_OUT = 3 };

struct PackArgs {
  uint64_t seed;
  int n, npack, max_out, n2;  // n2: power of two >= n
  const axx_pack_spec *spec;
  axx_basis *out;
  int *nout;
  double *side, *achieved;
  int *status;
};

// Two uniforms in (0, 1) with 53-bit mantissas from one Philox block keyed by
// the seed, counter (a, b, c, packing).
__device__ __forceinline__ void uniforms2(uint64_t seed, uint32_t a, uint32_t b, uint32_t c,
                                          uint32_t p, double &u0, double &u1) {
  const Words4 w = philox4x32_10(a, b, c, p, (uint32_t)seed, (uint32_t)(seed >> 32));
  const double s = 1.0 / 9007199254740992.0;  // 2^-53
  u0 = ((double)(((uint64_t)(w.x >> 5) << 26) | (w.y >> 6)) + 0.5) * s;
  u1 = ((double)(((uint64_t)(w.z >> 5) << 26) | (w.w >> 6)) + 0.5) * s;
}

// Gamma(k, theta) by Marsaglia-Tsang; k < 1 through gamma(k + 1) u^(1/k).
// Draws come from counter (i, trial, stream); returns a negative value when
// PK_TRIES trials find no sample.
__device__ double gamma_draw(uint64_t seed, uint32_t p, uint32_t i, uint32_t &trial, double k,
                             double theta) {
  double boost = 1.0;
  if (k < 1.0) {
    double u, v;
    uniforms2(seed, i, trial++, 3u, p, u, v);
    boost = pow(u, 1.0 / k);
    k += 1.0;
  }
  const double d = k - 1.0 / 3.0, c = 1.0 / sqrt(9.0 * d);
  for (int t = 0; t < PK_TRIES; ++t) {
    double u1, u2, u3, u4;
    uniforms2(seed, i, trial, 1u, p, u1, u2);
    uniforms2(seed, i, trial, 2u, p, u3, u4);
    ++trial;
    const double x = sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
    double v = 1.0 + c * x;
    if (v <= 0.0) continue;
    v = v * v * v;
    if (log(u3) < 0.5 * x * x + d - d * v + d * log(v)) return d * v * theta * boost;
  }
  return -1.0;
}

__device__ __forceinline__ double min_image(double d, double L) {
  return d - L * nearbyint(d / L);
}

// circleIntersectsLattice for a square cell of side L (RPSinitializer.h:251-276)
__device__ __forceinline__ bool circle_meets_cell(double x, double y, double r, double L) {
  const double h = 0.5 * L;
  const double dx = fabs(x - h), dy = fabs(y - h);
  if (dx > h + r || dy > h + r) return false;
  if (dx <= h || dy <= h) return true;
  return (dx - h) * (dx - h) + (dy - h) * (dy - h) <= r * r;
}

__global__ void __launch_bounds__(PK_THREADS) rps_pack_kernel(const __grid_constant__ PackArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  double *r = reinterpret_cast<double *>(smem);     // [n2] radii (sorted descending)
  double *x = r + a.n2;                              // [n] centres
  double *y = x + a.n;
  double *px = y + a.n;                              // [n] pushes (relaxation)
  double *py = px + a.n;
  int *cnt = reinterpret_cast<int *>(py + a.n);     // [n] images per cylinder, then offsets
  __shared__ double red[PK_THREADS];
  __shared__ int s_flag, s_winner, s_err;
  const int p = blockIdx.x, tid = threadIdx.x, n = a.n;
  const axx_pack_spec sp = a.spec[p];
  if (tid == 0) s_err = PK_OK;
  // 1. radii
  for (int i = tid; i < a.n2; i += PK_THREADS) {
    if (i >= n) {
      r[i] = -1.0;  // padding sorts last
      continue;
    }
    uint32_t trial = 0;
    double v = -1.0;
    for (int t = 0; t < PK_TRIES; ++t) {
      v = gamma_draw(a.seed, (uint32_t)p, (uint32_t)i, trial, sp.shape, sp.mean / sp.shape);
      if (v < 0.0 || (v > sp.rmin && v < sp.rmax)) break;
    }
    if (!(v > sp.rmin && v < sp.rmax)) {
      s_err = PK_ERR_RADII;
      v = sp.rmin > 0.0 ? sp.rmin : sp.mean;
    }
    r[i] = v;
  }
  __syncthreads();
  // 2. bitonic sort, descending
  for (int k = 2; k <= a.n2; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = tid; i < a.n2; i += PK_THREADS) {
        const int l = i ^ j;
        if (l > i) {
          const bool desc = (i & k) == 0;
          const double ri = r[i], rl = r[l];
          if (desc ? (ri < rl) : (ri > rl)) {
            r[i] = rl;
            r[l] = ri;
          }
        }
      }
      __syncthreads();
    }
  // area in a fixed order: per-thread strided sums, then a fixed tree
  double part = 0.0;
  for (int i = tid; i < n; i += PK_THREADS) part += 3.141592653589793 * r[i] * r[i];
  red[tid] = part;
  __syncthreads();
  for (int w = PK_THREADS / 2; w > 0; w >>= 1) {
    if (tid < w) red[tid] += red[tid + w];
    __syncthreads();
  }
  const double area = red[0];
  const double L = sqrt(area / sp.fraction);
  // 3. random sequential addition, largest first, in a cell of side Lc
  //    (attempt `att` draws its own candidates); false when a cylinder finds
  //    no place among PK_RSA_ROUNDS x 256 candidates
  auto rsa = [&](double Lc, uint32_t att) {
    for (int i = 0; i < n; ++i) {
      bool done = false;
      for (int round = 0; round < PK_RSA_ROUNDS && !done; ++round) {
        double cx, cy;
        uniforms2(a.seed, (uint32_t)i, (uint32_t)(round * PK_THREADS + tid), 0x40000000u + att,
                  (uint32_t)p, cx, cy);
        cx *= Lc;
        cy *= Lc;
        bool ok = true;
        for (int j = 0; j < i && ok; ++j) {
          const double dx = min_image(cx - x[j], Lc), dy = min_image(cy - y[j], Lc);
          const double sr = (r[i] + r[j]) * PK_GAP;
          ok = dx * dx + dy * dy >= sr * sr;
        }
        if (tid == 0) s_winner = PK_THREADS;
        __syncthreads();
        if (ok) atomicMin(&s_winner, tid);
        __syncthreads();
        if (s_winner < PK_THREADS) {
          if (tid == s_winner) {
            x[i] = cx;
            y[i] = cy;
          }
          done = true;
        }
        __syncthreads();
      }
      if (!done) return false;
    }
    return true;
  };
  // 4. overlap removal in a cell of side Lc: every pair closer than the
  //    minimum separation moves apart along its centre line by half the
  //    shortfall (plus 0.1 % and 1e-9 of the cell: an overlap below the
  //    rounding of the centres would otherwise move them by less than one
  //    ulp, forever), all pairs at once
  auto relax = [&](double Lc) {
    for (int it = 0; it < PK_RELAX_ITERS; ++it) {
      if (tid == 0) s_flag = 0;
      __syncthreads();
      bool any = false;
      for (int i = tid; i < n; i += PK_THREADS) {
        double sx = 0.0, sy = 0.0;
        for (int j = 0; j < n; ++j) {
          if (j == i) continue;
          double dx = min_image(x[i] - x[j], Lc), dy = min_image(y[i] - y[j], Lc);
          const double sr = (r[i] + r[j]) * PK_GAP;
          const double d2 = dx * dx + dy * dy;
          if (d2 >= sr * sr) continue;
          any = true;
          double d = sqrt(d2);
          if (d < 1e-12 * Lc) {  // coincident centres: apart along x, by index
            dx = j > i ? -1.0 : 1.0;
            dy = 0.0;
            d = 1.0;
          }
          const double push = 0.5 * (sr - sqrt(d2)) * 1.001 + 1e-9 * Lc;
          sx += push * dx / d;
          sy += push * dy / d;
        }
        px[i] = sx;
        py[i] = sy;
      }
      if (any) s_flag = 1;
      __syncthreads();
      if (!s_flag) return true;
      for (int i = tid; i < n; i += PK_THREADS) {
        const double nx = x[i] + px[i], ny = y[i] + py[i];
        x[i] = nx - Lc * floor(nx / Lc);
        y[i] = ny - Lc * floor(ny / Lc);
      }
      __syncthreads();
    }
    return false;
  };
  if (!rsa(L, 0u)) {
    // addition jammed: add at a lower fraction, then compress the cell in
    // steps of 0.01 in fraction, scaling the centres with it and removing
    // the overlaps after each step
    double fc = fmin(0.5, sp.fraction);
    uint32_t att = 1;
    while (!rsa(sqrt(area / fc), att++)) {
      fc -= 0.05;
      if (fc < 0.1) break;
    }
    if (fc < 0.1) {
      if (tid == 0) s_err = PK_ERR_RELAX;
    } else {
      double Lc = sqrt(area / fc);
      while (fc < sp.fraction) {
        fc = fmin(sp.fraction, fc + 0.01);
        const double Ln = fc == sp.fraction ? L : sqrt(area / fc);
        for (int i = tid; i < n; i += PK_THREADS) {
          x[i] *= Ln / Lc;
          y[i] *= Ln / Lc;
        }
        Lc = Ln;
        __syncthreads();
        if (!relax(Lc)) {
          if (tid == 0) s_err = PK_ERR_RELAX;
          break;
        }
      }
    }
  }
  __syncthreads();
  // 5. outputs: cylinder q = n - 1 - i (ascending radius), then the images
  auto idx = [&](int q) { return n - 1 - q; };  // storage index of output cylinder q
  for (int q = tid; q < n; q += PK_THREADS) {
    const int i = idx(q);
    const bool crosses =
        x[i] + r[i] > L || x[i] - r[i] < 0.0 || y[i] + r[i] > L || y[i] - r[i] < 0.0;
    int c = 0;
    if (crosses)
      for (int aa = -1; aa <= 1; ++aa)
        for (int bb = -1; bb <= 1; ++bb)
          if ((aa || bb) && circle_meets_cell(x[i] + L * aa, y[i] + L * bb, r[i], L)) ++c;
    cnt[q] = c;
  }
  __syncthreads();
  if (tid == 0) {  // exclusive scan (n <= 2048, once per packing)
    int s = n;
    for (int q = 0; q < n; ++q) {
      const int c = cnt[q];
      cnt[q] = s;
      s += c;
    }
    a.nout[p] = s;
    if (s > a.max_out) s_err = PK_ERR_OUT;
  }
  __syncthreads();
  axx_basis *o = a.out + (size_t)p * a.max_out;
  const bool room = s_err != PK_ERR_OUT;
  for (int q = tid; q < n && room; q += PK_THREADS) {
    const int i = idx(q);
    auto emit = [&](int slot, double cx, double cy) {
      axx_basis b;
      b.type = AXX_PRIM_CYLINDER_Z;
      b.region = q + 1;
      b.cx = cx;
      b.cy = cy;
      b.cz = 0.0;
      b.radius = r[i];
      b.D = sp.D;
      b.T2 = sp.T2;
      b.T1 = 0.0;
      b.permeability = sp.permeability;
      b.eps = 1e-14;  // the reference's default cylEPS (cylinderXY.cuh:26)
      b.nx = b.ny = b.nz = 0.0;
      o[slot] = b;
    };
    emit(q, x[i], y[i]);
    int slot = cnt[q];
    const bool crosses =
        x[i] + r[i] > L || x[i] - r[i] < 0.0 || y[i] + r[i] > L || y[i] - r[i] < 0.0;
    if (crosses)
      for (int aa = -1; aa <= 1; ++aa)
        for (int bb = -1; bb <= 1; ++bb)
          if ((aa || bb) && circle_meets_cell(x[i] + L * aa, y[i] + L * bb, r[i], L))
            emit(slot++, x[i] + L * aa, y[i] + L * bb);
  }
  if (tid == 0) {
    a.side[p] = L;
    a.achieved[p] = area / (L * L);
    a.status[p] = s_err;
  }
}

}  // namespace axx

using namespace axx;

extern "C" axx_status axx_substrate_rps_gamma_gpu(axx_ctx *ctx, uint64_t seed, int n, int npack,
                                                  const axx_pack_spec *spec, int max_out,
                                                  axx_basis *out, int *nout, double *side,
                                                  double *achieved) {
  if (!ctx) return AXX_ERR_INVALID_ARG;
  auto fail = [&](axx_status s, const std::string &m) {
    ctx->err = m;
    return s;
  };
  if (n < 1 || n > PK_MAX_N) return fail(AXX_ERR_INVALID_ARG, "n must be in [1, 2048]");
  if (npack < 1 || !spec || !out || !nout || !side || !achieved || max_out < n)
    return fail(AXX_ERR_INVALID_ARG, "invalid packing arguments");
  for (int p = 0; p < npack; ++p) {
    const axx_pack_spec &s = spec[p];
    if (!(s.shape > 0.0) || !(s.mean > 0.0) || !(s.rmax > s.rmin) || !(s.rmin >= 0.0) ||
        !(s.fraction > 0.0 && s.fraction < 0.9) || !std::isfinite(s.shape + s.mean + s.rmax))
      return fail(AXX_ERR_INVALID_ARG, "packing " + std::to_string(p) + ": invalid spec");
  }
  cudaError_t e = cudaSetDevice(ctx->device);
  int n2 = 1;
  while (n2 < n) n2 <<= 1;
  const size_t smem = (size_t)n2 * 8 + (size_t)n * 8 * 4 + (size_t)n * 4;
  char *d = nullptr;
  const size_t o_spec = 0, o_out = (sizeof(axx_pack_spec) * npack + 255) & ~(size_t)255;
  const size_t o_nout = o_out + ((sizeof(axx_basis) * (size_t)npack * max_out + 255) & ~(size_t)255);
  const size_t o_side = o_nout + ((4 * (size_t)npack + 255) & ~(size_t)255);
  const size_t o_ach = o_side + 8 * (size_t)npack;
  const size_t o_st = o_ach + 8 * (size_t)npack;
  const size_t total = o_st + 4 * (size_t)npack;
  if (e == cudaSuccess) e = cudaMalloc(&d, total);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d + o_spec, spec, sizeof(axx_pack_spec) * npack, cudaMemcpyHostToDevice,
                        ctx->stream);
  if (e == cudaSuccess && smem > 48 * 1024)
    e = cudaFuncSetAttribute(rps_pack_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
  if (e == cudaSuccess) {
    PackArgs a;
    a.seed = seed;
    a.n = n;
    a.npack = npack;
    a.max_out = max_out;
    a.n2 = n2;
    a.spec = reinterpret_cast<const axx_pack_spec *>(d + o_spec);
    a.out = reinterpret_cast<axx_basis *>(d + o_out);
    a.nout = reinterpret_cast<int *>(d + o_nout);
    a.side = reinterpret_cast<double *>(d + o_side);
    a.achieved = reinterpret_cast<double *>(d + o_ach);
    a.status = reinterpret_cast<int *>(d + o_st);
    rps_pack_kernel<<<npack, PK_THREADS, smem, ctx->stream>>>(a);
    e = cudaGetLastError();
  }
  std::vector<int> st(npack);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpy(out, d + o_out, sizeof(axx_basis) * (size_t)npack * max_out,
                   cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(nout, d + o_nout, 4 * (size_t)npack, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(side, d + o_side, 8 * (size_t)npack, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess)
    e = cudaMemcpy(achieved, d + o_ach, 8 * (size_t)npack, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(st.data(), d + o_st, 4 * (size_t)npack, cudaMemcpyDeviceToHost);
  if (d) cudaFree(d);
  if (e != cudaSuccess) {
    ctx->err = std::string("axx_substrate_rps_gamma_gpu: ") + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? AXX_ERR_OUT_OF_MEMORY : AXX_ERR_CUDA;
  }
  for (int p = 0; p < npack; ++p) {
    if (st[p] == PK_ERR_RADII)
      return fail(AXX_ERR_INVALID_ARG, "packing " + std::to_string(p) +
                                           ": no gamma radius in (rmin, rmax) after 4096 draws");
    if (st[p] == PK_ERR_RELAX)
      return fail(AXX_ERR_UNSUPPORTED, "packing " + std::to_string(p) +
                                           ": overlap removal did not converge");
    if (st[p] == PK_ERR_OUT)
      return fail(AXX_ERR_INVALID_ARG, "packing " + std::to_string(p) +
                                           ": more bases (with images) than max_out");
  }
  return AXX_OK;
}
