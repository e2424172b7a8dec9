// wc.cu -- the WCDMC comparison walker (Gaussian steps, simple rejection).
//
// Reference: kernelWC (src/kernels/kernelWC.cuh:13-89) driven by
// phaseAcquisitionStream::runAcquisitionWC
// (src/acquisition/phaseAcquisitionStream.cuh:193-252).  Per walker: a
// 32-bit xorshift state (x ^= x >> 13; x ^= x << 17; x ^= x >> 5; uniform
// (x + 1) / 2^32), and per step four uniforms -> two Box-Muller pairs ->
// displacements (dx, dy, dz) * sqrt(2 D dt); a move that leaves the pore is
// rejected; the phase accumulates G(t) . r with Kahan compensation and is
// scaled by gamma dt at the end.  The caller passes the per-walker states,
// start positions and the gradient table G[steps][3], as the reference's
// driver prepares them on the host.
//
// GB300: the walker's state, position and Kahan phase live in registers, the
// gradient row of a step is one uniform load per warp, the Box-Muller angles
// use this project's sin/cos(2 pi u) polynomial; FP32 throughout, FP64 sums
// of cos/sin of the phase per block.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/axx.h"
#include "axx_rng.cuh"
#include "ctx_internal.h"
#include "frame.h"
#include "walk_launch.h"

namespace axx {

struct WcArgs {
  long long n;
  int steps;
  int sph;
  float cx, cy, cz, R2;
  float sigma;         // sqrt(2 D dt)
  float gdt;           // gamma dt
  const uint32_t *state;
  const float4 *start;  // [n] (x, y, z, 0)
  const float4 *grad;   // [steps] (Gx, Gy, Gz, 0)
  float *phase;         // [n] or null
  double *partials;     // [grid][2]
};

__device__ __forceinline__ float xorshift_uniform(uint32_t &s) {
  uint32_t x = s;
  x ^= x >> 13;
  x ^= x << 17;
  x ^= x >> 5;
  s = x;
  return ((float)x + 1.0f) * 2.3283064365386963e-10f;  // (x + 1) / 2^32
}

__global__ void __launch_bounds__(256) wc_kernel(const __grid_constant__ WcArgs A) {
  __shared__ double red[2][8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double sc = 0.0, ss = 0.0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += stride) {
    uint32_t st = A.state[i];
    const float4 p0 = A.start[i];
    float x = p0.x, y = p0.y, z = p0.z;
    float ph = 0.0f, kc = 0.0f;
    for (int t = 0; t < A.steps; ++t) {
      const float u1 = xorshift_uniform(st), u2 = xorshift_uniform(st);
      const float u3 = xorshift_uniform(st), u4 = xorshift_uniform(st);
      float s1, c1, s2, c2;
      sincos_2pi(u2 - 0.5f, s1, c1);
      sincos_2pi(u4 - 0.5f, s2, c2);
      const float r1 = sqrt_f(-2.0f * logf(u1)), r2 = sqrt_f(-2.0f * logf(u3));
      const float x2 = fma_f(r1 * c1, A.sigma, x), y2 = fma_f(r1 * s1, A.sigma, y),
                  z2 = fma_f(r2 * c2, A.sigma, z);
      const float px = x2 - A.cx, py = y2 - A.cy, pz = A.sph ? (z2 - A.cz) : 0.0f;
      if (fma_f(px, px, fma_f(py, py, pz * pz)) < A.R2) {
        x = x2;
        y = y2;
        z = z2;
      }
      const float4 g = __ldg(&A.grad[t]);
      const float yk = fma_f(g.x, x, fma_f(g.y, y, g.z * z)) - kc;
      const float tk = ph + yk;
      kc = (tk - ph) - yk;
      ph = tk;
    }
    const float phase = ph * A.gdt;
    if (A.phase) A.phase[i] = phase;
    sc += (double)cosf(phase);
    ss += (double)sinf(phase);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sc += __shfl_xor_sync(0xffffffffu, sc, o);
    ss += __shfl_xor_sync(0xffffffffu, ss, o);
  }
  if (lane == 0) {
    red[0][w] = sc;
    red[1][w] = ss;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    double s = 0.0;
    for (int k = 0; k < 8; ++k) s += red[threadIdx.x][k];
    A.partials[(size_t)blockIdx.x * 2 + threadIdx.x] = s;
  }
}

}  // namespace axx

extern "C" axx_status axx_run_wc(axx_ctx *ctx, const axx_basis *pore, int64_t num_walkers,
                                 int32_t steps, double timestep, double gamma,
                                 const uint32_t *rng_state, const double *start,
                                 const double *grad, double *phase, double *sum_cos,
                                 double *sum_sin) {
  using namespace axx;
  if (!ctx) return AXX_ERR_INVALID_ARG;
  auto fail = [&](axx_status s, const std::string &m) {
    ctx->err = m;
    return s;
  };
  if (!pore || !rng_state || !start || !grad || num_walkers < 1 || steps < 0 ||
      !(timestep > 0.0) || !std::isfinite(gamma) || !(pore->radius > 0.0) || !(pore->D > 0.0))
    return fail(AXX_ERR_INVALID_ARG, "pore, walkers, steps, timestep or arrays out of range");
  if (pore->type != AXX_PRIM_CYLINDER_Z && pore->type != AXX_PRIM_SPHERE &&
      pore->type != AXX_PRIM_CYLINDER)
    return fail(AXX_ERR_INVALID_ARG, "unknown pore type");
  // an arbitrary-axis cylinder: positions and gradients in its frame
  Frame fr;
  std::string ferr = frame_single(pore, nullptr, 0, fr);
  if (!ferr.empty()) return fail(AXX_ERR_INVALID_ARG, ferr);
  pore = fr.basis_p;
  auto to_frame = [&](const double *v) {
    const double x = v[0], y = v[1], z = v[2];
    return make_float4((float)(fr.R[0][0] * x + fr.R[0][1] * y + fr.R[0][2] * z),
                       (float)(fr.R[1][0] * x + fr.R[1][1] * y + fr.R[1][2] * z),
                       (float)(fr.R[2][0] * x + fr.R[2][1] * y + fr.R[2][2] * z), 0.f);
  };
  const double g = gamma != 0.0 ? gamma : 267500.0;
  const long long n = num_walkers;
  std::vector<float4> h_start((size_t)n), h_grad((size_t)std::max(steps, 1));
  for (long long i = 0; i < n; ++i) h_start[i] = to_frame(start + 3 * i);
  for (int t = 0; t < steps; ++t) h_grad[t] = to_frame(grad + 3 * t);
  const int grid = (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, (long long)ctx->nsm * 8));
  auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t o_st = 0, o_p0 = up(o_st + (size_t)n * 4), o_g = up(o_p0 + (size_t)n * 16),
               o_ph = up(o_g + h_grad.size() * 16), o_part = up(o_ph + (size_t)n * 4),
               o_out = up(o_part + (size_t)grid * 16), total = up(o_out + 16);
  void *arena = nullptr;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e == cudaSuccess) e = cudaMalloc(&arena, total);
  if (e != cudaSuccess) {
    ctx->err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? AXX_ERR_OUT_OF_MEMORY : AXX_ERR_CUDA;
  }
  char *b = (char *)arena;
  WcArgs A{};
  A.n = n;
  A.steps = steps;
  A.sph = pore->type == AXX_PRIM_SPHERE;
  A.cx = (float)pore->cx;
  A.cy = (float)pore->cy;
  A.cz = (float)pore->cz;
  A.R2 = (float)(pore->radius * pore->radius);
  A.sigma = (float)std::sqrt(2.0 * pore->D * timestep);
  A.gdt = (float)(g * timestep);
  A.state = (const uint32_t *)(b + o_st);
  A.start = (const float4 *)(b + o_p0);
  A.grad = (const float4 *)(b + o_g);
  A.phase = (float *)(b + o_ph);
  A.partials = (double *)(b + o_part);
  e = cudaMemcpyAsync(b + o_st, rng_state, (size_t)n * 4, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b + o_p0, h_start.data(), (size_t)n * 16, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b + o_g, h_grad.data(), h_grad.size() * 16, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) {
    wc_kernel<<<grid, 256, 0, ctx->stream>>>(A);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = launch_reduce_partials(A.partials, grid, 2, (double *)(b + o_out), ctx->stream);
  double sums[2] = {0.0, 0.0};
  std::vector<float> ph;
  if (e == cudaSuccess) e = cudaMemcpyAsync(sums, b + o_out, 16, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess && phase) {
    ph.resize((size_t)n);
    e = cudaMemcpyAsync(ph.data(), A.phase, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(arena);
  if (e != cudaSuccess) {
    ctx->err = std::string("axx_run_wc: ") + cudaGetErrorString(e);
    return AXX_ERR_CUDA;
  }
  if (phase)
    for (long long i = 0; i < n; ++i) phase[i] = ph[i];
  if (sum_cos) *sum_cos = sums[0];
  if (sum_sin) *sum_sin = sums[1];
  return AXX_OK;
}
