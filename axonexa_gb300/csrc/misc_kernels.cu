// misc_kernels.cu -- final signal reduction and stream inspection kernels.
#include <cuda_runtime.h>
#include "axx_rng.cuh"
#include "walk_launch.h"

namespace axx {

// out[j] = sum over blocks b of partials[b * nout + j], one block per output,
// fixed summation order (deterministic across runs).
__global__ void __launch_bounds__(256) reduce_partials_kernel(const double *__restrict__ partials,
                                                              int nblocks, int nout,
                                                              double *__restrict__ out) {
  __shared__ double red[256];
  const int j = blockIdx.x;
  double s = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) s += partials[(size_t)b * nout + j];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[j] = red[0];
}

cudaError_t launch_reduce_partials(const double *partials, int nblocks, int nout, double *out,
                                   cudaStream_t s) {
  if (nout <= 0) return cudaSuccess;
  reduce_partials_kernel<<<nout, 256, 0, s>>>(partials, nblocks, nout, out);
  return cudaGetLastError();
}

// 8 independent FMA chains of 8 per iteration (64 FMAs), enough ILP to keep
// the FMA pipe busy at full occupancy.
__global__ void __launch_bounds__(256) fma_peak_kernel(int iters, float *out) {
  float a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = (float)(threadIdx.x + k) * 1e-3f;
  const float m = 0.999f, c = 1e-4f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int r = 0; r < 8; ++r)
#pragma unroll
      for (int k = 0; k < 8; ++k) a[k] = __fmaf_rn(a[k], m, c);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

cudaError_t launch_fma_peak(int grid, int block, int iters, float *out, cudaStream_t s) {
  fma_peak_kernel<<<grid, block, 0, s>>>(iters, out);
  return cudaGetLastError();
}

__global__ void philox_words_kernel(uint64_t seed, uint64_t walker, int n, uint32_t *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t blk = (uint32_t)(i >> 2);
  const Words4 o = philox4x32_10(blk, 0u, (uint32_t)walker, (uint32_t)(walker >> 32),
                                 (uint32_t)seed, (uint32_t)(seed >> 32));
  const int r = i & 3;
  out[i] = r == 0 ? o.x : r == 1 ? o.y : r == 2 ? o.z : o.w;
}

cudaError_t launch_philox_words(uint64_t seed, uint64_t walker, int n, uint32_t *out,
                                cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  philox_words_kernel<<<(n + 255) / 256, 256, 0, s>>>(seed, walker, n, out);
  return cudaGetLastError();
}

}  // namespace axx
