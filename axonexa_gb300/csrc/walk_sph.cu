// walk_sph.cu -- walk kernel instantiations for geometry class AXX_GEOM_SPH.
#include "walk_kernel.cuh"
#include "walk_launch.h"

namespace axx {

template <int KMAX, bool TRACE>
static cudaError_t go(const WalkParams &P, const TraceParams &T, int grid, size_t smem,
                      cudaStream_t s) {
  auto fn = walk_kernel<AXX_GEOM_SPH, KMAX, TRACE>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  fn<<<grid, AXX_BLOCK, smem, s>>>(P, T);
  return cudaGetLastError();
}

template <int KMAX, bool TRACE>
static int occ(size_t smem) {
  auto fn = walk_kernel<AXX_GEOM_SPH, KMAX, TRACE>;
  if (smem > 48 * 1024) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, AXX_BLOCK, smem) != cudaSuccess) return 0;
  return n;
}

cudaError_t launch_walk_sph(int kmax, bool trace, const WalkParams &P, const TraceParams &T,
                           int grid, size_t smem, cudaStream_t s) {
  if (trace) return go<1, true>(P, T, grid, smem, s);
  switch (kmax) {
    case 1: return go<1, false>(P, T, grid, smem, s);
    case 2: return go<2, false>(P, T, grid, smem, s);
    case 4: return go<4, false>(P, T, grid, smem, s);
    case 8: return go<8, false>(P, T, grid, smem, s);
    case 16: return go<16, false>(P, T, grid, smem, s);
  }
  return cudaErrorInvalidValue;
}

int occupancy_walk_sph(int kmax, bool trace, size_t smem) {
  if (trace) return occ<1, true>(smem);
  switch (kmax) {
    case 1: return occ<1, false>(smem);
    case 2: return occ<2, false>(smem);
    case 4: return occ<4, false>(smem);
    case 8: return occ<8, false>(smem);
    case 16: return occ<16, false>(smem);
  }
  return 0;
}

}  // namespace axx
