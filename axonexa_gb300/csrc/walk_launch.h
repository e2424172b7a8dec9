// walk_launch.h -- host entry points of the walk kernel instantiations.
#pragma once
#include <cuda_runtime.h>
#include "axx_walk.h"

namespace axx {

// One function pair per translation unit (geometry class x walk modes).
// kmax in {1, 2, 4, 8, 16}; km is AXX_KM_*.  Launches return the launch error.
#define AXX_DECLARE_WALK(name)                                                              \
  cudaError_t launch_walk_##name(int km, int kmax, bool trace, bool one, bool gt,            \
                                 const WalkParams &P, const TraceParams &T, int grid,         \
                                 size_t smem, cudaStream_t s);                                \
  int occupancy_walk_##name(int km, int kmax, bool trace, bool one, bool gt, size_t smem);
AXX_DECLARE_WALK(free)
AXX_DECLARE_WALK(cyl_lat)
AXX_DECLARE_WALK(cyl_single)
AXX_DECLARE_WALK(sph_lat)
AXX_DECLARE_WALK(sph_single)
AXX_DECLARE_WALK(mix)
#undef AXX_DECLARE_WALK

// one: the plan has a single instance and a single cell (P.n_inst == 1,
// P.ncell == 1) and no compartment sums, which selects the instantiations
// compiled for that case.
inline cudaError_t launch_walk(int geom, int km, int kmax, bool trace, const WalkParams &P,
                               const TraceParams &T, int grid, size_t smem, cudaStream_t s) {
  const bool single = km >= AXX_KM_SINGLE;
  const bool one = P.n_inst == 1 && P.ncell == 1 && !P.compart;
  const bool gt = P.global_tables != 0;
  switch (geom) {
    case AXX_GEOM_FREE: return launch_walk_free(km, kmax, trace, one, gt, P, T, grid, smem, s);
    case AXX_GEOM_CYL:
      return single ? launch_walk_cyl_single(km, kmax, trace, one, gt, P, T, grid, smem, s)
                    : launch_walk_cyl_lat(km, kmax, trace, one, gt, P, T, grid, smem, s);
    case AXX_GEOM_SPH:
      return single ? launch_walk_sph_single(km, kmax, trace, one, gt, P, T, grid, smem, s)
                    : launch_walk_sph_lat(km, kmax, trace, one, gt, P, T, grid, smem, s);
    default: return launch_walk_mix(km, kmax, trace, one, gt, P, T, grid, smem, s);
  }
}

inline int occupancy_walk(int geom, int km, int kmax, bool trace, bool one, bool gt,
                          size_t smem) {
  const bool single = km >= AXX_KM_SINGLE;
  switch (geom) {
    case AXX_GEOM_FREE: return occupancy_walk_free(km, kmax, trace, one, gt, smem);
    case AXX_GEOM_CYL:
      return single ? occupancy_walk_cyl_single(km, kmax, trace, one, gt, smem)
                    : occupancy_walk_cyl_lat(km, kmax, trace, one, gt, smem);
    case AXX_GEOM_SPH:
      return single ? occupancy_walk_sph_single(km, kmax, trace, one, gt, smem)
                    : occupancy_walk_sph_lat(km, kmax, trace, one, gt, smem);
    default: return occupancy_walk_mix(km, kmax, trace, one, gt, smem);
  }
}

cudaError_t launch_reduce_partials(const double *partials, int nblocks, int nout, double *out,
                                   cudaStream_t s);
// FMA microbenchmark: grid x block threads, iters x kFmaPerIter FMAs each.
constexpr int kFmaPerIter = 64;
cudaError_t launch_fma_peak(int grid, int block, int iters, float *out, cudaStream_t s);
cudaError_t launch_philox_words(uint64_t seed, uint64_t walker, int n, uint32_t *out,
                                cudaStream_t s);

}  // namespace axx
