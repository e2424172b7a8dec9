// walk_launch.h -- host entry points of the walk kernel instantiations.
#pragma once
#include <cuda_runtime.h>
#include "axx_walk.h"

namespace axx {

// One function per geometry class, compiled in its own translation unit.
// kmax in {1, 2, 4, 8, 16}.  Returns the launch error.
cudaError_t launch_walk_free(int kmax, bool trace, const WalkParams &P, const TraceParams &T,
                             int grid, size_t smem, cudaStream_t s);
cudaError_t launch_walk_cyl(int kmax, bool trace, const WalkParams &P, const TraceParams &T,
                            int grid, size_t smem, cudaStream_t s);
cudaError_t launch_walk_sph(int kmax, bool trace, const WalkParams &P, const TraceParams &T,
                            int grid, size_t smem, cudaStream_t s);
cudaError_t launch_walk_mix(int kmax, bool trace, const WalkParams &P, const TraceParams &T,
                            int grid, size_t smem, cudaStream_t s);
// Resident blocks per SM of one instantiation at the given dynamic smem.
int occupancy_walk_free(int kmax, bool trace, size_t smem);
int occupancy_walk_cyl(int kmax, bool trace, size_t smem);
int occupancy_walk_sph(int kmax, bool trace, size_t smem);
int occupancy_walk_mix(int kmax, bool trace, size_t smem);
inline int occupancy_walk(int geom, int kmax, bool trace, size_t smem) {
  switch (geom) {
    case AXX_GEOM_FREE: return occupancy_walk_free(kmax, trace, smem);
    case AXX_GEOM_CYL: return occupancy_walk_cyl(kmax, trace, smem);
    case AXX_GEOM_SPH: return occupancy_walk_sph(kmax, trace, smem);
    default: return occupancy_walk_mix(kmax, trace, smem);
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
