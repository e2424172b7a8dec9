// walk_free.cu -- walk kernel instantiations: geometry class AXX_GEOM_FREE, walk modes 0.
#include "walk_instances.cuh"

namespace axx {

cudaError_t launch_walk_free(int km, int kmax, bool trace, bool one, bool gt, const WalkParams &P,
                           const TraceParams &T, int grid, size_t smem, cudaStream_t s) {
  switch (km) {
    case 0: return walk_launch_km<AXX_GEOM_FREE, 0>(kmax, trace, one, gt, P, T, grid, smem, s);
  }
  return cudaErrorInvalidValue;
}

int occupancy_walk_free(int km, int kmax, bool trace, bool one, bool gt, size_t smem) {
  switch (km) {
    case 0: return walk_occ_km<AXX_GEOM_FREE, 0>(kmax, trace, one, gt, smem);
  }
  return 0;
}

}  // namespace axx
