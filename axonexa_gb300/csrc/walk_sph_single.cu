// walk_sph_single.cu -- walk kernel instantiations: geometry class AXX_GEOM_SPH, walk modes 3 4.
#include "walk_instances.cuh"

namespace axx {

cudaError_t launch_walk_sph_single(int km, int kmax, bool trace, bool one, bool gt, const WalkParams &P,
                           const TraceParams &T, int grid, size_t smem, cudaStream_t s) {
  switch (km) {
    case 3: return walk_launch_km<AXX_GEOM_SPH, 3>(kmax, trace, one, gt, P, T, grid, smem, s);
    case 4: return walk_launch_km<AXX_GEOM_SPH, 4>(kmax, trace, one, gt, P, T, grid, smem, s);
  }
  return cudaErrorInvalidValue;
}

int occupancy_walk_sph_single(int km, int kmax, bool trace, bool one, bool gt, size_t smem) {
  switch (km) {
    case 3: return walk_occ_km<AXX_GEOM_SPH, 3>(kmax, trace, one, gt, smem);
    case 4: return walk_occ_km<AXX_GEOM_SPH, 4>(kmax, trace, one, gt, smem);
  }
  return 0;
}

}  // namespace axx
