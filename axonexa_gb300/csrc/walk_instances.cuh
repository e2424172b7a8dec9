// walk_instances.cuh -- launch and occupancy helpers for the instantiations
// of walk_kernel; each walk_*.cu translation unit instantiates one geometry
// class and a subset of walk modes, so the variants compile in parallel.
#pragma once
#include "walk_kernel.cuh"
#include "walk_launch.h"

namespace axx {

template <int GEOM, int KMAX, int KM, bool TRACE, bool ONE = false, bool GT = false,
          int PAX = 7>
static cudaError_t walk_go(const WalkParams &P, const TraceParams &T, int grid, size_t smem,
                           cudaStream_t s) {
  auto fn = walk_kernel<GEOM, KMAX, KM, TRACE, ONE, GT, PAX>;
  if (smem > 48 * 1024) {
    const cudaError_t e =
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  fn<<<grid, AXX_BLOCK, smem, s>>>(P, T);
  return cudaGetLastError();
}

template <int GEOM, int KMAX, int KM, bool TRACE, bool ONE = false, bool GT = false>
static int walk_occ(size_t smem) {
  auto fn = walk_kernel<GEOM, KMAX, KM, TRACE, ONE, GT>;
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
          cudaSuccess)
    return 0;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, AXX_BLOCK, smem) != cudaSuccess)
    return 0;
  return n;
}

// ONE: instantiations compiled for a single instance.  Single-pore modes
// (KM >= AXX_KM_SINGLE) always have one; lattices use them for up to four
// channels without traces when the plan has one instance and one cell.
template <int GEOM, int KM>
constexpr bool walk_one_variant(int kmax, bool trace, bool one) {
  return KM >= AXX_KM_SINGLE ||
         (one && !trace && kmax <= 4 && (GEOM == AXX_GEOM_CYL || GEOM == AXX_GEOM_SPH));
}

// gt: the plan keeps its tables in global memory; those instantiations exist
// for lattice walks with 16 channels (the host pads the channels) and traces.
template <int GEOM, int KM>
static cudaError_t walk_launch_km(int kmax, bool trace, bool one, bool gt, const WalkParams &P,
                                  const TraceParams &T, int grid, size_t smem, cudaStream_t s) {
  constexpr bool single = KM >= AXX_KM_SINGLE;
  constexpr bool lat1 = !single && (GEOM == AXX_GEOM_CYL || GEOM == AXX_GEOM_SPH);
  constexpr bool gt_ok = !single && GEOM != AXX_GEOM_FREE;
  if constexpr (gt_ok) {
    if (gt) {
      if (trace) return walk_go<GEOM, 1, KM, true, false, true>(P, T, grid, smem, s);
      if (kmax == 16) return walk_go<GEOM, 16, KM, false, false, true>(P, T, grid, smem, s);
      return cudaErrorInvalidValue;
    }
  }
  if constexpr (single) {
    if (trace) return walk_go<GEOM, 1, KM, true, single>(P, T, grid, smem, s);
    switch (kmax) {
      case 1: return walk_go<GEOM, 1, KM, false, single>(P, T, grid, smem, s);
      case 2: return walk_go<GEOM, 2, KM, false, single>(P, T, grid, smem, s);
      case 4: return walk_go<GEOM, 4, KM, false, single>(P, T, grid, smem, s);
      case 8: return walk_go<GEOM, 8, KM, false, single>(P, T, grid, smem, s);
      case 16: return walk_go<GEOM, 16, KM, false, single>(P, T, grid, smem, s);
    }
    return cudaErrorInvalidValue;
  } else {
  if (lat1 && walk_one_variant<GEOM, KM>(kmax, trace, one)) {
    // impermeable single cylinders without z phase: the instantiations that
    // walk no z, and no unbounded y when only x carries phase (their
    // occupancy is that of the instantiation below: the same launch bounds,
    // which every one of them meets without spilling)
    if constexpr (GEOM == AXX_GEOM_CYL && KM == AXX_KM_LAT_IMP) {
      if (!(P.phase_axes & 4) && !(P.phase_axes & 2)) {
        switch (kmax) {
          case 1: return walk_go<GEOM, 1, KM, false, true, false, 1>(P, T, grid, smem, s);
          case 2: return walk_go<GEOM, 2, KM, false, true, false, 1>(P, T, grid, smem, s);
          case 4: return walk_go<GEOM, 4, KM, false, true, false, 1>(P, T, grid, smem, s);
        }
      } else if (!(P.phase_axes & 4)) {
        switch (kmax) {
          case 1: return walk_go<GEOM, 1, KM, false, true, false, 3>(P, T, grid, smem, s);
          case 2: return walk_go<GEOM, 2, KM, false, true, false, 3>(P, T, grid, smem, s);
          case 4: return walk_go<GEOM, 4, KM, false, true, false, 3>(P, T, grid, smem, s);
        }
      }
    }
    switch (kmax) {
      case 1: return walk_go<GEOM, 1, KM, false, lat1>(P, T, grid, smem, s);
      case 2: return walk_go<GEOM, 2, KM, false, lat1>(P, T, grid, smem, s);
      case 4: return walk_go<GEOM, 4, KM, false, lat1>(P, T, grid, smem, s);
    }
  }
  if (trace) return walk_go<GEOM, 1, KM, true>(P, T, grid, smem, s);
  switch (kmax) {
    case 1: return walk_go<GEOM, 1, KM, false>(P, T, grid, smem, s);
    case 2: return walk_go<GEOM, 2, KM, false>(P, T, grid, smem, s);
    case 4: return walk_go<GEOM, 4, KM, false>(P, T, grid, smem, s);
    case 8: return walk_go<GEOM, 8, KM, false>(P, T, grid, smem, s);
    case 12:  // lattice walks only; axis channels for permeable cylinder lattices
      // (the impermeable walk's paired-move loop spills with them)
      if constexpr (GEOM == AXX_GEOM_CYL && KM == AXX_KM_LAT_PERM) {
        if (P.axis_channels)
          return walk_go<GEOM, 12, KM, false, false, false, AXX_PAX_AXES>(P, T, grid, smem, s);
      }
      return walk_go<GEOM, 12, KM, false>(P, T, grid, smem, s);
    case 16: return walk_go<GEOM, 16, KM, false>(P, T, grid, smem, s);
  }
  return cudaErrorInvalidValue;
  }
}

template <int GEOM, int KM>
static int walk_occ_km(int kmax, bool trace, bool one, bool gt, size_t smem) {
  constexpr bool single = KM >= AXX_KM_SINGLE;
  constexpr bool lat1 = !single && (GEOM == AXX_GEOM_CYL || GEOM == AXX_GEOM_SPH);
  constexpr bool gt_ok = !single && GEOM != AXX_GEOM_FREE;
  if constexpr (gt_ok) {
    if (gt) {
      if (trace) return walk_occ<GEOM, 1, KM, true, false, true>(smem);
      if (kmax == 16) return walk_occ<GEOM, 16, KM, false, false, true>(smem);
      return 0;
    }
  }
  if constexpr (single) {
    if (trace) return walk_occ<GEOM, 1, KM, true, single>(smem);
    switch (kmax) {
      case 1: return walk_occ<GEOM, 1, KM, false, single>(smem);
      case 2: return walk_occ<GEOM, 2, KM, false, single>(smem);
      case 4: return walk_occ<GEOM, 4, KM, false, single>(smem);
      case 8: return walk_occ<GEOM, 8, KM, false, single>(smem);
      case 16: return walk_occ<GEOM, 16, KM, false, single>(smem);
    }
    return 0;
  } else {
  if (lat1 && walk_one_variant<GEOM, KM>(kmax, trace, one)) {
    switch (kmax) {
      case 1: return walk_occ<GEOM, 1, KM, false, lat1>(smem);
      case 2: return walk_occ<GEOM, 2, KM, false, lat1>(smem);
      case 4: return walk_occ<GEOM, 4, KM, false, lat1>(smem);
    }
  }
  if (trace) return walk_occ<GEOM, 1, KM, true>(smem);
  switch (kmax) {
    case 1: return walk_occ<GEOM, 1, KM, false>(smem);
    case 2: return walk_occ<GEOM, 2, KM, false>(smem);
    case 4: return walk_occ<GEOM, 4, KM, false>(smem);
    case 8: return walk_occ<GEOM, 8, KM, false>(smem);
    case 12: return walk_occ<GEOM, 12, KM, false>(smem);
    case 16: return walk_occ<GEOM, 16, KM, false>(smem);
  }
  return 0;
  }
}

}  // namespace axx
