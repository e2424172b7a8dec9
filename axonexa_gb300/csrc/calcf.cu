// calcf.cu -- Monte Carlo intracellular volume fraction of a lattice substrate.
//
// Reference: calcf + kernelCalcf (src/util/calcf.cuh:1-38): one point per
// stream, placed by Lattice::initializeUniformly, counted when
// Lattice::inRegion gives a region > 0; the fraction is the count over the
// points.  (As written the reference does not build -- it passes an
// undeclared `maxthreads` -- and divides two ints, which would return 0 or 1;
// this is the intended fraction.)  Here point i takes words 1..3 of stream
// (seed, i), the start-position draws of the walk, and the region is the
// walk's first-containing-instance lookup over the point's cell list; each
// warp sums its count and one atomic per warp adds it.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/axx.h"
#include "ctx_internal.h"
#include "frame.h"
#include "host_plan.h"
#include "plan_layout.h"
#include "walk_kernel.cuh"

namespace axx {

template <int GEOM>
__global__ void __launch_bounds__(256) calcf_kernel(const __grid_constant__ WalkParams P,
                                                     long long points,
                                                     unsigned long long *count) {
  SmemView S;
  S.geo = P.inst_geo;
  S.aux = P.inst_aux;
  S.slot = P.slot_tab;
  S.cstart = P.cell_start;
  S.region = P.slot_region;
  S.clist = P.cell_list;
  unsigned long long c = 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < points; i += stride) {
    DevStream st;
    st.init(P, (uint64_t)i, 1u);
    const float x = st.next(P) * P.a, y = st.next(P) * P.b, z = st.next(P) * P.c;
    int slot = P.ecs_slot;
    if (GEOM != AXX_GEOM_FREE) {
      const int cell = cell_of<GEOM>(P, x, y, z);
      slot = lookup_list<GEOM>(S, S.cstart[cell], S.cstart[cell + 1], P.ecs_slot, x, y, z);
    }
    c += S.region[slot] > 0 ? 1ull : 0ull;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

namespace {

template <int GEOM>
cudaError_t launch_calcf(const WalkParams &P, long long points, unsigned long long *count,
                         int grid, cudaStream_t s) {
  calcf_kernel<GEOM><<<grid, 256, 0, s>>>(P, points, count);
  return cudaGetLastError();
}

struct Buf {
  void *p = nullptr;
  ~Buf() {
    if (p) cudaFree(p);
  }
};

}  // namespace
}  // namespace axx

extern "C" axx_status axx_volume_fraction(axx_ctx *ctx, const axx_lattice *lat,
                                          const axx_basis *basis, int nbasis, int64_t points,
                                          uint64_t seed, double *fraction, int64_t *inside) {
  using namespace axx;
  if (!ctx) return AXX_ERR_INVALID_ARG;
  auto fail = [&](axx_status s, const std::string &m) {
    ctx->err = m;
    return s;
  };
  if (!lat || (nbasis > 0 && !basis) || nbasis < 0 || points < 1)
    return fail(AXX_ERR_INVALID_ARG, "lattice, bases or point count out of range");
  // a vanishing time step: the instance set and cell lists of the walk at
  // (almost) zero step length -- bases and the ghosts that meet the cell
  GeomPlan g;
  Frame fr;  // lattices of x- or y-axis cylinders run with permuted axes
  std::string err = frame_lattice(lat, basis, nbasis, nullptr, 0, fr);
  if (!err.empty()) return fail(AXX_ERR_INVALID_ARG, err);
  lat = fr.lat_p;
  basis = fr.basis_p;
  err = plan_lattice(lat, basis, nbasis, 1e-12, 0u, g);
  if (!err.empty()) return fail(AXX_ERR_INVALID_ARG, err);
  axx_run_params rp{points, 1, 0, 0, 0u, seed, 1e-12, kGammaDefault, 0};
  KernelTables kt;
  err = make_kernel_tables(g, SeqPlan(), 0, 1, AXX_MODE_LATTICE, 0u, kt);
  if (!err.empty()) return fail(AXX_ERR_UNSUPPORTED, err);
  InitSpec init;
  const ArenaLayout L = arena_layout(g, kt, 0);
  const size_t o_cnt = (L.fixed + 255) & ~(size_t)255;
  Buf arena;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e == cudaSuccess) e = cudaMalloc(&arena.p, o_cnt + 256);
  if (e != cudaSuccess) {
    ctx->err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? AXX_ERR_OUT_OF_MEMORY : AXX_ERR_CUDA;
  }
  char *base = (char *)arena.p;
  e = upload_tables(base, L, g, kt, ctx->stream);
  WalkParams P;
  const double cell[3] = {lat->a, lat->b, lat->c};
  fill_walk_params(P, base, L, g, kt, &rp, AXX_MODE_LATTICE, 0, init, cell, nullptr);
  unsigned long long *d_cnt = (unsigned long long *)(base + o_cnt);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_cnt, 0, 8, ctx->stream);
  const int grid = (int)std::max<long long>(
      1, std::min<long long>((points + 255) / 256, (long long)ctx->nsm * 8));
  if (e == cudaSuccess) {
    switch (g.geom) {
      case AXX_GEOM_FREE: e = launch_calcf<AXX_GEOM_FREE>(P, points, d_cnt, grid, ctx->stream); break;
      case AXX_GEOM_CYL: e = launch_calcf<AXX_GEOM_CYL>(P, points, d_cnt, grid, ctx->stream); break;
      case AXX_GEOM_SPH: e = launch_calcf<AXX_GEOM_SPH>(P, points, d_cnt, grid, ctx->stream); break;
      default: e = launch_calcf<AXX_GEOM_MIX>(P, points, d_cnt, grid, ctx->stream); break;
    }
  }
  unsigned long long h = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d_cnt, 8, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    ctx->err = std::string("axx_volume_fraction: ") + cudaGetErrorString(e);
    return AXX_ERR_CUDA;
  }
  if (inside) *inside = (int64_t)h;
  if (fraction) *fraction = (double)h / (double)points;
  return AXX_OK;
}
