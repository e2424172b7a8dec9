// noalloc.cu -- the lattice walk for callers that cannot allocate GPU memory.
//
// Some callers cannot call cudaMalloc at the moment they want a walk: code
// running under a memory pool or budget that owns all device memory, a
// framework that forbids allocation after start-up, or a host thread that
// must not synchronise the device the way cudaMalloc/cudaFree can.  For them
// axx_run_lattice_noalloc runs the same walk and reduction kernels as
// axx_run_lattice, but every device-side buffer of the call (the geometry,
// slot and waveform tables, the per-block FP64 partials, the reduced sums and
// the counters) lives in g_scratch below, a fixed array of kScratchBytes that
// is part of the library image.  Nothing is allocated on the device; the
// host-side planning uses ordinary host memory.
//
// Every GPU that loads this library holds the array until the process exits.
// Host code cannot use g_scratch's name as a device address: the address is
// obtained once per device with cudaGetSymbolAddress (with that device
// current) on the first call on that device, so that first call should come
// before any stream capture.  All calls on a device share the array and it
// keeps the previous call's contents: the counters are cleared at the start
// of every call, everything else is fully rewritten.  Calls whose work
// overlaps on the GPU (two host threads, or two contexts on one device) race
// on the array and must be serialised by the caller.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/axx.h"
#include "ctx_internal.h"
#include "host_plan.h"
#include "walk_launch.h"

namespace {

using namespace axx;

constexpr size_t kScratchBytes = (size_t)AXX_NOALLOC_SCRATCH_BYTES;
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_addr[kMaxDevices] = {};

// Device address of g_scratch on `device` (current on the calling thread).
cudaError_t scratch_address(int device, void **out) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[device]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess) return e;
    g_addr[device] = p;
  }
  *out = g_addr[device];
  return cudaSuccess;
}

axx_status fail(axx_ctx *ctx, axx_status s, const std::string &m) {
  ctx->err = m;
  return s;
}

axx_status cuda_fail(axx_ctx *ctx, cudaError_t e, const char *where) {
  ctx->err = std::string(where) + ": " + cudaGetErrorString(e);
  return AXX_ERR_CUDA;
}

size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }

cudaError_t launch(int geom, int kmax, const WalkParams &P, int grid, size_t smem,
                   cudaStream_t s) {
  TraceParams T{};
  switch (geom) {
    case AXX_GEOM_FREE: return launch_walk_free(kmax, false, P, T, grid, smem, s);
    case AXX_GEOM_CYL: return launch_walk_cyl(kmax, false, P, T, grid, smem, s);
    case AXX_GEOM_SPH: return launch_walk_sph(kmax, false, P, T, grid, smem, s);
    default: return launch_walk_mix(kmax, false, P, T, grid, smem, s);
  }
}

}  // namespace

extern "C" axx_status axx_run_lattice_noalloc(axx_ctx *ctx, const axx_lattice *lat,
                                              const axx_basis *basis, int nbasis,
                                              const axx_sequence *seqs, int nseq,
                                              const axx_run_params *p, double *mx, double *my,
                                              axx_stats *stats) {
  if (!ctx) return AXX_ERR_INVALID_ARG;
  if (!p) return fail(ctx, AXX_ERR_INVALID_ARG, "params is NULL");
  if (p->num_walkers < 1 || p->steps < 1 || !(p->timestep > 0.0) || !std::isfinite(p->timestep) ||
      !std::isfinite(p->gamma) || p->gamma < 0.0 || p->walker_offset < 0 || p->init_mode < 0 ||
      p->init_mode > 2)
    return fail(ctx, AXX_ERR_INVALID_ARG, "invalid run parameters");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaSetDevice");
  void *base_v = nullptr;
  e = scratch_address(ctx->device, &base_v);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaGetSymbolAddress(no-allocation scratch)");
  char *base = (char *)base_v;

  const double gamma = p->gamma > 0.0 ? p->gamma : kGammaDefault;
  GeomPlan g;
  std::string err = plan_lattice(lat, basis, nbasis, p->timestep, p->flags, g);
  if (!err.empty()) return fail(ctx, AXX_ERR_INVALID_ARG, err);
  SeqPlan sq;
  err = plan_sequences(seqs, nseq, p->steps, p->timestep, gamma, sq);
  if (!err.empty()) return fail(ctx, AXX_ERR_INVALID_ARG, err);
  const int K = (int)sq.channels.size();
  if (K > AXX_KMAX) return fail(ctx, AXX_ERR_UNSUPPORTED, "more than 16 phase channels");
  int kmax = 1;
  while (kmax < K) kmax <<= 1;
  int init_inst = 0;
  if (p->init_mode == AXX_INIT_IN_BASIS) {
    if (p->init_arg < 0 || p->init_arg >= nbasis)
      return fail(ctx, AXX_ERR_INVALID_ARG, "init_arg must name a basis for AXX_INIT_IN_BASIS");
    for (int n = 0; n < (int)g.aux.size(); ++n) {
      int slot;
      std::memcpy(&slot, &g.aux[n].z, 4);
      if (slot == p->init_arg) {
        init_inst = n;
        break;
      }
    }
  }
  const int M = nseq, ncell = (int)g.cstart.size() - 1, ninst = (int)g.geo.size();
  const size_t wsum = (size_t)(AXX_BLOCK / 32) * M * 5 * sizeof(double);
  const size_t geo_bytes =
      (size_t)ninst * 32 + (size_t)(ncell + 1) * 4 + ((g.clist.size() * 2 + 15) & ~(size_t)15);
  const bool smem_geom = g.geom != AXX_GEOM_FREE && geo_bytes <= 96 * 1024;
  const size_t smem = wsum + (smem_geom ? geo_bytes : 0);
  const int occ = occupancy_walk(g.geom, kmax, false, smem);
  if (occ <= 0) return fail(ctx, AXX_ERR_CUDA, "walk kernel cannot be resident");
  const long long ntask = (p->num_walkers + 31) / 32;
  const long long want = (ntask + AXX_BLOCK / 32 - 1) / (AXX_BLOCK / 32);
  long long grid = std::min<long long>(want, (long long)occ * ctx->nsm);

  // layout inside the scratch array; the partials shrink the grid if needed
  size_t fixed = 0;
  const size_t o_geo = fixed;
  fixed = up256(fixed + g.geo.size() * 16);
  const size_t o_aux = fixed;
  fixed = up256(fixed + g.aux.size() * 16);
  const size_t o_cs = fixed;
  fixed = up256(fixed + g.cstart.size() * 4);
  const size_t o_cl = fixed;
  fixed = up256(fixed + g.clist.size() * 2);
  const size_t o_slot = fixed;
  fixed = up256(fixed + g.slot_tab.size() * 16);
  const size_t o_reg = fixed;
  fixed = up256(fixed + g.slot_region.size() * 4);
  const size_t o_wave = fixed;
  fixed = up256(fixed + sq.wave.size() * 4);
  const size_t o_coef = fixed;
  fixed = up256(fixed + sq.coef.size() * 8);
  const size_t o_out = fixed;
  fixed = up256(fixed + (size_t)M * 5 * 8);
  const size_t o_cnt = fixed;
  fixed = up256(fixed + AXX_CNT_N * 8);
  const size_t o_part = fixed;
  const size_t per_block = (size_t)M * 5 * 8;
  if (fixed > kScratchBytes ||
      (per_block > 0 && fixed + per_block * std::min<long long>(grid, ctx->nsm) > kScratchBytes)) {
    return fail(ctx, AXX_ERR_INVALID_ARG,
                "this walk needs more than the " + std::to_string(kScratchBytes >> 20) +
                    " MiB no-allocation scratch (tables " + std::to_string(fixed) +
                    " bytes); use axx_run_lattice");
  }
  if (per_block > 0)
    grid = std::min<long long>(grid, (long long)((kScratchBytes - fixed) / per_block));

  cudaStream_t s = ctx->stream;
  auto up = [&](size_t off, const void *src, size_t bytes) {
    return bytes ? cudaMemcpyAsync(base + off, src, bytes, cudaMemcpyHostToDevice, s)
                 : cudaSuccess;
  };
  const cudaError_t ups[] = {up(o_geo, g.geo.data(), g.geo.size() * 16),
                             up(o_aux, g.aux.data(), g.aux.size() * 16),
                             up(o_cs, g.cstart.data(), g.cstart.size() * 4),
                             up(o_cl, g.clist.data(), g.clist.size() * 2),
                             up(o_slot, g.slot_tab.data(), g.slot_tab.size() * 16),
                             up(o_reg, g.slot_region.data(), g.slot_region.size() * 4),
                             up(o_wave, sq.wave.data(), sq.wave.size() * 4),
                             up(o_coef, sq.coef.data(), sq.coef.size() * 8)};
  for (cudaError_t x : ups)
    if (x != cudaSuccess) return cuda_fail(ctx, x, "cudaMemcpyAsync(no-allocation tables)");
  // counters start at zero on every call (the array keeps the last call's values)
  e = cudaMemsetAsync(base + o_cnt, 0, AXX_CNT_N * 8, s);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMemsetAsync(counters)");

  WalkParams P;
  std::memset(&P, 0, sizeof(P));
  P.a = (float)lat->a;
  P.b = (float)lat->b;
  P.c = (float)lat->c;
  P.mode = AXX_MODE_LATTICE;
  P.n_inst = ninst;
  P.n_list = (int)g.clist.size();
  P.ncell = ncell;
  P.smem_geom = smem_geom ? 1 : 0;
  P.inst_geo = (const float4 *)(base + o_geo);
  P.inst_aux = (const float4 *)(base + o_aux);
  P.cell_start = (const uint32_t *)(base + o_cs);
  P.cell_list = (const uint16_t *)(base + o_cl);
  P.gx = g.gx;
  P.gy = g.gy;
  P.gz = g.gz;
  P.inv_hx = g.inv_hx;
  P.inv_hy = g.inv_hy;
  P.inv_hz = g.inv_hz;
  P.slot_tab = (const float4 *)(base + o_slot);
  P.slot_region = (const int *)(base + o_reg);
  P.ecs_slot = g.ecs_slot;
  P.steps = p->steps;
  P.n_walkers = p->num_walkers;
  P.walker_offset = p->walker_offset;
  P.seed_lo = (uint32_t)p->seed;
  P.seed_hi = (uint32_t)(p->seed >> 32);
  P.flags = p->flags;
  P.init_mode = p->init_mode;
  P.init_arg = p->init_arg;
  P.init_inst = init_inst;
  if (p->init_mode == AXX_INIT_IN_BASIS) {
    const axx_basis &b = basis[p->init_arg];
    P.init_sph = b.type == AXX_PRIM_SPHERE;
    P.init_R = (float)b.radius;
    P.init_cx = (float)b.cx;
    P.init_cy = (float)b.cy;
    P.init_cz = (float)b.cz;
  }
  P.K = K;
  P.wave = (const float *)(base + o_wave);
  for (int c = 0; c < K; ++c) {
    P.ch_wave[c] = sq.channels[c].wave;
    for (int k = 0; k < 3; ++k) P.ch_p[c][k] = sq.channels[c].p[k];
  }
  P.M = M;
  P.coef = (const double *)(base + o_coef);
  P.partials = (double *)(base + o_part);
  P.counters = (unsigned long long *)(base + o_cnt);
  P.abort_flag = ctx->abort_dev;
  *ctx->abort_host = 0;
  e = launch(g.geom, kmax, P, (int)grid, smem, s);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "walk kernel launch");
  e = launch_reduce_partials(P.partials, (int)grid, M * 5, (double *)(base + o_out), s);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "reduction launch");

  std::vector<double> h((size_t)M * 5);
  unsigned long long cnt[AXX_CNT_N] = {0};
  if (M > 0) e = cudaMemcpyAsync(h.data(), base + o_out, h.size() * 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(cnt, base + o_cnt, sizeof(cnt), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "reading the no-allocation results");
  for (int m = 0; m < M; ++m) {
    if (mx) mx[m] = h[m * 5 + 0];
    if (my) my[m] = h[m * 5 + 1];
    if (stats) {
      if (stats->sxx) stats->sxx[m] = h[m * 5 + 2];
      if (stats->syy) stats->syy[m] = h[m * 5 + 3];
      if (stats->sxy) stats->sxy[m] = h[m * 5 + 4];
    }
  }
  if (stats) {
    stats->reflection_cap_hits = (int64_t)cnt[AXX_CNT_CAP];
    stats->walker_steps = p->num_walkers * (int64_t)(p->steps - 1);
    stats->boundary_hits = (int64_t)cnt[AXX_CNT_HITS];
  }
  if (cnt[AXX_CNT_ABORTED]) return fail(ctx, AXX_ERR_ABORTED, "run aborted by axx_abort");
  if (cnt[AXX_CNT_INIT_FAIL])
    return fail(ctx, AXX_ERR_INVALID_ARG,
                "start-position rejection sampling found no point in the requested region");
  for (int m = 0; m < M; ++m)
    if (!std::isfinite(h[m * 5]) || !std::isfinite(h[m * 5 + 1]))
      return fail(ctx, AXX_ERR_NUMERIC, "non-finite signal");
  if (cnt[AXX_CNT_CAP])
    return fail(ctx, AXX_ERR_REFLECTION_CAP, "some moves hit the reflection cap of 1024");
  return AXX_OK;
}
