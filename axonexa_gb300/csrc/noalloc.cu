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
// Every GPU that loads this library holds the array until the process exits
// (with lazy module loading the memory is committed when the module first
// loads on that device: at the first call, or at any earlier use of the
// library's kernels).  Host code cannot use g_scratch's name as a device
// address: the address is looked up with cudaGetSymbolAddress, with the
// device current, at the first call in each device context, so that first
// call should come before any stream capture.  A device reset (by the
// caller or by another library) destroys the context and reloads the module,
// which may move the array; the lookup is keyed on the context's id, which
// CUDA never reuses, so the first call after a reset looks the address up
// again.  All calls on a device share the array and it keeps the previous
// call's contents: the counters are cleared at the start of every call,
// everything else is fully rewritten.  Calls whose work overlaps on the GPU
// (two host threads, or two contexts on one device) race on the array and
// must be serialised by the caller.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/axx.h"
#include "ctx_internal.h"
#include "frame.h"
#include "host_plan.h"
#include "plan_layout.h"
#include "walk_launch.h"

namespace {

using namespace axx;

constexpr size_t kScratchBytes = (size_t)AXX_NOALLOC_SCRATCH_BYTES;
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
struct ScratchAddr {
  unsigned long long ctx_id = 0;  // 0: not looked up yet
  void *addr = nullptr;
};
ScratchAddr g_addr[kMaxDevices];

// Id of the context current on this thread (cuCtxGetId, reached through the
// runtime's driver entry points so that the library does not link libcuda).
cudaError_t current_context_id(unsigned long long *id) {
  static PFN_cuCtxGetCurrent_v4000 get_current = nullptr;
  static PFN_cuCtxGetId_v12000 get_id = nullptr;
  if (!get_current || !get_id) {
    cudaDriverEntryPointQueryResult q1, q2;
    void *f1 = nullptr, *f2 = nullptr;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 4000,
                                                     cudaEnableDefault, &q1);
    if (e == cudaSuccess)
      e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
    if (e != cudaSuccess) return e;
    if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
      return cudaErrorNotSupported;
    get_current = (PFN_cuCtxGetCurrent_v4000)f1;
    get_id = (PFN_cuCtxGetId_v12000)f2;
  }
  CUcontext c = nullptr;
  if (get_current(&c) != CUDA_SUCCESS || !c) return cudaErrorInvalidResourceHandle;
  if (get_id(c, id) != CUDA_SUCCESS) return cudaErrorInvalidResourceHandle;
  return cudaSuccess;
}

// Device address of g_scratch on `device` (current on the calling thread),
// looked up once per device context.
cudaError_t scratch_address(int device, void **out) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mu);
  unsigned long long id = 0;
  cudaError_t e = current_context_id(&id);
  if (e != cudaSuccess) return e;
  if (g_addr[device].ctx_id != id) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess) return e;
    g_addr[device].addr = p;
    g_addr[device].ctx_id = id;
  }
  *out = g_addr[device].addr;
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
  Frame fr;
  std::string err = frame_lattice(lat, basis, nbasis, seqs, nseq, fr);
  if (!err.empty()) return fail(ctx, AXX_ERR_INVALID_ARG, err);
  lat = fr.lat_p;
  basis = fr.basis_p;
  seqs = fr.seqs_p;
  SeqPlan sq;
  err = plan_sequences(seqs, nseq, p->steps, p->timestep, gamma, sq);
  if (!err.empty()) return fail(ctx, AXX_ERR_INVALID_ARG, err);
  err = plan_lattice(lat, basis, nbasis, p->timestep, p->flags, g,
                     list_table_budget((int)sq.channels.size()));
  if (!err.empty()) return fail(ctx, AXX_ERR_INVALID_ARG, err);
  const int M = nseq;
  const int Mo = (p->flags & AXX_FLAG_COMPARTMENTS) ? 2 * M : M;  // rows of sums
  // the same layout as axx_run_lattice: per-warp rows of partials, tables
  // beyond the shared-memory budget in global memory (16-channel
  // instantiations)
  const bool rows = true;
  const bool global_tables = walk_smem_bytes(g, Mo, rows) > AXX_SMEM_MAX;
  KernelTables kt;
  err = make_kernel_tables(g, sq, M, p->steps, AXX_MODE_LATTICE, p->flags, kt,
                           global_tables ? AXX_KMAX : 1);
  if (!err.empty()) return fail(ctx, AXX_ERR_UNSUPPORTED, err);
  InitSpec init;
  err = init_spec(g, basis, nbasis, AXX_MODE_LATTICE, p, init);
  if (!err.empty()) return fail(ctx, AXX_ERR_INVALID_ARG, err);
  const size_t smem = global_tables ? walk_sums_bytes(Mo, rows) : walk_smem_bytes(g, Mo, rows);
  if (smem > AXX_SMEM_MAX)
    return fail(ctx, AXX_ERR_UNSUPPORTED, "the sequence sums exceed the shared-memory budget");
  // one instance, one cell, no compartment sums: the single-instance kernels
  const bool one = g.geo.size() == 1 && g.cstart.size() == 2 && !(p->flags & AXX_FLAG_COMPARTMENTS);
  const int occ = occupancy_walk(g.geom, kt.km, kt.kmax, false, one, global_tables, smem);
  if (occ <= 0) return fail(ctx, AXX_ERR_CUDA, "walk kernel cannot be resident");
  const long long ntask = (p->num_walkers + 31) / 32;
  const long long want = (ntask + AXX_BLOCK / 32 - 1) / (AXX_BLOCK / 32);
  long long grid = std::min<long long>(want, (long long)occ * ctx->nsm);

  // layout inside the scratch array; the partials shrink the grid if needed
  const ArenaLayout Lo = arena_layout(g, kt, Mo, rows);
  if (Lo.fixed > kScratchBytes ||
      (Lo.per_block > 0 &&
       Lo.fixed + Lo.per_block * std::min<long long>(grid, ctx->nsm) > kScratchBytes)) {
    return fail(ctx, AXX_ERR_INVALID_ARG,
                "this walk needs more than the " + std::to_string(kScratchBytes >> 20) +
                    " MiB no-allocation scratch (tables " + std::to_string(Lo.fixed) +
                    " bytes); use axx_run_lattice");
  }
  if (Lo.per_block > 0)
    grid = std::min<long long>(grid, (long long)((kScratchBytes - Lo.fixed) / Lo.per_block));

  cudaStream_t s = ctx->stream;
  e = upload_tables(base, Lo, g, kt, s);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMemcpyAsync(no-allocation tables)");
  ctx->h2d_bytes += Lo.upload;
  // counters start at zero on every call (the array keeps the last call's values)
  e = cudaMemsetAsync(base + Lo.o_cnt, 0, AXX_CNT_N * 8, s);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMemsetAsync(counters)");
  WalkParams P;
  const double cell[3] = {lat->a, lat->b, lat->c};
  fill_walk_params(P, base, Lo, g, kt, p, AXX_MODE_LATTICE, M, init, cell, ctx->abort_dev, rows);
  P.global_tables = global_tables ? 1 : 0;
  *ctx->abort_host = 0;
  TraceParams T{};
  e = launch_walk(g.geom, kt.km, kt.kmax, false, P, T, (int)grid, smem, s);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "walk kernel launch");
  e = launch_reduce_partials(P.partials, (int)grid * (AXX_BLOCK / 32), Mo * 5,
                             (double *)(base + Lo.o_out), s);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "reduction launch");
  const size_t o_out = Lo.o_out, o_cnt = Lo.o_cnt;

  std::vector<double> h((size_t)Mo * 5);
  unsigned long long cnt[AXX_CNT_N] = {0};
  if (Mo > 0) e = cudaMemcpyAsync(h.data(), base + o_out, h.size() * 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(cnt, base + o_cnt, sizeof(cnt), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "reading the no-allocation results");
  ctx->d2h_bytes += (Mo > 0 ? h.size() * 8 : 0) + sizeof(cnt);
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
    if (Mo > M) {
      for (int m = 0; m < M; ++m) {
        if (stats->mx_in) stats->mx_in[m] = h[(M + m) * 5 + 0];
        if (stats->my_in) stats->my_in[m] = h[(M + m) * 5 + 1];
      }
      stats->walkers_in = (int64_t)cnt[AXX_CNT_START_IN];
    }
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
