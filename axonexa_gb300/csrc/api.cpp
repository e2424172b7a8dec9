// api.cpp -- the C ABI of include/axx.h over the walk kernels.
//
// A context owns one CUDA stream on one device, eight timing events and a
// host-mapped abort word.  A plan owns one device arena holding every table
// of one walk (geometry, slots, waveforms, coefficients), the per-block FP64
// partials, the reduced sums and the counters; it is built once and launched
// any number of times.  The one-shot calls (axx_run_lattice, axx_run_single)
// build a plan, launch it, read it back and free it, mirroring the
// allocate-copy-run-copy-free sequence of runAcquisitionLattice
// (src/acquisition/phaseAcquisitionStream.cuh:126-190).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/axx.h"
#include "ctx_internal.h"
#include "frame.h"
#include "host_plan.h"
#include "plan_layout.h"
#include "walk_launch.h"

using namespace axx;


struct axx_plan {
  axx_ctx *ctx = nullptr;
  WalkParams P{};
  int geom = 0, km = 0, kmax = 1, grid = 0, M = 0, K = 0, n_inst = 0;
  int Mo = 0;  // rows of sums: M, or 2M with the start-compartment sums
  bool rows = false;  // partials per warp instead of per block
  size_t smem = 0;
  size_t upload_bytes = 0;
  // boundary candidates a move tests, averaged over the cell (walkers are
  // uniform in it): the cell lists' entries per grid cell
  double cand_per_move = 0.0;
  void *arena = nullptr;
  double *out = nullptr;  // [M*5]
  unsigned long long *counters = nullptr;
  long long walker_steps = 0;
  bool launched = false;
  // the walk runs in the frame of arbitrary-axis cylinders: traces are
  // rotated back with R^T
  bool rotated = false;
  double R[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
};

namespace {

axx_status fail(axx_ctx *ctx, axx_status s, const std::string &msg) {
  if (ctx) ctx->err = msg;
  return s;
}

axx_status cuda_fail(axx_ctx *ctx, cudaError_t e, const char *where) {
  if (ctx) ctx->err = std::string(where) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return AXX_ERR_OUT_OF_MEMORY;
  return AXX_ERR_CUDA;
}

#define AXX_CUDA(ctx, call)                                  \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
  } while (0)

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

axx_status check_params(axx_ctx *ctx, const axx_run_params *p) {
  if (!p) return fail(ctx, AXX_ERR_INVALID_ARG, "params is NULL");
  if (p->num_walkers < 1) return fail(ctx, AXX_ERR_INVALID_ARG, "num_walkers must be >= 1");
  if (p->steps < 1) return fail(ctx, AXX_ERR_INVALID_ARG, "steps must be >= 1");
  if (!(p->timestep > 0.0) || !std::isfinite(p->timestep))
    return fail(ctx, AXX_ERR_INVALID_ARG, "timestep must be > 0");
  if (!std::isfinite(p->gamma) || p->gamma < 0.0)
    return fail(ctx, AXX_ERR_INVALID_ARG, "gamma must be finite and >= 0");
  if (p->walker_offset < 0) return fail(ctx, AXX_ERR_INVALID_ARG, "walker_offset must be >= 0");
  if (p->init_mode < 0 || p->init_mode > 2)
    return fail(ctx, AXX_ERR_INVALID_ARG, "unknown init_mode");
  return AXX_OK;
}

// Builds the plan's device arena and kernel parameters.
axx_status build_plan(axx_ctx *ctx, const GeomPlan &g, const SeqPlan &sq, int M,
                      const axx_run_params *p, int mode, const axx_basis *basis, int nbasis,
                      const double cell[3], axx_plan **out) {
  if ((p->flags & AXX_FLAG_COMPARTMENTS) && mode != AXX_MODE_LATTICE)
    return fail(ctx, AXX_ERR_INVALID_ARG, "compartment sums exist for lattice walks only");
  const int Mo = (p->flags & AXX_FLAG_COMPARTMENTS) ? 2 * M : M;
  // the sums go to per-warp rows of the partials in global memory, which
  // leaves the shared memory to the substrate tables; tables that do not fit
  // the shared-memory budget are read from global memory (instantiations with
  // 16 channels)
  const bool rows = true;
  const bool global_tables = walk_smem_bytes(g, Mo, rows) > AXX_SMEM_MAX;
  KernelTables kt;
  std::string err =
      make_kernel_tables(g, sq, M, p->steps, mode, p->flags, kt, global_tables ? AXX_KMAX : 1);
  if (!err.empty()) return fail(ctx, AXX_ERR_UNSUPPORTED, err);
  InitSpec init;
  err = init_spec(g, basis, nbasis, mode, p, init);
  if (!err.empty()) return fail(ctx, AXX_ERR_INVALID_ARG, err);
  const size_t smem = global_tables ? walk_sums_bytes(Mo, rows) : walk_smem_bytes(g, Mo, rows);
  if (smem > AXX_SMEM_MAX)
    return fail(ctx, AXX_ERR_UNSUPPORTED,
                "the sequence sums exceed the shared-memory budget (" + std::to_string(smem) +
                    " bytes)");
  // one instance, one cell, no compartment sums: the single-instance kernels
  const bool one = g.geo.size() == 1 && g.cstart.size() == 2 && !(p->flags & AXX_FLAG_COMPARTMENTS);
  const int occ = occupancy_walk(g.geom, kt.km, kt.kmax, false, one, global_tables, smem);
  if (occ <= 0) return fail(ctx, AXX_ERR_CUDA, "walk kernel cannot be resident (occupancy 0)");
  auto *pl = new axx_plan();
  pl->ctx = ctx;
  pl->geom = g.geom;
  pl->km = kt.km;
  pl->kmax = kt.kmax;
  pl->K = kt.K;
  pl->M = M;
  pl->Mo = Mo;
  pl->n_inst = (int)g.geo.size();
  pl->smem = smem;
  // grid: the device's resident capacity, at most one warp per 32 walkers
  const long long ntask = (p->num_walkers + 31) / 32;
  const long long want = (ntask + AXX_BLOCK / 32 - 1) / (AXX_BLOCK / 32);
  pl->grid = (int)std::min<long long>(want, (long long)occ * ctx->nsm);
  pl->rows = rows;
  const ArenaLayout L = arena_layout(g, kt, Mo, rows);
  pl->upload_bytes = L.upload;
  cudaError_t e = cudaMalloc(&pl->arena, L.fixed + L.per_block * pl->grid);
  if (e != cudaSuccess) {
    delete pl;
    return cuda_fail(ctx, e, "cudaMalloc(plan arena)");
  }
  char *base = (char *)pl->arena;
  e = upload_tables(base, L, g, kt, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    cudaFree(pl->arena);
    delete pl;
    return cuda_fail(ctx, e, "uploading the plan tables");
  }
  ctx->h2d_bytes += L.upload;
  pl->cand_per_move = g.geom == AXX_GEOM_FREE || g.cstart.size() < 2
                          ? 0.0
                          : (double)g.cstart.back() / (double)(g.cstart.size() - 1);
  fill_walk_params(pl->P, base, L, g, kt, p, mode, M, init, cell, ctx->abort_dev, rows);
  pl->P.global_tables = global_tables ? 1 : 0;
  pl->out = (double *)(base + L.o_out);
  pl->counters = pl->P.counters;
  pl->walker_steps = p->num_walkers * (long long)(p->steps - 1);
  *out = pl;
  return AXX_OK;
}

void keep_frame(axx_plan *pl, const Frame &fr) {
  pl->rotated = !fr.identity;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) pl->R[i][j] = fr.R[i][j];
}

axx_status make_lattice_plan(axx_ctx *ctx, const axx_lattice *lat, const axx_basis *basis,
                             int nbasis, const axx_sequence *seqs, int nseq,
                             const axx_run_params *params, axx_plan **out) {
  axx_status s = check_params(ctx, params);
  if (s != AXX_OK) return s;
  const double gamma = params->gamma > 0.0 ? params->gamma : kGammaDefault;
  GeomPlan g;
  Frame fr;
  std::string e = frame_lattice(lat, basis, nbasis, seqs, nseq, fr);
  if (!e.empty()) return fail(ctx, AXX_ERR_INVALID_ARG, e);
  SeqPlan sq;
  e = plan_sequences(fr.seqs_p, nseq, params->steps, params->timestep, gamma, sq);
  if (!e.empty()) return fail(ctx, AXX_ERR_INVALID_ARG, e);
  e = plan_lattice(fr.lat_p, fr.basis_p, nbasis, params->timestep, params->flags, g,
                   list_table_budget((int)sq.channels.size()));
  if (!e.empty()) return fail(ctx, AXX_ERR_INVALID_ARG, e);
  const double cell[3] = {fr.lat_p->a, fr.lat_p->b, fr.lat_p->c};
  s = build_plan(ctx, g, sq, nseq, params, AXX_MODE_LATTICE, fr.basis_p, nbasis, cell, out);
  if (s == AXX_OK) keep_frame(*out, fr);
  return s;
}

axx_status make_single_plan(axx_ctx *ctx, const axx_basis *basis, const axx_sequence *seqs,
                            int nseq, const axx_run_params *params, axx_plan **out) {
  axx_status s = check_params(ctx, params);
  if (s != AXX_OK) return s;
  if (params->flags & (AXX_FLAG_PERMEABLE | AXX_FLAG_RELAXATION))
    return fail(ctx, AXX_ERR_INVALID_ARG,
                "the single-pore walk has no permeability or relaxation (kernelPhase.cuh:4-66)");
  const double gamma = params->gamma > 0.0 ? params->gamma : kGammaDefault;
  GeomPlan g;
  float sp = 0.f, st = 0.f;
  Frame fr;
  std::string e = frame_single(basis, seqs, nseq, fr);
  if (!e.empty()) return fail(ctx, AXX_ERR_INVALID_ARG, e);
  e = plan_single(fr.basis_p, params->timestep, g, sp, st);
  if (!e.empty()) return fail(ctx, AXX_ERR_INVALID_ARG, e);
  SeqPlan sq;
  e = plan_sequences(fr.seqs_p, nseq, params->steps, params->timestep, gamma, sq);
  if (!e.empty()) return fail(ctx, AXX_ERR_INVALID_ARG, e);
  const double cell[3] = {1.0, 1.0, 1.0};
  s = build_plan(ctx, g, sq, nseq, params, AXX_MODE_SINGLE, fr.basis_p, 1, cell, out);
  if (s == AXX_OK) keep_frame(*out, fr);
  return s;
}

axx_status read_results(axx_plan *pl, double *mx, double *my, axx_stats *stats) {
  axx_ctx *ctx = pl->ctx;
  AXX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  std::vector<double> h((size_t)pl->Mo * 5);
  unsigned long long cnt[AXX_CNT_N] = {0};
  if (pl->Mo > 0)
    AXX_CUDA(ctx, cudaMemcpy(h.data(), pl->out, h.size() * 8, cudaMemcpyDeviceToHost));
  AXX_CUDA(ctx, cudaMemcpy(cnt, pl->counters, sizeof(cnt), cudaMemcpyDeviceToHost));
  ctx->d2h_bytes += (pl->Mo > 0 ? h.size() * 8 : 0) + sizeof(cnt);
  for (int m = 0; m < pl->M; ++m) {
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
    stats->walker_steps = pl->walker_steps;
    stats->boundary_hits = (int64_t)cnt[AXX_CNT_HITS];
    if (pl->Mo > pl->M) {
      for (int m = 0; m < pl->M; ++m) {
        if (stats->mx_in) stats->mx_in[m] = h[(pl->M + m) * 5 + 0];
        if (stats->my_in) stats->my_in[m] = h[(pl->M + m) * 5 + 1];
      }
      stats->walkers_in = (int64_t)cnt[AXX_CNT_START_IN];
    }
  }
  if (cnt[AXX_CNT_ABORTED]) return fail(ctx, AXX_ERR_ABORTED, "run aborted by axx_abort");
  if (cnt[AXX_CNT_INIT_FAIL])
    return fail(ctx, AXX_ERR_INVALID_ARG,
                "start-position rejection sampling found no point in the requested region");
  for (int m = 0; m < pl->M; ++m)
    if (!std::isfinite(h[m * 5]) || !std::isfinite(h[m * 5 + 1]))
      return fail(ctx, AXX_ERR_NUMERIC, "non-finite signal");
  if (cnt[AXX_CNT_CAP])
    return fail(ctx, AXX_ERR_REFLECTION_CAP, "some moves hit the reflection cap of 1024");
  return AXX_OK;
}

}  // namespace

extern "C" {

int axx_abi_version(void) { return AXX_ABI_VERSION; }

const char *axx_status_string(axx_status s) {
  switch (s) {
    case AXX_OK: return "ok";
    case AXX_ERR_INVALID_ARG: return "invalid argument";
    case AXX_ERR_CUDA: return "CUDA error";
    case AXX_ERR_REFLECTION_CAP: return "reflection cap hit";
    case AXX_ERR_TIMEOUT: return "timeout";
    case AXX_ERR_NO_DEVICE: return "no CUDA device";
    case AXX_ERR_OUT_OF_MEMORY: return "out of device memory";
    case AXX_ERR_ABORTED: return "aborted";
    case AXX_ERR_UNSUPPORTED: return "unsupported";
    case AXX_ERR_NUMERIC: return "non-finite value";
  }
  return "unknown status";
}

axx_status axx_create(axx_ctx **out, int device) {
  if (!out) return AXX_ERR_INVALID_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return AXX_ERR_NO_DEVICE;
  if (device < 0 || device >= n) return AXX_ERR_INVALID_ARG;
  auto *ctx = new axx_ctx();
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  for (int i = 0; i < 8 && e == cudaSuccess; ++i) e = cudaEventCreate(&ctx->ev[i]);
  cudaDeviceProp prop;
  if (e == cudaSuccess) e = cudaGetDeviceProperties(&prop, device);
  int *h = nullptr;
  if (e == cudaSuccess) e = cudaHostAlloc((void **)&h, sizeof(int), cudaHostAllocMapped);
  if (e == cudaSuccess) {
    *h = 0;
    ctx->abort_host = h;
    e = cudaHostGetDevicePointer((void **)&ctx->abort_dev, h, 0);
  }
  if (e != cudaSuccess) {
    axx_destroy(ctx);
    return AXX_ERR_CUDA;
  }
  ctx->nsm = prop.multiProcessorCount;
  ctx->ccmaj = prop.major;
  ctx->ccmin = prop.minor;
  ctx->gmem = prop.totalGlobalMem;
  *out = ctx;
  return AXX_OK;
}

axx_status axx_destroy(axx_ctx *ctx) {
  if (!ctx) return AXX_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (auto &e : ctx->ev)
    if (e) cudaEventDestroy(e);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  if (ctx->abort_host) cudaFreeHost((void *)ctx->abort_host);
  delete ctx;
  return AXX_OK;
}

const char *axx_last_error(const axx_ctx *ctx) { return ctx ? ctx->err.c_str() : "no context"; }

axx_status axx_device_info(axx_ctx *ctx, int *num_sms, int *cc_major, int *cc_minor,
                           size_t *global_mem_bytes) {
  if (!ctx) return AXX_ERR_INVALID_ARG;
  if (num_sms) *num_sms = ctx->nsm;
  if (cc_major) *cc_major = ctx->ccmaj;
  if (cc_minor) *cc_minor = ctx->ccmin;
  if (global_mem_bytes) *global_mem_bytes = ctx->gmem;
  return AXX_OK;
}

axx_status axx_abort(axx_ctx *ctx) {
  if (!ctx || !ctx->abort_host) return AXX_ERR_INVALID_ARG;
  *ctx->abort_host = 1;
  return AXX_OK;
}

axx_status axx_plan_lattice(axx_ctx *ctx, const axx_lattice *lat, const axx_basis *basis,
                            int nbasis, const axx_sequence *seqs, int nseq,
                            const axx_run_params *params, axx_plan **out) {
  if (!ctx || !out) return AXX_ERR_INVALID_ARG;
  *out = nullptr;
  AXX_CUDA(ctx, cudaSetDevice(ctx->device));
  return make_lattice_plan(ctx, lat, basis, nbasis, seqs, nseq, params, out);
}

axx_status axx_plan_single(axx_ctx *ctx, const axx_basis *basis, const axx_sequence *seqs,
                           int nseq, const axx_run_params *params, axx_plan **out) {
  if (!ctx || !out) return AXX_ERR_INVALID_ARG;
  *out = nullptr;
  AXX_CUDA(ctx, cudaSetDevice(ctx->device));
  return make_single_plan(ctx, basis, seqs, nseq, params, out);
}

axx_status axx_plan_launch(axx_plan *pl) {
  if (!pl) return AXX_ERR_INVALID_ARG;
  axx_ctx *ctx = pl->ctx;
  *ctx->abort_host = 0;
  AXX_CUDA(ctx, cudaMemsetAsync(pl->counters, 0, AXX_CNT_N * 8, ctx->stream));
  TraceParams T{};
  AXX_CUDA(ctx, launch_walk(pl->geom, pl->km, pl->kmax, false, pl->P, T, pl->grid, pl->smem,
                            ctx->stream));
  const int nrows = pl->grid * (pl->rows ? AXX_BLOCK / 32 : 1);
  AXX_CUDA(ctx, launch_reduce_partials(pl->P.partials, nrows, pl->Mo * 5, pl->out, ctx->stream));
  pl->launched = true;
  return AXX_OK;
}

axx_status axx_plan_read(axx_plan *pl, double *mx, double *my, axx_stats *stats) {
  if (!pl) return AXX_ERR_INVALID_ARG;
  if (!pl->launched) return fail(pl->ctx, AXX_ERR_INVALID_ARG, "plan was never launched");
  return read_results(pl, mx, my, stats);
}

axx_status axx_plan_info(const axx_plan *pl, int *channels, int *instances, int *kernel_launches,
                         int64_t *walker_steps) {
  if (!pl) return AXX_ERR_INVALID_ARG;
  if (channels) *channels = pl->K;
  if (instances) *instances = pl->n_inst;
  if (kernel_launches) *kernel_launches = 2;
  if (walker_steps) *walker_steps = pl->walker_steps;
  return AXX_OK;
}

axx_status axx_plan_candidates(const axx_plan *pl, double *per_move) {
  if (!pl || !per_move) return AXX_ERR_INVALID_ARG;
  *per_move = pl->cand_per_move;
  return AXX_OK;
}

axx_status axx_transfer_bytes(axx_ctx *ctx, int64_t *h2d, int64_t *d2h) {
  if (!ctx) return AXX_ERR_INVALID_ARG;
  if (h2d) *h2d = (int64_t)ctx->h2d_bytes;
  if (d2h) *d2h = (int64_t)ctx->d2h_bytes;
  return AXX_OK;
}

axx_status axx_plan_destroy(axx_plan *pl) {
  if (!pl) return AXX_OK;
  cudaStreamSynchronize(pl->ctx->stream);
  cudaFree(pl->arena);
  delete pl;
  return AXX_OK;
}

axx_status axx_event_record(axx_ctx *ctx, int slot) {
  if (!ctx || slot < 0 || slot >= 8) return AXX_ERR_INVALID_ARG;
  AXX_CUDA(ctx, cudaEventRecord(ctx->ev[slot], ctx->stream));
  return AXX_OK;
}

axx_status axx_event_elapsed(axx_ctx *ctx, int a, int b, float *ms) {
  if (!ctx || a < 0 || a >= 8 || b < 0 || b >= 8 || !ms) return AXX_ERR_INVALID_ARG;
  AXX_CUDA(ctx, cudaEventSynchronize(ctx->ev[b]));
  AXX_CUDA(ctx, cudaEventElapsedTime(ms, ctx->ev[a], ctx->ev[b]));
  return AXX_OK;
}

axx_status axx_sync(axx_ctx *ctx) {
  if (!ctx) return AXX_ERR_INVALID_ARG;
  AXX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return AXX_OK;
}

axx_status axx_run_lattice(axx_ctx *ctx, const axx_lattice *lat, const axx_basis *basis,
                           int nbasis, const axx_sequence *seqs, int nseq,
                           const axx_run_params *params, double *mx, double *my,
                           axx_stats *stats) {
  axx_plan *pl = nullptr;
  axx_status s = axx_plan_lattice(ctx, lat, basis, nbasis, seqs, nseq, params, &pl);
  if (s != AXX_OK) return s;
  s = axx_plan_launch(pl);
  if (s == AXX_OK) s = read_results(pl, mx, my, stats);
  axx_plan_destroy(pl);
  return s;
}

axx_status axx_run_single(axx_ctx *ctx, const axx_basis *basis, const axx_sequence *seqs,
                          int nseq, const axx_run_params *params, double *mx, double *my,
                          axx_stats *stats) {
  axx_plan *pl = nullptr;
  axx_status s = axx_plan_single(ctx, basis, seqs, nseq, params, &pl);
  if (s != AXX_OK) return s;
  s = axx_plan_launch(pl);
  if (s == AXX_OK) s = read_results(pl, mx, my, stats);
  axx_plan_destroy(pl);
  return s;
}

axx_status axx_fp32_fma_peak(axx_ctx *ctx, double *fma_per_s) {
  if (!ctx || !fma_per_s) return AXX_ERR_INVALID_ARG;
  AXX_CUDA(ctx, cudaSetDevice(ctx->device));
  float *d = nullptr;
  const int grid = ctx->nsm * 8, block = 256, iters = 4096;
  AXX_CUDA(ctx, cudaMalloc(&d, (size_t)grid * block * sizeof(float)));
  cudaError_t e = launch_fma_peak(grid, block, iters, d, ctx->stream);  // warm-up
  if (e == cudaSuccess) e = cudaEventRecord(ctx->ev[6], ctx->stream);
  for (int r = 0; r < 5 && e == cudaSuccess; ++r) e = launch_fma_peak(grid, block, iters, d, ctx->stream);
  if (e == cudaSuccess) e = cudaEventRecord(ctx->ev[7], ctx->stream);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventSynchronize(ctx->ev[7]);
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ctx->ev[6], ctx->ev[7]);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "axx_fp32_fma_peak");
  *fma_per_s = 5.0 * (double)grid * block * iters * kFmaPerIter / (ms * 1e-3);
  return AXX_OK;
}

axx_status axx_bvalue(const axx_sequence *seq, double gamma, double *b) {
  if (!seq || !b) return AXX_ERR_INVALID_ARG;
  *b = bvalue(*seq, gamma > 0.0 ? gamma : kGammaDefault);
  return AXX_OK;
}

axx_status axx_gradient_eval(const axx_sequence *seq, const double *t, int n, double *out) {
  if (!seq || n < 0 || (n > 0 && (!t || !out))) return AXX_ERR_INVALID_ARG;
  for (int i = 0; i < n; ++i) gradient(*seq, t[i], out + 3 * i);
  return AXX_OK;
}

axx_status axx_philox_words(axx_ctx *ctx, uint64_t seed, uint64_t walker, int n, uint32_t *out) {
  if (!ctx || n < 0 || (n > 0 && !out)) return AXX_ERR_INVALID_ARG;
  if (n == 0) return AXX_OK;
  AXX_CUDA(ctx, cudaSetDevice(ctx->device));
  uint32_t *d = nullptr;
  AXX_CUDA(ctx, cudaMalloc(&d, (size_t)n * 4));
  cudaError_t e = launch_philox_words(seed, walker, n, d, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpy(out, d, (size_t)n * 4, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "axx_philox_words");
  return AXX_OK;
}

static axx_status run_trace(axx_ctx *ctx, axx_plan *pl, int ntrace, float *init_pos, float *pos,
                            int32_t *region, int32_t *hits, int32_t *words) {
  const int steps = pl->P.steps;
  const size_t nrec = (size_t)ntrace * (size_t)std::max(steps - 1, 0);
  void *buf = nullptr;
  const size_t bytes = align256(ntrace * 12) + align256(nrec * 12) + 3 * align256(nrec * 4);
  AXX_CUDA(ctx, cudaMalloc(&buf, bytes));
  char *b = (char *)buf;
  TraceParams T;
  T.ntrace = ntrace;
  T.init_pos = (float *)b;
  b += align256(ntrace * 12);
  T.pos = (float *)b;
  b += align256(nrec * 12);
  T.region = (int32_t *)b;
  b += align256(nrec * 4);
  T.hits = (int32_t *)b;
  b += align256(nrec * 4);
  T.words = (int32_t *)b;
  cudaError_t e = cudaMemsetAsync(pl->counters, 0, AXX_CNT_N * 8, ctx->stream);
  // the plan's grid (its partial rows); warps stride over the walkers
  const int grid = std::min(pl->grid, (ntrace + AXX_BLOCK - 1) / AXX_BLOCK);
  if (e == cudaSuccess)
    e = launch_walk(pl->geom, pl->km, 1, true, pl->P, T, grid, pl->smem, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e == cudaSuccess && init_pos) e = cudaMemcpy(init_pos, T.init_pos, ntrace * 12, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && pos) e = cudaMemcpy(pos, T.pos, nrec * 12, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && region) e = cudaMemcpy(region, T.region, nrec * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && hits) e = cudaMemcpy(hits, T.hits, nrec * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && words) e = cudaMemcpy(words, T.words, nrec * 4, cudaMemcpyDeviceToHost);
  cudaFree(buf);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "trace");
  if (pl->rotated) {
    if (init_pos) frame_to_sim(pl->R, init_pos, (size_t)ntrace);
    if (pos) frame_to_sim(pl->R, pos, nrec);
  }
  return AXX_OK;
}

axx_status axx_trace_lattice(axx_ctx *ctx, const axx_lattice *lat, const axx_basis *basis,
                             int nbasis, const axx_run_params *params, int ntrace,
                             float *init_pos, float *pos, int32_t *region, int32_t *hits,
                             int32_t *words) {
  if (!ctx || !params || ntrace < 1) return AXX_ERR_INVALID_ARG;
  axx_run_params p = *params;
  p.num_walkers = ntrace;
  axx_plan *pl = nullptr;
  axx_status s = axx_plan_lattice(ctx, lat, basis, nbasis, nullptr, 0, &p, &pl);
  if (s != AXX_OK) return s;
  s = run_trace(ctx, pl, ntrace, init_pos, pos, region, hits, words);
  axx_plan_destroy(pl);
  return s;
}

axx_status axx_trace_single(axx_ctx *ctx, const axx_basis *basis, const axx_run_params *params,
                            int ntrace, float *init_pos, float *pos, int32_t *region,
                            int32_t *hits, int32_t *words) {
  if (!ctx || !params || ntrace < 1) return AXX_ERR_INVALID_ARG;
  axx_run_params p = *params;
  p.num_walkers = ntrace;
  axx_plan *pl = nullptr;
  axx_status s = axx_plan_single(ctx, basis, nullptr, 0, &p, &pl);
  if (s != AXX_OK) return s;
  s = run_trace(ctx, pl, ntrace, init_pos, pos, region, hits, words);
  axx_plan_destroy(pl);
  return s;
}

}  // extern "C"
