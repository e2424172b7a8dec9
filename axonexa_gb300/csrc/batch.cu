// batch.cu -- many acquisitions (substrates x sequences, uneven walker
// counts) in one persistent launch, replayed from a captured CUDA graph, with
// the launch shape chosen by the project's autotuner.
//
// The reference runs acquisitions one after another, two streams per device
// (phaseAcquisitionStream::runAcquisitionStreamLattice / runAcquisitionStream,
// src/acquisition/phaseAcquisitionStream.cuh:254-613).  Here every job's
// tables are uploaded once; each job's walker range is cut into work items of
// `tile` walkers; the items, longest (walkers x steps) first, are taken by
// resident blocks from one atomic counter.  A block stages the job's walk
// parameters and substrate in shared memory when its item belongs to a new
// job, walks the item with the same per-walker code as the single-job kernel
// (walk_one: identical trajectories), and writes the item's FP64 partial sums
// to the item's fixed slot; batch_reduce_kernel then adds each job's item
// partials in item order, so results do not depend on which block ran which
// item.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include <sys/stat.h>

#include "../../include/axx.h"
#include "ctx_internal.h"
#include "frame.h"
#include "host_plan.h"
#include "plan_layout.h"
#include "walk_kernel.cuh"

namespace axx {

constexpr int kBatchMaxSeq = 64;  // sequences per job (shared-memory sums)

struct BatchJob {
  WalkParams P;       // tables point into the batch arena
  int one;            // single-instance path
  int M;
  long long part_off; // first partial (in doubles) of this job's items
  long long out_off;  // first output (in doubles) of this job
};

struct BatchItem {
  int job;
  int local;          // item index within its job (its partial slot)
  long long first;    // first walker id of the job
  int count;          // walkers in the item
  int pad;
};

// Job classes: each runs its own instantiation of the batch kernel, compiled
// for the geometry and walk of its jobs alone (fewer code paths, so fewer
// registers) at the channel capacity of its own jobs.
enum { BC_SCYL = 0,  // single cylinder pores
       BC_SSPH = 1,  // single sphere pores
       BC_LCYL = 2,  // permeable lattices of cylinders along z
       BC_LMIX = 3,  // other lattices (spheres, mixed types, planes)
       BC_LCYI = 4,  // impermeable lattices of cylinders along z
       BC_N = 5 };

// Resident blocks per SM the register budget targets: single pores as the
// single-instance walk kernels; lattices one block fewer than the list walks
// from eight channels up (the job switching and the staged parameters cost
// registers the list walk spills without).
constexpr int batch_min_blocks(int kmax, int cls) {
  return (cls <= BC_SSPH && kmax <= 4) ? AXX_MIN_BLOCKS + 1
         : (cls >= BC_LCYL && kmax >= 8) ? 5
                                         : AXX_MIN_BLOCKS_FOR(kmax);
}

// Table budget of a lattice job's plan (the finer cell grids of the list
// walk, which leave fewer candidates per move): the shared memory of one
// block at the lattice classes' minimum resident blocks for the job's
// channels (228 KB per SM, 1 KB of it reserved per block), less the staged
// parameters, the per-warp sums and the slot table.
static size_t batch_list_budget(int channels, int nbasis) {
  int k = 1;
  while (k < channels) k <<= 1;
  const size_t per_block = (size_t)228 * 1024 / batch_min_blocks(k, BC_LCYL) - 1024;
  const size_t fixed = ((sizeof(WalkParams) + 15) & ~(size_t)15) +
                       (size_t)(AXX_BLOCK / 32) * kBatchMaxSeq * 5 * sizeof(double) +
                       (size_t)(nbasis + 2) * 20;
  return per_block > fixed ? per_block - fixed : 0;
}

template <int KMAX, int CLS>
__global__ void __launch_bounds__(AXX_BLOCK, batch_min_blocks(KMAX, CLS))
    batch_kernel(const BatchJob *__restrict__ jobs, const BatchItem *__restrict__ items,
                 int nitems, unsigned *item_counter, double *partials) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int warps = AXX_BLOCK / 32;
  WalkParams &sP = *reinterpret_cast<WalkParams *>(smem);
  constexpr size_t p_bytes = (sizeof(WalkParams) + 15) & ~(size_t)15;
  double *wsum = reinterpret_cast<double *>(smem + p_bytes);
  unsigned char *geo_base = smem + p_bytes + (size_t)warps * kBatchMaxSeq * 5 * sizeof(double);
  __shared__ int s_item;
  __shared__ int s_one;
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int cur = -1;
  TraceParams T{};
  SmemView S;
  for (;;) {
    if (threadIdx.x == 0) s_item = (int)atomicAdd(item_counter, 1u);
    __syncthreads();
    const int it = s_item;
    if (it >= nitems) break;
    const BatchItem item = items[it];
    if (item.job != cur) {
      // stage the job's parameters and substrate tables
      const int *src = reinterpret_cast<const int *>(&jobs[item.job].P);
      int *dst = reinterpret_cast<int *>(smem);
      for (int j = threadIdx.x; j < (int)(sizeof(WalkParams) / 4); j += blockDim.x) dst[j] = src[j];
      if (threadIdx.x == 0) {
        s_one = jobs[item.job].one;
      }
      __syncthreads();
      float4 *sg = reinterpret_cast<float4 *>(geo_base);
      float4 *sa = sg + sP.n_inst;
      float4 *ss = sa + sP.n_inst;
      uint32_t *sc = reinterpret_cast<uint32_t *>(ss + sP.n_slot);
      int *sr = reinterpret_cast<int *>(sc + sP.ncell + 1);
      uint16_t *sl = reinterpret_cast<uint16_t *>(sr + sP.n_slot);
      for (int j = threadIdx.x; j < sP.n_inst; j += blockDim.x) {
        sg[j] = sP.inst_geo[j];
        sa[j] = sP.inst_aux[j];
      }
      for (int j = threadIdx.x; j < sP.n_slot; j += blockDim.x) {
        ss[j] = sP.slot_tab[j];
        sr[j] = sP.slot_region[j];
      }
      for (int j = threadIdx.x; j <= sP.ncell; j += blockDim.x) sc[j] = sP.cell_start[j];
      for (int j = threadIdx.x; j < sP.n_list; j += blockDim.x) sl[j] = sP.cell_list[j];
      S.geo = sg;
      S.aux = sa;
      S.slot = ss;
      S.cstart = sc;
      S.region = sr;
      S.clist = sl;
      cur = item.job;
    }
    const int M = sP.M;
    for (int j = threadIdx.x; j < warps * M * 5; j += blockDim.x) wsum[j] = 0.0;
    __syncthreads();
    const bool one = s_one != 0;
    const int ntask = (item.count + 31) / 32;
    unsigned caps = 0, hits = 0, init_fail = 0, aborted = 0;
    for (int task = wib; task < ntask; task += warps) {
      const int off = task * 32 + lane;
      const bool active = off < item.count;
      const long long wid = item.first + off;
      Walker<KMAX> W;
#pragma unroll
      for (int c = 0; c < KMAX; ++c) W.acc[c] = W.cmp[c] = 0.0f;
      W.t2s = W.t2c = 0.0f;
      if (active) {
        WalkResult r{0u, 0u, false, false};
        if constexpr (CLS == BC_SCYL) {
          r = walk_one<AXX_GEOM_CYL, KMAX, AXX_KM_SINGLE, false, true>(sP, S, T, wid, W);
        } else if constexpr (CLS == BC_SSPH) {
          r = walk_one<AXX_GEOM_SPH, KMAX, AXX_KM_SINGLE, false, true>(sP, S, T, wid, W);
        } else if constexpr (CLS == BC_LCYL || CLS == BC_LCYI) {
          // the single-instance walk up to four channels (as the single-job
          // kernels), the list walk otherwise and above; permeable and
          // impermeable lattices are separate classes, so that each kernel
          // holds one walk (the two together spilled 148 bytes at eight
          // channels, the permeable walk alone 32)
          constexpr bool one_ok = KMAX <= 4;
          constexpr int km = CLS == BC_LCYL ? AXX_KM_LAT_PERM : AXX_KM_LAT_IMP;
          r = (one_ok && one) ? walk_one<AXX_GEOM_CYL, KMAX, km, false, one_ok>(sP, S, T, wid, W)
                              : walk_one<AXX_GEOM_CYL, KMAX, km, false, false>(sP, S, T, wid, W);
        } else {
          // other lattices: the mixed-type walk (single instance or list)
          if (sP.km == AXX_KM_LAT_PERM) {
            r = one ? walk_one<AXX_GEOM_MIX, KMAX, AXX_KM_LAT_PERM, false, true>(sP, S, T, wid, W)
                    : walk_one<AXX_GEOM_MIX, KMAX, AXX_KM_LAT_PERM, false, false>(sP, S, T, wid, W);
          } else {
            r = one ? walk_one<AXX_GEOM_MIX, KMAX, AXX_KM_LAT_IMP, false, true>(sP, S, T, wid, W)
                    : walk_one<AXX_GEOM_MIX, KMAX, AXX_KM_LAT_IMP, false, false>(sP, S, T, wid, W);
          }
        }
        caps += r.caps;
        hits += r.hits;
        init_fail += r.init_fail ? 1u : 0u;
        aborted += r.aborted ? 1u : 0u;
      }
      double ph[KMAX];
#pragma unroll
      for (int c = 0; c < KMAX; ++c) ph[c] = (double)W.acc[c] - (double)W.cmp[c];
      const double w = exp(-((double)W.t2s - (double)W.t2c));
      for (int m = 0; m < M; ++m) {
        double ang = 0.0;
#pragma unroll
        for (int c = 0; c < KMAX; ++c) ang = fma(sP.coef[m * KMAX + c], ph[c], ang);
        double sn, cs;
        sincos(ang, &sn, &cs);
        const double xv = active ? cs * w : 0.0, yv = active ? sn * w : 0.0;
        const double s0 = warp_sum(xv), s1 = warp_sum(yv), s2 = warp_sum(xv * xv),
                     s3 = warp_sum(yv * yv), s4 = warp_sum(xv * yv);
        if (lane == 0) {
          double *d = wsum + ((size_t)wib * M + m) * 5;
          d[0] += s0;
          d[1] += s1;
          d[2] += s2;
          d[3] += s3;
          d[4] += s4;
        }
      }
    }
    if (caps) atomicAdd(&sP.counters[AXX_CNT_CAP], (unsigned long long)caps);
    if (hits) atomicAdd(&sP.counters[AXX_CNT_HITS], (unsigned long long)hits);
    if (init_fail) atomicAdd(&sP.counters[AXX_CNT_INIT_FAIL], (unsigned long long)init_fail);
    if (aborted) atomicAdd(&sP.counters[AXX_CNT_ABORTED], (unsigned long long)aborted);
    __syncthreads();
    double *dst = partials + jobs[item.job].part_off + (long long)item.local * M * 5;
    for (int j = threadIdx.x; j < M * 5; j += blockDim.x) {
      double s = 0.0;
      for (int q = 0; q < warps; ++q) s += wsum[(size_t)q * M * 5 + j];
      dst[j] = s;
    }
    __syncthreads();
  }
}

// out[o] for output o = (job j, index within the job) sums the job's item
// partials in item order.
__global__ void __launch_bounds__(256)
    batch_reduce_kernel(const BatchJob *__restrict__ jobs, const int2 *__restrict__ out_map,
                        const int *__restrict__ job_items, const double *__restrict__ partials,
                        double *__restrict__ out) {
  __shared__ double red[256];
  const int o = blockIdx.x;
  const int2 jm = out_map[o];
  const BatchJob &J = jobs[jm.x];
  const int n = job_items[jm.x];
  const int stride = J.M * 5;
  double s = 0.0;
  for (int t = threadIdx.x; t < n; t += blockDim.x) s += partials[J.part_off + (long long)t * stride + jm.y];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[J.out_off + jm.y] = red[0];
}

template <int KMAX, int CLS>
static cudaError_t batch_prepare(size_t smem) {
  if (smem > 48 * 1024)
    return cudaFuncSetAttribute(batch_kernel<KMAX, CLS>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  return cudaSuccess;
}

template <int KMAX, int CLS>
static int batch_occ(size_t smem) {
  if (batch_prepare<KMAX, CLS>(smem) != cudaSuccess) return 0;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_kernel<KMAX, CLS>, AXX_BLOCK,
                                                    smem) != cudaSuccess)
    return 0;
  return n;
}

template <int CLS>
static cudaError_t batch_go_cls(int kmax, int grid, size_t smem, cudaStream_t s,
                                const BatchJob *jobs, const BatchItem *items, int nitems,
                                unsigned *ctr, double *part) {
  switch (kmax) {
    case 1: batch_kernel<1, CLS><<<grid, AXX_BLOCK, smem, s>>>(jobs, items, nitems, ctr, part); break;
    case 2: batch_kernel<2, CLS><<<grid, AXX_BLOCK, smem, s>>>(jobs, items, nitems, ctr, part); break;
    case 4: batch_kernel<4, CLS><<<grid, AXX_BLOCK, smem, s>>>(jobs, items, nitems, ctr, part); break;
    case 8: batch_kernel<8, CLS><<<grid, AXX_BLOCK, smem, s>>>(jobs, items, nitems, ctr, part); break;
    default: batch_kernel<16, CLS><<<grid, AXX_BLOCK, smem, s>>>(jobs, items, nitems, ctr, part); break;
  }
  return cudaGetLastError();
}

static cudaError_t batch_go(int cls, int kmax, int grid, size_t smem, cudaStream_t s,
                            const BatchJob *jobs, const BatchItem *items, int nitems,
                            unsigned *ctr, double *part) {
  switch (cls) {
    case BC_SCYL: return batch_go_cls<BC_SCYL>(kmax, grid, smem, s, jobs, items, nitems, ctr, part);
    case BC_SSPH: return batch_go_cls<BC_SSPH>(kmax, grid, smem, s, jobs, items, nitems, ctr, part);
    case BC_LCYL: return batch_go_cls<BC_LCYL>(kmax, grid, smem, s, jobs, items, nitems, ctr, part);
    case BC_LCYI: return batch_go_cls<BC_LCYI>(kmax, grid, smem, s, jobs, items, nitems, ctr, part);
    default: return batch_go_cls<BC_LMIX>(kmax, grid, smem, s, jobs, items, nitems, ctr, part);
  }
}

template <int CLS>
static int batch_occupancy_cls(int kmax, size_t smem) {
  switch (kmax) {
    case 1: return batch_occ<1, CLS>(smem);
    case 2: return batch_occ<2, CLS>(smem);
    case 4: return batch_occ<4, CLS>(smem);
    case 8: return batch_occ<8, CLS>(smem);
    default: return batch_occ<16, CLS>(smem);
  }
}

static int batch_occupancy(int cls, int kmax, size_t smem) {
  switch (cls) {
    case BC_SCYL: return batch_occupancy_cls<BC_SCYL>(kmax, smem);
    case BC_SSPH: return batch_occupancy_cls<BC_SSPH>(kmax, smem);
    case BC_LCYL: return batch_occupancy_cls<BC_LCYL>(kmax, smem);
    case BC_LCYI: return batch_occupancy_cls<BC_LCYI>(kmax, smem);
    default: return batch_occupancy_cls<BC_LMIX>(kmax, smem);
  }
}

}  // namespace axx

using namespace axx;

struct axx_batch {
  axx_ctx *ctx = nullptr;
  int njobs = 0, nitems = 0, kmax = 1, tile = 0, bps = 0, grid = 0, nout = 0;
  size_t smem = 0;
  // per job class (BC_*): its channel capacity, shared memory, grid, item
  // range, resident blocks per SM; classes without items are skipped
  int c_kmax[BC_N] = {}, c_grid[BC_N] = {}, c_first[BC_N] = {}, c_items[BC_N] = {},
      c_bps[BC_N] = {};
  size_t c_smem[BC_N] = {};
  // the classes run concurrently: forked from the context stream onto these
  cudaStream_t cs[BC_N] = {};
  cudaEvent_t fork = nullptr, join[BC_N] = {};
  void *arena = nullptr;
  BatchJob *d_jobs = nullptr;
  BatchItem *d_items = nullptr;
  int2 *d_outmap = nullptr;
  int *d_jobitems = nullptr;
  unsigned *d_ctr = nullptr;
  double *d_part = nullptr, *d_out = nullptr;
  unsigned long long *d_counters = nullptr;
  std::vector<int> job_M;
  std::vector<long long> job_ws;
  long long walker_steps = 0;
  bool use_graph = false;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool launched = false;
};

namespace {

axx_status bfail(axx_ctx *ctx, axx_status s, const std::string &m) {
  if (ctx) ctx->err = m;
  return s;
}

axx_status bcuda(axx_ctx *ctx, cudaError_t e, const char *where) {
  if (ctx) ctx->err = std::string(where) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? AXX_ERR_OUT_OF_MEMORY : AXX_ERR_CUDA;
}

size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }

uint64_t fnv(uint64_t h, uint64_t v) {
  for (int i = 0; i < 8; ++i) {
    h ^= (v >> (8 * i)) & 0xffu;
    h *= 1099511628211ull;
  }
  return h;
}

// Shape of a batch for the tuning cache.
// The batch's shape for the autotuner's cache: per job its mode, walkers,
// steps, flags and timestep, its substrate (cell, basis types and radii:
// instances, grid lists and hit rates follow from them) and its sequences'
// waveforms and directions (the channel capacity follows from them; the
// amplitudes G do not change the cost).
uint64_t batch_shape(const axx_job *jobs, int njobs) {
  auto bits = [](double v) {
    uint64_t u;
    std::memcpy(&u, &v, 8);
    return u;
  };
  uint64_t h = 1469598103934665603ull;
  h = fnv(h, (uint64_t)njobs);
  for (int j = 0; j < njobs; ++j) {
    const axx_job &J = jobs[j];
    h = fnv(h, (uint64_t)J.mode);
    h = fnv(h, (uint64_t)J.params.num_walkers);
    h = fnv(h, (uint64_t)J.params.steps);
    h = fnv(h, (uint64_t)J.nbasis);
    h = fnv(h, (uint64_t)J.nseq);
    h = fnv(h, (uint64_t)J.params.flags);
    h = fnv(h, bits(J.params.timestep));
    if (J.mode == 0) {
      h = fnv(h, bits(J.lattice.a));
      h = fnv(h, bits(J.lattice.b));
      h = fnv(h, bits(J.lattice.c));
    }
    for (int k = 0; k < J.nbasis && J.basis; ++k) {
      h = fnv(h, (uint64_t)J.basis[k].type);
      h = fnv(h, bits(J.basis[k].radius));
    }
    for (int m = 0; m < J.nseq && J.seqs; ++m) {
      const axx_sequence &q = J.seqs[m];
      h = fnv(h, (uint64_t)q.kind);
      h = fnv(h, (uint64_t)q.num_periods);
      h = fnv(h, bits(q.duration));
      h = fnv(h, bits(q.spacing));
      h = fnv(h, bits(q.gx));
      h = fnv(h, bits(q.gy));
      h = fnv(h, bits(q.gz));
    }
  }
  return h;
}

std::string cache_path() {
  const char *e = std::getenv("AXX_AUTOTUNE_CACHE");
  if (e && *e) return e;
  const char *home = std::getenv("HOME");
  return std::string(home ? home : ".") + "/.cache/axonexa_gb300/autotune.tsv";
}

std::string device_key(axx_ctx *ctx) {
  cudaDeviceProp p;
  if (cudaGetDeviceProperties(&p, ctx->device) != cudaSuccess) return "unknown";
  std::string n = p.name;
  for (char &c : n)
    if (c == ' ' || c == '\t') c = '_';
  return n + "_sm" + std::to_string(p.major) + std::to_string(p.minor);
}

std::mutex g_cache_mu;

bool cache_lookup(axx_ctx *ctx, uint64_t shape, axx_batch_options &o) {
  std::lock_guard<std::mutex> lock(g_cache_mu);
  std::ifstream f(cache_path());
  if (!f) return false;
  const std::string dev = device_key(ctx);
  std::string line;
  bool found = false;
  while (std::getline(f, line)) {
    std::istringstream ss(line);
    std::string d;
    unsigned long long h;
    int tile, bps;
    double ms;
    if (ss >> d >> h >> tile >> bps >> ms && d == dev && h == shape) {
      o.tile = tile;
      o.blocks_per_sm = bps;
      found = true;
    }
  }
  return found;
}

// mkdir -p of the directory part of `path`
void make_parent_dirs(const std::string &path) {
  for (size_t i = 1; i < path.size(); ++i)
    if (path[i] == '/') ::mkdir(path.substr(0, i).c_str(), 0755);
}

void cache_store(axx_ctx *ctx, uint64_t shape, const axx_batch_options &o, double ms) {
  std::lock_guard<std::mutex> lock(g_cache_mu);
  const std::string path = cache_path();
  make_parent_dirs(path);
  std::ofstream f(path, std::ios::app);
  if (f)
    f << device_key(ctx) << '\t' << (unsigned long long)shape << '\t' << o.tile << '\t'
      << o.blocks_per_sm << '\t' << ms << '\n';
}

}  // namespace

static axx_status batch_build(axx_ctx *ctx, const axx_job *jobs, int njobs,
                              const axx_batch_options &opt, int steps_cap, axx_batch **out);

extern "C" axx_status axx_autotune_batch(axx_ctx *ctx, const axx_job *jobs, int njobs,
                                         int probe_steps, axx_batch_options *best,
                                         double *best_ms) {
  if (!ctx || !jobs || njobs < 1 || !best) return AXX_ERR_INVALID_ARG;
  if (probe_steps < 2) probe_steps = 300;
  const int tiles[] = {256, 512, 1024, 2048, 4096, 8192};
  double bms = 1e300;
  axx_batch_options bo{0, 0, 0};
  for (int tile : tiles) {
    for (int bsel = 0; bsel < 2; ++bsel) {
      axx_batch_options o{tile, bsel == 0 ? 0 : -2, 0};
      axx_batch *b = nullptr;
      axx_status s = batch_build(ctx, jobs, njobs, o, probe_steps, &b);
      if (s != AXX_OK) return s;
      if (bsel == 1 && b->bps <= 1) {
        axx_batch_destroy(b);
        continue;
      }
      double ms = 1e300;
      for (int r = 0; r < 3 && s == AXX_OK; ++r) {
        cudaEventRecord(ctx->ev[6], ctx->stream);
        s = axx_batch_launch(b);
        cudaEventRecord(ctx->ev[7], ctx->stream);
        cudaEventSynchronize(ctx->ev[7]);
        float t = 0.f;
        cudaEventElapsedTime(&t, ctx->ev[6], ctx->ev[7]);
        if (r > 0) ms = std::min(ms, (double)t);
      }
      const int bps_used = b->bps;
      axx_batch_destroy(b);
      if (s != AXX_OK) return s;
      if (ms < bms) {
        bms = ms;
        bo = axx_batch_options{tile, bps_used, 0};
      }
    }
  }
  *best = bo;
  if (best_ms) *best_ms = bms;
  cache_store(ctx, batch_shape(jobs, njobs), bo, bms);
  return AXX_OK;
}

// The batch's work on stream s: counters reset, the class kernels forked onto
// their streams (they run concurrently, each over its own items) and joined
// back, then the per-job reduction.
static cudaError_t batch_enqueue(axx_batch *b, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(b->d_ctr, 0, 16, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->d_counters, 0, 8 * AXX_CNT_N * b->njobs, s);
  if (e == cudaSuccess) e = cudaEventRecord(b->fork, s);
  for (int c = 0; c < BC_N && e == cudaSuccess; ++c) {
    if (b->c_items[c] == 0) continue;
    e = cudaStreamWaitEvent(b->cs[c], b->fork, 0);
    if (e == cudaSuccess)
      e = batch_go(c, b->c_kmax[c], b->c_grid[c], b->c_smem[c], b->cs[c], b->d_jobs,
                   b->d_items + b->c_first[c], b->c_items[c], b->d_ctr + c, b->d_part);
    if (e == cudaSuccess) e = cudaEventRecord(b->join[c], b->cs[c]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, b->join[c], 0);
  }
  if (e == cudaSuccess && b->nout > 0) {
    batch_reduce_kernel<<<b->nout, 256, 0, s>>>(b->d_jobs, b->d_outmap, b->d_jobitems, b->d_part,
                                                b->d_out);
    e = cudaGetLastError();
  }
  return e;
}

static axx_status batch_build(axx_ctx *ctx, const axx_job *jobs, int njobs,
                              const axx_batch_options &opt, int steps_cap, axx_batch **out) {
  *out = nullptr;
  if (njobs < 1) return bfail(ctx, AXX_ERR_INVALID_ARG, "njobs must be >= 1");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return bcuda(ctx, e, "cudaSetDevice");
  struct JobPlan {
    GeomPlan g;
    SeqPlan sq;
    KernelTables kt;
    InitSpec init;
    axx_run_params p;
    int mode;
    int cls;  // BC_*
    double cell[3];
    Frame f;  // arbitrary-axis cylinders: the job in the cylinders' frame
  };
  std::vector<JobPlan> jp(njobs);
  int kmax = 1;
  int ckmax[BC_N] = {1, 1, 1, 1, 1};
  for (int j = 0; j < njobs; ++j) {
    const axx_job &J = jobs[j];
    JobPlan &q = jp[j];
    q.p = J.params;
    if (steps_cap > 0 && q.p.steps > steps_cap) q.p.steps = steps_cap;
    q.mode = J.mode;
    const axx_run_params &p = q.p;
    if (p.num_walkers < 1 || p.steps < 1 || !(p.timestep > 0.0) || p.walker_offset < 0 ||
        p.init_mode < 0 || p.init_mode > 2 || !std::isfinite(p.gamma) || p.gamma < 0.0)
      return bfail(ctx, AXX_ERR_INVALID_ARG, "job " + std::to_string(j) + ": invalid run parameters");
    if (p.flags & AXX_FLAG_SIMPLE_REJECTION)
      return bfail(ctx, AXX_ERR_UNSUPPORTED, "batched jobs use specular reflection");
    if (p.flags & AXX_FLAG_COMPARTMENTS)
      return bfail(ctx, AXX_ERR_UNSUPPORTED, "batched jobs return whole-substrate sums only");
    if (J.nseq > kBatchMaxSeq)
      return bfail(ctx, AXX_ERR_INVALID_ARG, "a batched job has at most 64 sequences");
    const double gamma = p.gamma > 0.0 ? p.gamma : kGammaDefault;
    std::string err;
    if (J.mode == AXX_MODE_SINGLE) {
      if (p.flags & (AXX_FLAG_PERMEABLE | AXX_FLAG_RELAXATION))
        return bfail(ctx, AXX_ERR_INVALID_ARG, "single-pore jobs have no permeability or relaxation");
      float sp, st;
      err = frame_single(J.basis, J.seqs, J.nseq, q.f);
      if (err.empty()) err = plan_single(q.f.basis_p, p.timestep, q.g, sp, st);
      q.cell[0] = q.cell[1] = q.cell[2] = 1.0;
    } else {
      err = frame_lattice(&J.lattice, J.basis, J.nbasis, J.seqs, J.nseq, q.f);
      if (err.empty()) err = plan_sequences(q.f.seqs_p, J.nseq, p.steps, p.timestep, gamma, q.sq);
      if (err.empty())
        err = plan_lattice(q.f.lat_p, q.f.basis_p, J.nbasis, p.timestep, p.flags, q.g,
                           batch_list_budget((int)q.sq.channels.size(), J.nbasis));
      if (err.empty()) {
        q.cell[0] = q.f.lat_p->a;
        q.cell[1] = q.f.lat_p->b;
        q.cell[2] = q.f.lat_p->c;
      }
    }
    if (err.empty() && J.mode == AXX_MODE_SINGLE)
      err = plan_sequences(q.f.seqs_p, J.nseq, p.steps, p.timestep, gamma, q.sq);
    if (!err.empty()) return bfail(ctx, AXX_ERR_INVALID_ARG, "job " + std::to_string(j) + ": " + err);
    if (J.mode == AXX_MODE_SINGLE)
      q.cls = q.g.geom == AXX_GEOM_SPH ? BC_SSPH : BC_SCYL;
    else if (q.g.geom == AXX_GEOM_CYL)
      q.cls = walk_mode(J.mode, q.g.geom, p.flags) == AXX_KM_LAT_PERM ? BC_LCYL : BC_LCYI;
    else
      q.cls = BC_LMIX;
    int k = 1;
    while (k < (int)q.sq.channels.size()) k <<= 1;
    kmax = std::max(kmax, k);
    ckmax[q.cls] = std::max(ckmax[q.cls], k);
  }
  if (kmax > AXX_KMAX) return bfail(ctx, AXX_ERR_UNSUPPORTED, "more than 16 channels in a job");
  size_t geo_max[BC_N] = {};
  std::vector<size_t> job_off(njobs);
  size_t off = 0;
  for (int j = 0; j < njobs; ++j) {
    JobPlan &q = jp[j];
    std::string err = make_kernel_tables(q.g, q.sq, jobs[j].nseq, q.p.steps, q.mode, q.p.flags,
                                         q.kt, ckmax[q.cls]);
    if (err.empty()) err = init_spec(q.g, q.f.basis_p, jobs[j].nbasis, q.mode, &q.p, q.init);
    if (!err.empty()) return bfail(ctx, AXX_ERR_INVALID_ARG, "job " + std::to_string(j) + ": " + err);
    geo_max[q.cls] = std::max(geo_max[q.cls], batch_table_bytes(q.g));
    job_off[j] = off;
    off = up256(off + arena_layout(q.g, q.kt, jobs[j].nseq).fixed);
  }
  const size_t p_bytes = (sizeof(WalkParams) + 15) & ~(size_t)15;
  size_t csmem[BC_N] = {};
  size_t smem = 0;
  for (int c = 0; c < BC_N; ++c) {
    csmem[c] = p_bytes + (size_t)(AXX_BLOCK / 32) * kBatchMaxSeq * 5 * 8 + geo_max[c];
    smem = std::max(smem, csmem[c]);
  }
  if (smem > AXX_SMEM_MAX) return bfail(ctx, AXX_ERR_UNSUPPORTED, "a job's substrate exceeds shared memory");
  // work items, longest first
  axx_batch_options o = opt;
  if (o.tile == 0) {
    const uint64_t shape = batch_shape(jobs, njobs);
    if (!cache_lookup(ctx, shape, o)) {
      double ms = 0.0;
      axx_status s = axx_autotune_batch(ctx, jobs, njobs, 300, &o, &ms);
      if (s != AXX_OK) return s;
    }
  }
  if (o.tile <= 0 || o.tile % 128 != 0)
    return bfail(ctx, AXX_ERR_INVALID_ARG, "tile must be a positive multiple of 128");
  std::vector<BatchItem> items;
  std::vector<int> job_items(njobs, 0);
  std::vector<double> cost;
  for (int j = 0; j < njobs; ++j) {
    const long long n = jp[j].p.num_walkers;
    for (long long f = 0; f < n; f += o.tile) {
      BatchItem it;
      it.job = j;
      it.local = job_items[j]++;
      it.first = f;
      it.count = (int)std::min<long long>(o.tile, n - f);
      it.pad = 0;
      items.push_back(it);
    }
  }
  std::vector<size_t> order(items.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = i;
  auto item_cost = [&](const BatchItem &it) {
    const JobPlan &q = jp[it.job];
    return (double)it.count * (double)q.p.steps * (1.0 + 0.05 * (double)q.g.geo.size());
  };
  // by class (each class kernel takes its own range), longest first within it
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
    const int ca = jp[items[a].job].cls, cb = jp[items[b].job].cls;
    if (ca != cb) return ca < cb;
    return item_cost(items[a]) > item_cost(items[b]);
  });
  std::vector<BatchItem> sorted(items.size());
  for (size_t i = 0; i < order.size(); ++i) sorted[i] = items[order[i]];
  int cfirst[BC_N] = {}, citems[BC_N] = {};
  for (size_t i = 0; i < sorted.size(); ++i) {
    const int c = jp[sorted[i].job].cls;
    if (citems[c]++ == 0) cfirst[c] = (int)i;
  }
  // partials and outputs
  std::vector<long long> part_off(njobs), out_off(njobs);
  long long npart = 0, nout = 0;
  std::vector<int2> outmap;
  for (int j = 0; j < njobs; ++j) {
    part_off[j] = npart;
    npart += (long long)job_items[j] * jobs[j].nseq * 5;
    out_off[j] = nout;
    for (int k = 0; k < jobs[j].nseq * 5; ++k) outmap.push_back(make_int2(j, k));
    nout += jobs[j].nseq * 5;
  }
  // arena: job tables | jobs | items | outmap | job_items | counter | partials | out | counters
  const size_t o_jobs = up256(off);
  const size_t o_items = up256(o_jobs + sizeof(BatchJob) * njobs);
  const size_t o_outmap = up256(o_items + sizeof(BatchItem) * sorted.size());
  const size_t o_jitems = up256(o_outmap + sizeof(int2) * std::max<size_t>(outmap.size(), 1));
  const size_t o_ctr = up256(o_jitems + 4 * njobs);
  const size_t o_part = up256(o_ctr + 16);
  const size_t o_out = up256(o_part + 8 * std::max<long long>(npart, 1));
  const size_t o_cnt = up256(o_out + 8 * std::max<long long>(nout, 1));
  const size_t total = up256(o_cnt + 8 * AXX_CNT_N * njobs);
  auto *b = new axx_batch();
  b->ctx = ctx;
  b->njobs = njobs;
  b->nitems = (int)sorted.size();
  b->kmax = kmax;
  b->tile = o.tile;
  b->smem = smem;
  for (int c = 0; c < BC_N; ++c) {
    b->c_kmax[c] = ckmax[c];
    b->c_smem[c] = csmem[c];
    b->c_first[c] = cfirst[c];
    b->c_items[c] = citems[c];
  }
  b->nout = (int)nout;
  b->use_graph = opt.use_graph != 0;
  e = cudaMalloc(&b->arena, total);
  if (e != cudaSuccess) {
    delete b;
    return bcuda(ctx, e, "cudaMalloc(batch arena)");
  }
  char *base = (char *)b->arena;
  b->d_jobs = (BatchJob *)(base + o_jobs);
  b->d_items = (BatchItem *)(base + o_items);
  b->d_outmap = (int2 *)(base + o_outmap);
  b->d_jobitems = (int *)(base + o_jitems);
  b->d_ctr = (unsigned *)(base + o_ctr);
  b->d_part = (double *)(base + o_part);
  b->d_out = (double *)(base + o_out);
  b->d_counters = (unsigned long long *)(base + o_cnt);
  std::vector<BatchJob> hj(njobs);
  for (int j = 0; j < njobs; ++j) {
    JobPlan &q = jp[j];
    const ArenaLayout L = arena_layout(q.g, q.kt, jobs[j].nseq);
    char *jb = base + job_off[j];
    e = upload_tables(jb, L, q.g, q.kt, ctx->stream);
    if (e != cudaSuccess) break;
    fill_walk_params(hj[j].P, jb, L, q.g, q.kt, &q.p, q.mode, jobs[j].nseq, q.init, q.cell,
                     ctx->abort_dev);
    hj[j].P.counters = b->d_counters + (size_t)AXX_CNT_N * j;
    hj[j].one = (q.g.geom != AXX_GEOM_FREE && q.g.geo.size() == 1 && q.g.cstart.size() == 2) ? 1 : 0;

    hj[j].M = jobs[j].nseq;
    hj[j].part_off = part_off[j];
    hj[j].out_off = out_off[j];
    b->job_M.push_back(jobs[j].nseq);
    const long long ws = q.p.num_walkers * (long long)(q.p.steps - 1);
    b->job_ws.push_back(ws);
    b->walker_steps += ws;
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_jobs, hj.data(), sizeof(BatchJob) * njobs, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess && !sorted.empty())
    e = cudaMemcpyAsync(b->d_items, sorted.data(), sizeof(BatchItem) * sorted.size(),
                        cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess && !outmap.empty())
    e = cudaMemcpyAsync(b->d_outmap, outmap.data(), sizeof(int2) * outmap.size(),
                        cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_jobitems, job_items.data(), 4 * njobs, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    axx_batch_destroy(b);
    return bcuda(ctx, e, "uploading the batch tables");
  }
  // each class kernel: its occupancy, the requested resident blocks, a grid
  // no larger than its items
  for (int c = 0; c < BC_N; ++c) {
    if (citems[c] == 0) continue;
    const int occ = batch_occupancy(c, ckmax[c], csmem[c]);
    if (occ <= 0) {
      axx_batch_destroy(b);
      return bfail(ctx, AXX_ERR_CUDA, "batch kernel cannot be resident");
    }
    int bps = occ;
    if (o.blocks_per_sm > 0) bps = std::min(occ, o.blocks_per_sm);
    if (o.blocks_per_sm < 0) bps = std::max(1, occ + o.blocks_per_sm);
    b->c_bps[c] = bps;
    b->c_grid[c] = std::max(1, std::min(bps * ctx->nsm, citems[c]));
    b->bps = std::max(b->bps, bps);
    b->grid += b->c_grid[c];
    e = cudaStreamCreateWithFlags(&b->cs[c], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->join[c], cudaEventDisableTiming);
    if (e != cudaSuccess) {
      axx_batch_destroy(b);
      return bcuda(ctx, e, "batch streams");
    }
  }
  e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    axx_batch_destroy(b);
    return bcuda(ctx, e, "batch streams");
  }
  if (b->use_graph) {
    // capture: reset the counters, the class kernels (forked onto their
    // streams and joined back), the reduction
    cudaStream_t s = ctx->stream;
    e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      e = batch_enqueue(b, s);
      const cudaError_t e2 = cudaStreamEndCapture(s, &b->graph);
      if (e == cudaSuccess) e = e2;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
    if (e != cudaSuccess) {
      axx_batch_destroy(b);
      return bcuda(ctx, e, "capturing the batch graph");
    }
  }
  *out = b;
  return AXX_OK;
}

extern "C" axx_status axx_batch_create(axx_ctx *ctx, const axx_job *jobs, int njobs,
                                       const axx_batch_options *opt, axx_batch **out) {
  if (!ctx || !jobs || !out) return AXX_ERR_INVALID_ARG;
  axx_batch_options o = opt ? *opt : axx_batch_options{0, 0, 1};
  return batch_build(ctx, jobs, njobs, o, 0, out);
}

extern "C" axx_status axx_batch_launch(axx_batch *b) {
  if (!b) return AXX_ERR_INVALID_ARG;
  axx_ctx *ctx = b->ctx;
  *ctx->abort_host = 0;
  cudaError_t e;
  if (b->use_graph)
    e = cudaGraphLaunch(b->exec, ctx->stream);
  else
    e = batch_enqueue(b, ctx->stream);
  if (e != cudaSuccess) return bcuda(ctx, e, "axx_batch_launch");
  b->launched = true;
  return AXX_OK;
}

extern "C" axx_status axx_batch_read(axx_batch *b, double *mx, double *my, axx_stats *stats) {
  if (!b) return AXX_ERR_INVALID_ARG;
  axx_ctx *ctx = b->ctx;
  if (!b->launched) return bfail(ctx, AXX_ERR_INVALID_ARG, "batch was never launched");
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  std::vector<double> h((size_t)b->nout);
  std::vector<unsigned long long> cnt((size_t)AXX_CNT_N * b->njobs);
  if (e == cudaSuccess && b->nout > 0)
    e = cudaMemcpy(h.data(), b->d_out, 8 * h.size(), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess)
    e = cudaMemcpy(cnt.data(), b->d_counters, 8 * cnt.size(), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return bcuda(ctx, e, "axx_batch_read");
  size_t o = 0, m0 = 0;
  bool capped = false, aborted = false, initf = false;
  for (int j = 0; j < b->njobs; ++j) {
    const int M = b->job_M[j];
    for (int m = 0; m < M; ++m) {
      if (mx) mx[m0 + m] = h[o + m * 5 + 0];
      if (my) my[m0 + m] = h[o + m * 5 + 1];
      if (stats) {
        if (stats[j].sxx) stats[j].sxx[m] = h[o + m * 5 + 2];
        if (stats[j].syy) stats[j].syy[m] = h[o + m * 5 + 3];
        if (stats[j].sxy) stats[j].sxy[m] = h[o + m * 5 + 4];
      }
    }
    const unsigned long long *c = &cnt[(size_t)AXX_CNT_N * j];
    if (stats) {
      stats[j].reflection_cap_hits = (int64_t)c[AXX_CNT_CAP];
      stats[j].walker_steps = b->job_ws[j];
      stats[j].boundary_hits = (int64_t)c[AXX_CNT_HITS];
    }
    capped |= c[AXX_CNT_CAP] != 0;
    aborted |= c[AXX_CNT_ABORTED] != 0;
    initf |= c[AXX_CNT_INIT_FAIL] != 0;
    o += (size_t)M * 5;
    m0 += M;
  }
  if (aborted) return bfail(ctx, AXX_ERR_ABORTED, "batch aborted by axx_abort");
  if (initf) return bfail(ctx, AXX_ERR_INVALID_ARG, "a job's start region is empty");
  if (capped) return bfail(ctx, AXX_ERR_REFLECTION_CAP, "some moves hit the reflection cap of 1024");
  return AXX_OK;
}

extern "C" axx_status axx_batch_info(const axx_batch *b, int *items, int *tile, int *bps,
                                     int *kernel_launches, int64_t *walker_steps) {
  if (!b) return AXX_ERR_INVALID_ARG;
  if (items) *items = b->nitems;
  if (tile) *tile = b->tile;
  if (bps) *bps = b->bps;
  if (kernel_launches) {
    int k = b->nout > 0 ? 1 : 0;
    for (int c = 0; c < BC_N; ++c) k += b->c_items[c] > 0 ? 1 : 0;
    *kernel_launches = k;
  }
  if (walker_steps) *walker_steps = b->walker_steps;
  return AXX_OK;
}

extern "C" axx_status axx_batch_destroy(axx_batch *b) {
  if (!b) return AXX_OK;
  if (b->ctx) cudaStreamSynchronize(b->ctx->stream);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (int c = 0; c < BC_N; ++c) {
    if (b->cs[c]) cudaStreamDestroy(b->cs[c]);
    if (b->join[c]) cudaEventDestroy(b->join[c]);
  }
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->arena) cudaFree(b->arena);
  delete b;
  return AXX_OK;
}

extern "C" axx_status axx_run_batch(axx_ctx *ctx, const axx_job *jobs, int njobs,
                                    const axx_batch_options *opt, double *mx, double *my,
                                    axx_stats *stats) {
  axx_batch *b = nullptr;
  axx_status s = axx_batch_create(ctx, jobs, njobs, opt, &b);
  if (s != AXX_OK) return s;
  s = axx_batch_launch(b);
  if (s == AXX_OK) s = axx_batch_read(b, mx, my, stats);
  axx_batch_destroy(b);
  return s;
}
