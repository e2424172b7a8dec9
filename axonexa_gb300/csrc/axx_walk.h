// axx_walk.h -- device-side records of one walk (shared by the host planner
// and the kernels).  All device arrays are built by the host planner
// (host_plan.cpp) from the C-ABI records in include/axx.h.
//
// Layout in HBM (per plan, uploaded once):
//   inst_geo[n_inst]   float4 (cx, cy, cz, -R^2)   basis instances: every basis
//   inst_aux[n_inst]   float4 (1/R, eps, slot, type) plus its periodic ghosts
//   cell_start[ncell+1], cell_list[...] uint32/uint16: per grid cell of the
//                      periodic box, the instances whose bounding box meets the
//                      cell dilated by the longest step, in ascending basis order
//   slot_tab[nbasis+1] float4 (speed, step length, dt/T2, 4*kappa); the last
//                      slot is the extracellular space
//   wave[W*steps]      FP32 unit waveforms s_w(i*dt) of the distinct sequences
//   coef[M*K]          FP64 gamma*dt*G_m*(g_m . p_c): phase of sequence m from
//                      the K channel accumulators
//   partials[grid*M*5] FP64 per-block sums (x, y, x^2, y^2, xy), scratch
#pragma once
#include <stdint.h>

#define AXX_KMAX 16          // channel accumulators per pass
#define AXX_MAX_SEQ 256      // sequences per pass (epilogue smem bound)
#define AXX_REFL_CAP 1024    // boundary hits per move before the cap flag
#define AXX_BLOCK 128        // threads per block of the walk kernels
#define AXX_INIT_TRIES 100000

enum { AXX_MODE_LATTICE = 0, AXX_MODE_SINGLE = 1 };
enum { AXX_GEOM_FREE = 0, AXX_GEOM_CYL = 1, AXX_GEOM_SPH = 2, AXX_GEOM_MIX = 3 };

// counters[] slots
enum { AXX_CNT_CAP = 0, AXX_CNT_INIT_FAIL = 1, AXX_CNT_ABORTED = 2, AXX_CNT_HITS = 3,
       AXX_CNT_N = 4 };

struct WalkParams {
  float a, b, c;  // periodic cell
  int mode;       // AXX_MODE_*
  int n_inst;
  int n_list;
  int ncell;
  int smem_geom;  // 1: stage instances and cell lists in shared memory
  const float4 *inst_geo;
  const float4 *inst_aux;
  const uint32_t *cell_start;
  const uint16_t *cell_list;
  int gx, gy, gz;
  float inv_hx, inv_hy, inv_hz;
  const float4 *slot_tab;
  int ecs_slot;
  int steps;
  long long n_walkers;
  long long walker_offset;
  uint32_t seed_lo, seed_hi;
  uint32_t flags;
  int init_mode, init_arg;    // AXX_INIT_*; region id for AXX_INIT_IN_REGION
  int init_quirk;             // single pore: start position drawn on a copy of the stream
  int init_inst;              // instance used by AXX_INIT_IN_BASIS and the single pore
  int init_sph;
  float init_R, init_cx, init_cy, init_cz;
  const int *slot_region;     // region id of each slot (0 for the extracellular slot)
  float single_speed, single_step;  // single pore: speed and step of basis 0
  int K;
  const float *wave;
  int ch_wave[AXX_KMAX];
  float ch_p[AXX_KMAX][3];
  int M;
  const double *coef;
  double *partials;
  unsigned long long *counters;
  const volatile int *abort_flag;  // host-mapped; checked every 1024 moves
};

struct TraceParams {
  int ntrace;
  float *init_pos;  // [ntrace*3]
  float *pos;       // [ntrace*(steps-1)*3]
  int32_t *region;  // [ntrace*(steps-1)]
  int32_t *hits;
  int32_t *words;
};
