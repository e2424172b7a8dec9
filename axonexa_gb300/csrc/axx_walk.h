// axx_walk.h -- device-side records of one walk (shared by the host planner
// and the kernels).  All device arrays are built by the host planner
// (host_plan.cpp) from the C-ABI records in include/axx.h.
//
// Layout in HBM (per plan, uploaded once):
//   inst_geo[n_inst]   float4 (cx, cy, cz, -R^2)   basis instances: every basis
//                      (lattices of z-cylinders: cz is (R + h)^2 of the
//                      annulus test)
//   inst_aux[n_inst]   float4 (1/R, eps, slot, type) plus its periodic ghosts
//   cell_start[ncell+1], cell_list[...] uint32/uint16: per grid cell of the
//                      periodic box, the instances whose bounding box meets the
//                      cell dilated by the longest step, in ascending basis order
//   slot_tab[nbasis+1] float4 (speed, step length, dt/T2, 4*kappa); the last
//                      slot is the extracellular space
//   wave_il[steps*KMAX] FP32 unit waveform of each phase channel, step-major
//                      (one row of KMAX values per step; padded channels 0)
//   wave4[steps]       float4: axis-channel plans (channel 3w + a is waveform
//                      w along axis a, w < 4): the four waveforms per step
//   coef[M*KMAX]       FP64 gamma*dt*G_m*alpha_mc: phase of sequence m from
//                      the channel accumulators (0 for padded channels)
//   partials[rows*Mo*5] FP64 sums (x, y, x^2, y^2, xy) of the Mo = M rows (2M
//                      with compartment sums), one row set per block, or per
//                      warp (warp_rows: the shared memory holds no sums), scratch
#pragma once
#include <stdint.h>

#define AXX_KMAX 16          // channel accumulators per pass
#define AXX_MAX_SEQ 256      // sequences per pass (epilogue smem bound)
#define AXX_REFL_CAP 1024    // boundary hits per move before the cap flag
#define AXX_BLOCK 128        // threads per block of the walk kernels
#define AXX_INIT_TRIES 100000

#ifndef AXX_MIN_BLOCKS
#define AXX_MIN_BLOCKS 6      // resident blocks per SM the register budget targets
#endif
// 16 channels (32 accumulator registers) spill under the 80 registers of 6
// resident blocks; 5 blocks (102 registers) measured 2 % faster than 6 and
// 10 % faster than 4 on the 400-cylinder pack.
#ifndef AXX_MIN_BLOCKS_WIDE
#define AXX_MIN_BLOCKS_WIDE 5
#endif
#define AXX_MIN_BLOCKS_FOR(kmax) ((kmax) >= 12 ? AXX_MIN_BLOCKS_WIDE : AXX_MIN_BLOCKS)
#define AXX_SMEM_MAX (200 * 1024)

enum { AXX_MODE_LATTICE = 0, AXX_MODE_SINGLE = 1 };
// walk modes (template parameter of the kernels)
enum { AXX_KM_LAT_IMP = 0,     // lattice, specular, impermeable
       AXX_KM_LAT_PERM = 1,    // lattice, specular, permeable
       AXX_KM_LAT_REJ = 2,     // lattice, simple rejection
       AXX_KM_SINGLE = 3,      // single pore, specular
       AXX_KM_SINGLE_REJ = 4,  // single pore, simple rejection
       AXX_KM_N = 5 };
enum { AXX_GEOM_FREE = 0, AXX_GEOM_CYL = 1, AXX_GEOM_SPH = 2, AXX_GEOM_MIX = 3 };

// counters[] slots
enum { AXX_CNT_CAP = 0, AXX_CNT_INIT_FAIL = 1, AXX_CNT_ABORTED = 2, AXX_CNT_HITS = 3,
       AXX_CNT_START_IN = 4, AXX_CNT_N = 5 };

struct WalkParams {
  float a, b, c;  // periodic cell
  int mode;       // AXX_MODE_*
  int km;         // AXX_KM_*
  int n_inst;
  int n_slot;
  int n_list;
  int ncell;
  const float4 *inst_geo;
  const float4 *inst_aux;
  const uint32_t *cell_start;
  const uint16_t *cell_list;
  int gx, gy, gz;
  float inv_hx, inv_hy, inv_hz;
  float ann_h2x2;             // cylinder lattices: 2 h^2 of the annulus test (geo.z = (R+h)^2)
  const float4 *slot_tab;
  const int *slot_region;     // region id of each slot (0 for the extracellular slot)
  int ecs_slot;
  int steps;
  long long n_walkers;
  long long walker_offset;
  uint32_t seed_lo, seed_hi;
  uint32_t rk0[10], rk1[10];  // Philox round keys of the seed (key schedule precomputed)
  uint32_t flags;
  int init_mode, init_arg;    // AXX_INIT_*; region id for AXX_INIT_IN_REGION
  int init_quirk;             // single pore: start position drawn on a copy of the stream
  int picking;                // single pore: LATTICE_PICKING moves
  int init_inst;              // instance used by AXX_INIT_IN_BASIS and the single pore
  int init_sph;
  float init_R, init_cx, init_cy, init_cz;
  int K, kmax;                // channels in use, channel capacity (padded)
  const float *wave_il;       // [steps][kmax]
  const float4 *wave4;        // axis channels: [steps] the four waveforms' values
  float ch_p[AXX_KMAX][3];    // channel projections (0 for padded channels)
  int one_dir;                // every channel in use has the same projection
  int phase_axes;             // axes some channel projects on (bits x, y, z)
  int axis_channels;          // channel 3w + a is waveform w along axis a (w < 4)
  int M;
  int compart;                // also sums over walkers starting in a basis: rows M..2M-1
  int global_tables;          // substrate tables read from global memory (too big to stage)
  int warp_rows;              // partials: one row per warp (gwarp) instead of per block
  const double *coef;         // [M][kmax]
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
