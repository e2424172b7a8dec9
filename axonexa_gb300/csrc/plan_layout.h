// plan_layout.h -- device layout of one walk: kernel tables in the kernels'
// format, their placement in one device arena, and the kernel parameters.
// Shared by the plan path (api.cpp, arena from cudaMalloc) and the
// no-allocation path (noalloc.cu, arena in a static device array).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/axx.h"
#include "axx_walk.h"
#include "host_plan.h"

namespace axx {

struct KernelTables {
  int km = AXX_KM_LAT_IMP;
  int kmax = 1;
  int K = 0;
  std::vector<float> wave_il;  // [steps][kmax]
  // channel 3w + a is waveform w along axis a (x, y, z), for every channel,
  // with at most four waveforms: the walk reads wave4 (one float4 per step)
  bool axis_channels = false;
  std::vector<float> wave4;    // [steps][4]
  std::vector<double> coef;    // [M][kmax]
  float ch_p[AXX_KMAX][3] = {};
};

struct ArenaLayout {
  size_t o_geo = 0, o_aux = 0, o_cs = 0, o_cl = 0, o_slot = 0, o_reg = 0, o_wave = 0,
         o_wave4 = 0, o_coef = 0, o_out = 0, o_cnt = 0, o_part = 0;
  size_t fixed = 0;      // bytes before the partials
  size_t per_block = 0;  // partials per block
  size_t upload = 0;     // bytes copied host -> device per plan
};

// Walk mode for a plan.
int walk_mode(int mode, int geom, uint32_t flags);
// Kernel-format tables (interleaved, padded channels) from the plans.
// min_kmax pads the channel capacity further (a batch shares one capacity).
std::string make_kernel_tables(const GeomPlan &g, const SeqPlan &sq, int M, int steps, int mode,
                               uint32_t flags, KernelTables &kt, int min_kmax = 1);
// Dynamic shared memory of the walk kernel: the per-warp sums (unless the
// sums go to per-warp rows in global memory, warp_rows) and the staged
// instances, cell starts and cell lists (the slot tables stay in global
// memory).
size_t walk_smem_bytes(const GeomPlan &g, int M, bool warp_rows = false);
// The per-warp sums alone (substrates whose tables stay in global memory).
size_t walk_sums_bytes(int M, bool warp_rows = false);
// The staged instances, cell starts and lists (what a finer grid grows).
size_t walk_table_bytes(const GeomPlan &g);
// Shared memory the walk kernel's staged tables may take so that the blocks
// its register budget allows stay resident (K phase channels): the budget a
// finer grid of a cylinder lattice may fill.
size_t list_table_budget(int K);
// The substrate tables the batch kernel stages per job (slot tables included).
size_t batch_table_bytes(const GeomPlan &g);
// Partials: one row of M x 5 sums per block, or per warp with warp_rows.
ArenaLayout arena_layout(const GeomPlan &g, const KernelTables &kt, int M,
                         bool warp_rows = false);
cudaError_t upload_tables(char *base, const ArenaLayout &L, const GeomPlan &g,
                          const KernelTables &kt, cudaStream_t s);

struct InitSpec {
  int inst = 0, sph = 0;
  double R = 0, cx = 0, cy = 0, cz = 0;
};
// Start-position parameters (basis init_arg for AXX_INIT_IN_BASIS, basis 0
// for the single pore); "" or an error message.
std::string init_spec(const GeomPlan &g, const axx_basis *basis, int nbasis, int mode,
                      const axx_run_params *p, InitSpec &out);

void fill_walk_params(WalkParams &P, char *base, const ArenaLayout &L, const GeomPlan &g,
                      const KernelTables &kt, const axx_run_params *p, int mode, int M,
                      const InitSpec &init, const double cell[3],
                      const volatile int *abort_flag, bool warp_rows = false);

}  // namespace axx
