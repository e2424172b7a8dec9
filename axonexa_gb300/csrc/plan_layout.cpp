// plan_layout.cpp -- see plan_layout.h.
#include "plan_layout.h"

#include <cstring>

namespace axx {

static size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }

int walk_mode(int mode, int geom, uint32_t flags) {
  const bool reject = flags & AXX_FLAG_SIMPLE_REJECTION;
  if (mode == AXX_MODE_SINGLE) return reject ? AXX_KM_SINGLE_REJ : AXX_KM_SINGLE;
  if (geom == AXX_GEOM_FREE) return AXX_KM_LAT_IMP;  // no boundaries: the modes coincide
  if (reject) return AXX_KM_LAT_REJ;
  return (flags & AXX_FLAG_PERMEABLE) ? AXX_KM_LAT_PERM : AXX_KM_LAT_IMP;
}

std::string make_kernel_tables(const GeomPlan &g, const SeqPlan &sq, int M, int steps, int mode,
                               uint32_t flags, KernelTables &kt, int min_kmax) {
  kt = KernelTables();
  kt.K = (int)sq.channels.size();
  if (kt.K > AXX_KMAX)
    return "more than 16 phase channels (distinct waveform x direction) in one walk";
  kt.km = walk_mode(mode, g.geom, flags);
  kt.kmax = 1;
  while (kt.kmax < kt.K || kt.kmax < min_kmax) kt.kmax <<= 1;
  // lattice walks of 9-12 channels (four waveforms along three axes): a
  // 12-channel capacity instead of 16 padded ones
  if (mode == AXX_MODE_LATTICE && kt.kmax == 16 && kt.K <= 12 && min_kmax <= 12) kt.kmax = 12;
  if (kt.kmax > AXX_KMAX) return "channel capacity above 16";
  const int km = kt.kmax;
  kt.wave_il.assign((size_t)steps * km, 0.f);
  for (int c = 0; c < kt.K; ++c) {
    const float *src = &sq.wave[(size_t)sq.channels[c].wave * steps];
    for (int i = 0; i < steps; ++i) kt.wave_il[(size_t)i * km + c] = src[i];
    for (int k = 0; k < 3; ++k) kt.ch_p[c][k] = sq.channels[c].p[k];
  }
  // axis channels: every waveform carries the three axis vectors in order
  // (plan_sequences chooses the axes when a waveform's directions span
  // space), lattice walks with the 12-channel capacity
  kt.axis_channels = mode == AXX_MODE_LATTICE && km == 12 && kt.K % 3 == 0;
  for (int c = 0; c < kt.K && kt.axis_channels; ++c) {
    const Channel &ch = sq.channels[c];
    if (ch.wave != sq.channels[c - c % 3].wave || (c % 3 == 0 && c > 0 &&
                                                   ch.wave == sq.channels[c - 1].wave))
      kt.axis_channels = false;
    for (int k = 0; k < 3; ++k)
      if (ch.p[k] != (k == c % 3 ? 1.0f : 0.0f)) kt.axis_channels = false;
  }
  if (kt.axis_channels) {
    kt.wave4.assign((size_t)steps * 4, 0.f);
    for (int w = 0; w < kt.K / 3; ++w) {
      const float *src = &sq.wave[(size_t)sq.channels[3 * w].wave * steps];
      for (int i = 0; i < steps; ++i) kt.wave4[(size_t)i * 4 + w] = src[i];
    }
  }
  kt.coef.assign((size_t)M * km, 0.0);
  for (int m = 0; m < M; ++m)
    for (int c = 0; c < kt.K; ++c) kt.coef[(size_t)m * km + c] = sq.coef[(size_t)m * kt.K + c];
  return "";
}

size_t walk_sums_bytes(int M, bool warp_rows) {
  return warp_rows ? 0 : (size_t)(AXX_BLOCK / 32) * M * 5 * sizeof(double);  // 160 M
}

size_t walk_table_bytes(const GeomPlan &g) {
  return g.geo.size() * 32 + g.cstart.size() * 4 + g.clist.size() * 2;
}

size_t walk_smem_bytes(const GeomPlan &g, int M, bool warp_rows) {
  return walk_sums_bytes(M, warp_rows) + walk_table_bytes(g);
}

size_t list_table_budget(int K) {
  int kmax = 1;
  while (kmax < K) kmax <<= 1;
  if (kmax == 16 && K <= 12) kmax = 12;
  // 228 KB of shared memory per SM, 1 KB of it reserved per resident block
  const size_t per_sm = 228 * 1024;
  return per_sm / AXX_MIN_BLOCKS_FOR(kmax) - 1024;
}

size_t batch_table_bytes(const GeomPlan &g) {
  return walk_table_bytes(g) + g.slot_tab.size() * 20;
}

ArenaLayout arena_layout(const GeomPlan &g, const KernelTables &kt, int M, bool warp_rows) {
  ArenaLayout L;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off = up256(off + bytes);
    return o;
  };
  L.o_geo = take(g.geo.size() * 16);
  L.o_aux = take(g.aux.size() * 16);
  L.o_cs = take(g.cstart.size() * 4);
  L.o_cl = take(g.clist.size() * 2);
  L.o_slot = take(g.slot_tab.size() * 16);
  L.o_reg = take(g.slot_region.size() * 4);
  L.o_wave = take(kt.wave_il.size() * 4);
  L.o_wave4 = take(kt.wave4.size() * 4);
  L.o_coef = take(kt.coef.size() * 8);
  L.o_out = take((size_t)M * 5 * 8);
  L.o_cnt = take(AXX_CNT_N * 8);
  L.o_part = off;
  L.fixed = off;
  L.per_block = (size_t)M * 5 * 8 * (warp_rows ? AXX_BLOCK / 32 : 1);
  L.upload = g.geo.size() * 16 + g.aux.size() * 16 + g.cstart.size() * 4 + g.clist.size() * 2 +
             g.slot_tab.size() * 16 + g.slot_region.size() * 4 + kt.wave_il.size() * 4 +
             kt.wave4.size() * 4 + kt.coef.size() * 8;
  return L;
}

cudaError_t upload_tables(char *base, const ArenaLayout &L, const GeomPlan &g,
                          const KernelTables &kt, cudaStream_t s) {
  auto up = [&](size_t o, const void *src, size_t bytes) {
    return bytes ? cudaMemcpyAsync(base + o, src, bytes, cudaMemcpyHostToDevice, s)
                 : cudaSuccess;
  };
  const cudaError_t es[] = {up(L.o_geo, g.geo.data(), g.geo.size() * 16),
                            up(L.o_aux, g.aux.data(), g.aux.size() * 16),
                            up(L.o_cs, g.cstart.data(), g.cstart.size() * 4),
                            up(L.o_cl, g.clist.data(), g.clist.size() * 2),
                            up(L.o_slot, g.slot_tab.data(), g.slot_tab.size() * 16),
                            up(L.o_reg, g.slot_region.data(), g.slot_region.size() * 4),
                            up(L.o_wave, kt.wave_il.data(), kt.wave_il.size() * 4),
                            up(L.o_wave4, kt.wave4.data(), kt.wave4.size() * 4),
                            up(L.o_coef, kt.coef.data(), kt.coef.size() * 8)};
  for (cudaError_t e : es)
    if (e != cudaSuccess) return e;
  return cudaSuccess;
}

std::string init_spec(const GeomPlan &g, const axx_basis *basis, int nbasis, int mode,
                      const axx_run_params *p, InitSpec &out) {
  out = InitSpec();
  int k = -1;
  if (mode == AXX_MODE_SINGLE) {
    k = 0;
  } else if (p->init_mode == AXX_INIT_IN_BASIS) {
    if (p->init_arg < 0 || p->init_arg >= nbasis)
      return "init_arg must name a basis for AXX_INIT_IN_BASIS";
    k = p->init_arg;
    if (basis[k].type == AXX_PRIM_PLANE)
      return "a plane has no inside to start walkers in (AXX_INIT_IN_BASIS)";
  }
  if (k < 0) return "";
  for (int n = 0; n < (int)g.aux.size(); ++n) {
    int slot;
    std::memcpy(&slot, &g.aux[n].z, 4);
    if (slot == k) {
      out.inst = n;
      break;
    }
  }
  const axx_basis &b = basis[k];
  out.sph = b.type == AXX_PRIM_SPHERE;
  out.R = b.radius;
  out.cx = b.cx;
  out.cy = b.cy;
  out.cz = b.cz;
  return "";
}

void fill_walk_params(WalkParams &P, char *base, const ArenaLayout &L, const GeomPlan &g,
                      const KernelTables &kt, const axx_run_params *p, int mode, int M,
                      const InitSpec &init, const double cell[3],
                      const volatile int *abort_flag, bool warp_rows) {
  std::memset(&P, 0, sizeof(P));
  P.a = (float)cell[0];
  P.b = (float)cell[1];
  P.c = (float)cell[2];
  P.mode = mode;
  P.km = kt.km;
  P.n_inst = (int)g.geo.size();
  P.n_slot = (int)g.slot_tab.size();
  P.n_list = (int)g.clist.size();
  P.ncell = (int)g.cstart.size() - 1;
  P.inst_geo = (const float4 *)(base + L.o_geo);
  P.inst_aux = (const float4 *)(base + L.o_aux);
  P.cell_start = (const uint32_t *)(base + L.o_cs);
  P.cell_list = (const uint16_t *)(base + L.o_cl);
  P.gx = g.gx;
  P.gy = g.gy;
  P.gz = g.gz;
  P.inv_hx = g.inv_hx;
  P.inv_hy = g.inv_hy;
  P.inv_hz = g.inv_hz;
  P.ann_h2x2 = g.ann_h2x2;
  P.slot_tab = (const float4 *)(base + L.o_slot);
  P.slot_region = (const int *)(base + L.o_reg);
  P.ecs_slot = g.ecs_slot;
  P.steps = p->steps;
  P.n_walkers = p->num_walkers;
  P.walker_offset = p->walker_offset;
  P.seed_lo = (uint32_t)p->seed;
  P.seed_hi = (uint32_t)(p->seed >> 32);
  for (int r = 0; r < 10; ++r) {  // Philox4x32 Weyl key schedule
    P.rk0[r] = P.seed_lo + (uint32_t)r * 0x9E3779B9u;
    P.rk1[r] = P.seed_hi + (uint32_t)r * 0xBB67AE85u;
  }
  P.flags = p->flags;
  P.init_mode = p->init_mode;
  P.init_arg = p->init_arg;
  P.init_quirk = (mode == AXX_MODE_SINGLE) && !(p->flags & AXX_FLAG_FIX_INIT_QUIRK);
  P.picking = (mode == AXX_MODE_SINGLE) && (p->flags & AXX_FLAG_LATTICE_PICKING);
  P.init_inst = init.inst;
  P.init_sph = init.sph;
  P.init_R = (float)init.R;
  P.init_cx = (float)init.cx;
  P.init_cy = (float)init.cy;
  P.init_cz = (float)init.cz;
  P.K = kt.K;
  P.kmax = kt.kmax;
  P.wave_il = (const float *)(base + L.o_wave);
  P.wave4 = (const float4 *)(base + L.o_wave4);
  P.axis_channels = kt.axis_channels ? 1 : 0;
  for (int c = 0; c < AXX_KMAX; ++c)
    for (int k = 0; k < 3; ++k) P.ch_p[c][k] = kt.ch_p[c][k];
  P.one_dir = 1;
  for (int c = 1; c < kt.K; ++c)
    for (int k = 0; k < 3; ++k)
      if (kt.ch_p[c][k] != kt.ch_p[0][k]) P.one_dir = 0;
  P.phase_axes = 0;
  for (int c = 0; c < AXX_KMAX; ++c)
    for (int k = 0; k < 3; ++k)
      if (kt.ch_p[c][k] != 0.0f) P.phase_axes |= 1 << k;
  P.M = M;
  P.compart = (mode == AXX_MODE_LATTICE && (p->flags & AXX_FLAG_COMPARTMENTS)) ? 1 : 0;
  P.coef = (const double *)(base + L.o_coef);
  P.partials = (double *)(base + L.o_part);
  P.counters = (unsigned long long *)(base + L.o_cnt);
  P.abort_flag = abort_flag;
  P.warp_rows = warp_rows ? 1 : 0;
}

}  // namespace axx
