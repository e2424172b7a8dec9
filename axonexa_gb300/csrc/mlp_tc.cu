// mlp_tc.cu -- fused MLP inference on the 5th-generation tensor cores.
//
// A persistent CTA per SM carries two 128-row tiles of queries through every
// layer, with three warp roles (576 threads):
//   * warp 16 (producer) streams the packed BF16 weights, chunk by chunk
//     (N 256 x K 64, 32 KB), into a 3-slot shared-memory ring with
//     cp.async.bulk; each slot has a "full" mbarrier (transaction bytes) and
//     an "empty" one (released by the tensor cores when the chunk's MMAs are
//     done);
//   * warp 17 (MMA) allocates all 512 TMEM columns -- one 256-column FP32
//     accumulator per row tile -- and, for each (layer, tile) once that tile's
//     input is ready, issues K/16 tcgen05.mma (kind::f16, M 128, N 256,
//     BF16 x BF16 -> FP32) and commits them to the tile's "accumulator full"
//     mbarrier;
//   * warps 0-15 (epilogue; warp w reads TMEM lanes 32(w%4).. -- one row per
//     thread -- and the 64 columns 64(w/4)..) read the accumulator with
//     tcgen05.ld, add the bias (read through L1: one address per warp), apply
//     SiLU (z sigmoid z = h + h tanh h with h = z/2, on the MUFU tanh) and
//     write the BF16 activations back into the tile's shared-memory operand;
//     after the last hidden layer the four column groups' parts of
//     y = h . w_out meet in the tail of the tile's operand (an mbarrier) and
//     the first group adds b_out and stores y.
// Shared memory holds the two 64 KB operands and the 96 KB ring and nothing
// else: 64-column chunks halve the MMA warp's waits per MMA against 32-column
// ones (a wait between MMAs lets the tensor pipe drain), and three of them
// fit only with the biases out of shared memory.
// The MMA warp alternates the two tiles, so one tile's epilogue overlaps the
// other tile's MMAs, and weight copies run ahead of both.
// Operand layout (A activations and B weight chunks): canonical K-major
// without swizzle, 8-row x 16-byte core matrices, core (g, c) of a tile with K
// columns at byte (g * K/8 + c) * 128.
// Every wait is bounded by a wall-clock limit: a wait that runs out sets
// *err and a shared fail flag that ends every role's loop; the producer then
// waits (bounded) for its copies in flight, the MMA warp for its last MMAs,
// and the TMEM is released before the CTA returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <string>

#include "../../include/axx.h"
#include "mlp_internal.h"
#include "tc_ptx.cuh"

namespace axx {

constexpr int TC_ROWS = 128;
constexpr int TC_N = 256;
constexpr int TC_KC = 64;                          // K columns per weight chunk
constexpr int TC_CHUNK_BYTES = TC_N * TC_KC * 2;   // 32 KB
constexpr int TC_STAGES = 3;
constexpr int TC_TILES = 2;                        // row tiles in flight
constexpr int TC_ACT_BYTES = TC_ROWS * TC_N * 2;   // 64 KB per row tile
constexpr int TC_OFF_RING = TC_TILES * TC_ACT_BYTES;
constexpr int TC_GROUPS = 4;                       // epilogue column groups
constexpr int TC_GCOLS = TC_N / TC_GROUPS;
// the column groups' parts of y meet in the last 1.5 KB of the tile's
// operand, which the tile's last-layer MMAs have finished reading
constexpr int TC_YPART_BYTES = (TC_GROUPS - 1) * TC_ROWS * 4;
constexpr int TC_OFF_BAR = TC_OFF_RING + TC_STAGES * TC_CHUNK_BYTES;
constexpr int TC_SMEM = TC_OFF_BAR + 256;
constexpr int TC_EPI_THREADS = TC_GROUPS * TC_ROWS;
constexpr int TC_THREADS = TC_EPI_THREADS + 64;
constexpr int TC_PRODUCER_WARP = TC_EPI_THREADS / 32, TC_MMA_WARP = TC_PRODUCER_WARP + 1;
constexpr unsigned long long TC_WAIT_NS = 2000000000ull;  // 2 s per wait
static_assert(TC_SMEM <= 227 * 1024, "shared memory budget");

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, volatile int *fail) {
  return mbar_wait(mbar, parity, fail, TC_WAIT_NS);
}

// SiLU of z = acc + b from acc and the pre-halved bias hb = b/2:
// z sigmoid(z) = h + h tanh(h) with h = z/2.
__device__ __forceinline__ float silu_half(float acc, float hb) {
  const float h = fmaf(0.5f, acc, hb);
  float t;
  asm("tanh.approx.f32 %0, %1;\n" : "=f"(t) : "f"(h));
  return fmaf(h, t, h);
}

struct TcArgs {
  const float *X;                  // [n][in_dim]
  float *y;                        // [n]
  int n, in_dim, in_pad, depth;
  const __nv_bfloat16 *W[8];       // packed weights per hidden layer, K-chunked
  const float *bias[8];            // per hidden layer
  const float *w_out, *b_out;      // output layer
  int *err;
};

__device__ __forceinline__ int layer_k(const TcArgs &a, int l) { return l == 0 ? a.in_pad : TC_N; }

__global__ void __launch_bounds__(TC_THREADS, 1) mlp_tc_kernel(const __grid_constant__ TcArgs a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ volatile int s_fail;
  __shared__ uint32_t s_tmem;
  const uint32_t bar0 = smem_u32(smem + TC_OFF_BAR);
  // barrier addresses: full[5], empty[5], act_ready[2], acc_full[2], drain,
  // y_half[2]
  auto full_bar = [&](int s) { return bar0 + 8u * (uint32_t)s; };
  auto empty_bar = [&](int s) { return bar0 + 8u * (uint32_t)(TC_STAGES + s); };
  auto act_bar = [&](int t) { return bar0 + 8u * (uint32_t)(2 * TC_STAGES + t); };
  auto acc_bar = [&](int t) { return bar0 + 8u * (uint32_t)(2 * TC_STAGES + 2 + t); };
  const uint32_t drain_bar = bar0 + 8u * (uint32_t)(2 * TC_STAGES + 4);
  auto yh_bar = [&](int t) { return bar0 + 8u * (uint32_t)(2 * TC_STAGES + 5 + t); };
  const uint32_t act0 = smem_u32(smem), ring0 = smem_u32(smem + TC_OFF_RING);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (tid == 0) {
    s_fail = 0;
    for (int s = 0; s < TC_STAGES; ++s) {
      mbar_init(full_bar(s), 1);
      mbar_init(empty_bar(s), 1);
    }
    for (int t = 0; t < TC_TILES; ++t) {
      mbar_init(act_bar(t), TC_EPI_THREADS);
      mbar_init(acc_bar(t), 1);
      mbar_init(yh_bar(t), (TC_GROUPS - 1) * TC_ROWS);
    }
    mbar_init(drain_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == TC_MMA_WARP) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     smem_u32(&s_tmem)),
                 "r"(TC_TILES * TC_N));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
  const uint32_t tmem = s_tmem;
  const int ntiles = (a.n + TC_ROWS - 1) / TC_ROWS;
  const int pair_step = gridDim.x * TC_TILES;

  if (warp == TC_PRODUCER_WARP) {
    // ---------------- producer: weight chunks into the ring
    if (lane == 0) {
      uint32_t g = 0;
      bool ok = true;
      for (int base = blockIdx.x * TC_TILES; base < ntiles && ok; base += pair_step)
        for (int l = 0; l < a.depth && ok; ++l)
#pragma unroll
          for (int t = 0; t < TC_TILES && ok; ++t) {
            if (base + t >= ntiles) continue;
            const int K = layer_k(a, l);
            const unsigned char *src = reinterpret_cast<const unsigned char *>(a.W[l]);
            for (int q = 0; q * TC_KC < K; ++q, ++g) {
              const int kc = min(TC_KC, K - q * TC_KC);
              const uint32_t bytes = (uint32_t)(TC_N * kc * 2);
              const int slot = (int)(g % TC_STAGES);
              const uint32_t ph = (g / TC_STAGES) & 1u;
              if (!mbar_wait(empty_bar(slot), ph ^ 1u, &s_fail)) {
                ok = false;
                break;
              }
              mbar_expect_tx(full_bar(slot), bytes);
              bulk_g2s(ring0 + (uint32_t)slot * TC_CHUNK_BYTES, src + (size_t)q * TC_CHUNK_BYTES,
                       bytes, full_bar(slot));
            }
          }
      if (!ok) {
        s_fail = 1;
        atomicExch(a.err, 1);
        // copies in flight land before the CTA's shared memory is released
        const uint32_t first = g > (uint32_t)TC_STAGES ? g - TC_STAGES : 0u;
        for (uint32_t j = first; j < g; ++j)
          mbar_wait(full_bar((int)(j % TC_STAGES)), (j / TC_STAGES) & 1u, nullptr);
      }
    }
  } else if (warp == TC_MMA_WARP) {
    // ---------------- MMA issuer
    if (lane == 0) {
      uint32_t g = 0, pa[TC_TILES] = {0u, 0u};
      bool ok = true;
      const uint32_t idesc = idesc_bf16(TC_ROWS, TC_N);
      for (int base = blockIdx.x * TC_TILES; base < ntiles && ok; base += pair_step)
        for (int l = 0; l < a.depth && ok; ++l)
#pragma unroll
          for (int t = 0; t < TC_TILES && ok; ++t) {
            if (base + t >= ntiles) continue;
            if (!mbar_wait(act_bar(t), pa[t], &s_fail)) {
              ok = false;
              break;
            }
            pa[t] ^= 1u;
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
            const int K = layer_k(a, l);
            const uint32_t a_tile = act0 + (uint32_t)t * TC_ACT_BYTES;
            const uint32_t sbo_a = (uint32_t)(K >> 3) * 128u;
            for (int q = 0; q * TC_KC < K; ++q, ++g) {
              const int kc = min(TC_KC, K - q * TC_KC);
              const int slot = (int)(g % TC_STAGES);
              const uint32_t ph = (g / TC_STAGES) & 1u;
              if (!mbar_wait(full_bar(slot), ph, &s_fail)) {
                ok = false;
                break;
              }
              asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
              const uint32_t b_chunk = ring0 + (uint32_t)slot * TC_CHUNK_BYTES;
              const uint32_t sbo_b = (uint32_t)(kc >> 3) * 128u;
              for (int kk = 0; kk < kc / 16; ++kk) {
                const int ks = q * (TC_KC / 16) + kk;  // 16-column step within the layer
                const uint64_t ad = smem_desc(a_tile + (uint32_t)ks * 256u, 128u, sbo_a);
                const uint64_t bd = smem_desc(b_chunk + (uint32_t)kk * 256u, 128u, sbo_b);
                mma_issue(tmem + (uint32_t)(t * TC_N), ad, bd, idesc, ks > 0 ? 1u : 0u);
              }
              mma_commit(empty_bar(slot));
            }
            if (ok) mma_commit(acc_bar(t));
          }
      if (!ok) {
        s_fail = 1;
        atomicExch(a.err, 1);
        mma_commit(drain_bar);
        mbar_wait(drain_bar, 0u, nullptr);
      }
    }
  } else {
    // ---------------- epilogue: row r of the tile, column group `grp`
    const int r = tid & (TC_ROWS - 1);
    const int grp = tid >> 7;
    const int c0 = grp * TC_GCOLS;
    const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
    uint32_t pf[TC_TILES] = {0u, 0u}, py[TC_TILES] = {0u, 0u};
    bool ok = true;
    for (int base = blockIdx.x * TC_TILES; base < ntiles && ok; base += pair_step) {
      // layer-0 operands: FP32 queries -> BF16 (K = in_pad, zero padded)
#pragma unroll
      for (int t = 0; t < TC_TILES; ++t) {
        if (base + t >= ntiles) continue;
        const int gr = (base + t) * TC_ROWS + r;
        unsigned char *tile = smem + t * TC_ACT_BYTES;
        for (int k0 = 8 * grp; k0 < a.in_pad; k0 += 8 * TC_GROUPS) {
          __align__(16) __nv_bfloat162 hb[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int k = k0 + 2 * j;
            const float v0 = (gr < a.n && k < a.in_dim) ? __ldg(&a.X[(size_t)gr * a.in_dim + k]) : 0.f;
            const float v1 =
                (gr < a.n && k + 1 < a.in_dim) ? __ldg(&a.X[(size_t)gr * a.in_dim + k + 1]) : 0.f;
            hb[j] = __floats2bfloat162_rn(v0, v1);
          }
          *reinterpret_cast<uint4 *>(tile + canon_off(r, k0, a.in_pad)) =
              *reinterpret_cast<const uint4 *>(hb);
        }
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
        mbar_arrive(act_bar(t));
      }
      float yacc[TC_TILES] = {0.f, 0.f};
      for (int l = 0; l < a.depth && ok; ++l) {
        const bool last = (l == a.depth - 1);
        const float *bl = a.bias[l];  // read through L1: the same address across a warp
#pragma unroll
        for (int t = 0; t < TC_TILES; ++t) {
          if (base + t >= ntiles) continue;
          const bool got = mbar_wait(acc_bar(t), pf[t], &s_fail);
          if (!__all_sync(0xffffffffu, got)) {
            ok = false;
            break;
          }
          pf[t] ^= 1u;
          asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
          unsigned char *tile = smem + t * TC_ACT_BYTES;
          const uint32_t tacc = tmem + lane_base + (uint32_t)(t * TC_N);
          float ys = 0.f;
#pragma unroll 1
          for (int cb = c0; cb < c0 + TC_GCOLS; cb += 32) {
            // 32 columns per TMEM read: 32 registers of accumulator in flight
            uint32_t v[32];
            AXX_TMEM_LD32(tacc + (uint32_t)cb, v);
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            if (last) {
#pragma unroll
              for (int q = 0; q < 8; ++q) {
                const float4 b4 = __ldg(reinterpret_cast<const float4 *>(bl + cb + 4 * q));
                const float4 w4 = __ldg(reinterpret_cast<const float4 *>(a.w_out + cb + 4 * q));
                // the biases halved (exact): the epilogue works on h = z/2
                const float bb[4] = {0.5f * b4.x, 0.5f * b4.y, 0.5f * b4.z, 0.5f * b4.w},
                            ww[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
                for (int j = 0; j < 4; ++j)
                  ys = fmaf(silu_half(__uint_as_float(v[4 * q + j]), bb[j]), ww[j], ys);
              }
            } else {
#pragma unroll
              for (int q = 0; q < 4; ++q) {
                const float4 b0 = __ldg(reinterpret_cast<const float4 *>(bl + cb + 8 * q));
                const float4 b1 = __ldg(reinterpret_cast<const float4 *>(bl + cb + 8 * q + 4));
                const float bb[8] = {0.5f * b0.x, 0.5f * b0.y, 0.5f * b0.z, 0.5f * b0.w,
                                     0.5f * b1.x, 0.5f * b1.y, 0.5f * b1.z, 0.5f * b1.w};
                __align__(16) __nv_bfloat162 hb[4];
#pragma unroll
                for (int j = 0; j < 4; ++j)
                  hb[j] = __floats2bfloat162_rn(silu_half(__uint_as_float(v[8 * q + 2 * j]), bb[2 * j]),
                                                silu_half(__uint_as_float(v[8 * q + 2 * j + 1]),
                                                          bb[2 * j + 1]));
                *reinterpret_cast<uint4 *>(tile + canon_off(r, cb + q * 8, TC_N)) =
                    *reinterpret_cast<const uint4 *>(hb);
              }
            }
          }
          if (last) {
            yacc[t] = ys;
          } else {
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
            mbar_arrive(act_bar(t));
          }
        }
      }
      if (!ok) break;
      // the column groups' parts of y meet: groups 1.. park theirs in shared
      // memory, group 0 adds them, adds b_out and stores
#pragma unroll
      for (int t = 0; t < TC_TILES; ++t) {
        if (base + t >= ntiles) continue;
        if (grp > 0) {
          reinterpret_cast<float *>(smem + (t + 1) * TC_ACT_BYTES - TC_YPART_BYTES)[(grp - 1) * TC_ROWS + r] =
              yacc[t];
          mbar_arrive(yh_bar(t));
        } else {
          const bool got = mbar_wait(yh_bar(t), py[t], &s_fail);
          if (!__all_sync(0xffffffffu, got)) {
            ok = false;
            break;
          }
          const int gr = (base + t) * TC_ROWS + r;
          float yv = yacc[t];
          const float *yp =
              reinterpret_cast<const float *>(smem + (t + 1) * TC_ACT_BYTES - TC_YPART_BYTES);
#pragma unroll
          for (int g2 = 1; g2 < TC_GROUPS; ++g2) yv += yp[(g2 - 1) * TC_ROWS + r];
          if (gr < a.n) a.y[gr] = yv + __ldg(a.b_out);
        }
        py[t] ^= 1u;
      }
    }
    if (!ok) {
      s_fail = 1;
      atomicExch(a.err, 1);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
  if (warp == TC_MMA_WARP)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                 "r"(TC_TILES * TC_N));
}

// Packs W [256][in] (FP32 master, row-major) into BF16 K-chunks of TC_KC
// (64) columns (32 KB each; the last holds what is left, e.g. 16 columns of
// a 16-column input layer), each chunk in the canonical layout with its own
// K, zero padded to in_pad columns.
__global__ void pack_tc_kernel(const float *__restrict__ W, __nv_bfloat16 *__restrict__ out,
                               int in, int in_pad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= TC_N * in_pad) return;
  const int n = i / in_pad, k = i % in_pad;
  const int q = k / TC_KC, kc = min(TC_KC, in_pad - q * TC_KC);
  const float v = k < in ? W[(size_t)n * in + k] : 0.f;
  *reinterpret_cast<__nv_bfloat16 *>(reinterpret_cast<unsigned char *>(out) +
                                     (size_t)q * TC_CHUNK_BYTES +
                                     canon_off(n, k - q * TC_KC, kc)) = __float2bfloat16(v);
}

}  // namespace axx

using namespace axx;

cudaError_t mlp_tc_init(axx_mlp *m) {
  size_t total = 0;
  for (int l = 0; l < m->depth; ++l) total += (size_t)TC_N * (l == 0 ? m->in_pad : TC_N);
  cudaError_t e = cudaMalloc(&m->wtc, total * 2 + 256);
  if (e != cudaSuccess) return e;
  size_t o = 0;
  for (int l = 0; l < m->depth; ++l) {
    m->Wtc.push_back(m->wtc + o);
    o += (size_t)TC_N * (l == 0 ? m->in_pad : TC_N);
  }
  m->tc_error = reinterpret_cast<int *>(m->wtc + total + 64);
  e = cudaMemset(m->tc_error, 0, 4);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(mlp_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              TC_SMEM);
}

void mlp_tc_free(axx_mlp *m) {
  if (m->wtc) cudaFree(m->wtc);
  m->wtc = nullptr;
}

long long mlp_tc_rows_per_wave(const axx_mlp *m) {
  return (long long)TC_ROWS * TC_TILES * m->ctx->nsm;
}

void mlp_pack_tc(axx_mlp *m) {
  for (int l = 0; l < m->depth; ++l) {
    const int in = l == 0 ? m->in_dim : TC_N, pad = l == 0 ? m->in_pad : TC_N;
    pack_tc_kernel<<<(TC_N * pad + 255) / 256, 256, 0, m->ctx->stream>>>(m->weight(l), m->Wtc[l],
                                                                         in, pad);
  }
}

extern "C" axx_status axx_mlp_predict_device(axx_mlp *m, const float *dX, int n, float *dy) {
  if (!m || !dX || !dy || n < 0) return AXX_ERR_INVALID_ARG;
  if (n == 0) return AXX_OK;
  if (m->in_pad > 256 || m->depth > 8) return AXX_ERR_UNSUPPORTED;
  TcArgs a{};
  a.X = dX;
  a.y = dy;
  a.n = n;
  a.in_dim = m->in_dim;
  a.in_pad = m->in_pad;
  a.depth = m->depth;
  for (int l = 0; l < m->depth; ++l) {
    a.W[l] = m->Wtc[l];
    a.bias[l] = m->bias(l);
  }
  a.w_out = m->weight(m->depth);
  a.b_out = m->bias(m->depth);
  a.err = m->tc_error;
  const int ntiles = (n + TC_ROWS - 1) / TC_ROWS;
  const int grid = std::min((ntiles + TC_TILES - 1) / TC_TILES, m->ctx->nsm);
  mlp_tc_kernel<<<grid, TC_THREADS, TC_SMEM, m->ctx->stream>>>(a);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    m->ctx->err = std::string("mlp_tc_kernel: ") + cudaGetErrorString(e);
    return AXX_ERR_CUDA;
  }
  return AXX_OK;
}
