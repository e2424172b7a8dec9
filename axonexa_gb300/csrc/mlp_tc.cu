// mlp_tc.cu -- fused MLP inference on the 5th-generation tensor cores.
//
// One CTA (128 threads) evaluates 128 query rows through every layer:
//   * the layer input (128 x K BF16) sits in shared memory in the canonical
//     K-major layout without swizzle: 8-row x 16-byte core matrices, core
//     (g, c) of rows 8g.. and columns 8c.. at byte ((g*K/8 + c) * 128);
//   * the layer's weights (256 x K BF16, packed once into the same layout by
//     pack_tc_kernel) are copied into shared memory;
//   * one elected thread issues K/16 tcgen05.mma (kind::f16, M 128, N 256,
//     BF16 x BF16 -> FP32) into a 256-column TMEM accumulator and commits them
//     to an mbarrier;
//   * after the (bounded) wait every warp reads its 32 TMEM lanes with
//     tcgen05.ld, adds the bias, applies SiLU and writes the BF16 result as
//     the next layer's input; the last hidden layer instead forms the scalar
//     output y = h . w_out + b_out in FP32.
// Shared memory: 64 KB activations + 128 KB weights; one CTA per SM, TMEM
// 256 of 512 columns.  A wait that runs out of iterations sets *err, and the
// CTA still releases its TMEM before returning.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <string>

#include "../../include/axx.h"
#include "mlp_internal.h"

namespace axx {

constexpr int TC_ROWS = 128;
constexpr int TC_N = 256;
constexpr int TC_A_BYTES = TC_ROWS * 256 * 2;   // activations, K <= 256
constexpr int TC_B_BYTES = TC_N * 256 * 2;      // one layer's weights
constexpr int TC_SMEM = TC_A_BYTES + TC_B_BYTES + 64;
constexpr long long TC_WAIT_LIMIT = 1ll << 26;

// Byte offset of element (row, k) in the canonical K-major no-swizzle layout
// of a tile with K columns.
__host__ __device__ __forceinline__ uint32_t canon_off(int row, int k, int K) {
  return (uint32_t)((((row >> 3) * (K >> 3) + (k >> 3)) << 7) + ((row & 7) << 4) + ((k & 7) << 1));
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor: start address, leading (K-direction) and
// stride (M/N-direction) byte offsets between core matrices, descriptor
// version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N and M.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_issue(uint32_t tmem, uint64_t adesc, uint64_t bdesc,
                                          uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "setp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
      "}\n" ::"r"(tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
  for (long long it = 0; it < TC_WAIT_LIMIT; ++it) {
    uint32_t done;
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

#define AXX_TMEM_LD32(taddr, r)                                                              \
  asm volatile(                                                                              \
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13," \
      "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"   \
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),  \
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),           \
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),        \
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),        \
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),        \
        "=r"(r[31])                                                                          \
      : "r"(taddr))

struct TcArgs {
  const float *X;                  // [n][in_dim]
  float *y;                        // [n]
  int n, in_dim, in_pad, depth;
  const __nv_bfloat16 *W[8];       // packed weights per hidden layer (N 256 x K)
  const float *bias[8];            // per hidden layer
  const float *w_out, *b_out;      // output layer
  int *err;
};

__global__ void __launch_bounds__(128, 1) mlp_tc_kernel(const __grid_constant__ TcArgs a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char *sA = smem;
  unsigned char *sB = smem + TC_A_BYTES;
  uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + TC_A_BYTES + TC_B_BYTES);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + TC_A_BYTES + TC_B_BYTES + 16);
  __shared__ int s_fail;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t mbar_a = smem_u32(mbar);
  if (tid == 0) {
    s_fail = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mbar_a));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::);
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(TC_N));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
  const uint32_t tmem = *tmem_slot;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
  uint32_t phase = 0;
  const int ntiles = (a.n + TC_ROWS - 1) / TC_ROWS;
  for (int tile = blockIdx.x; tile < ntiles && !s_fail; tile += gridDim.x) {
    const int row0 = tile * TC_ROWS;
    // layer-0 input: FP32 queries -> BF16 canonical tile (K = in_pad)
    for (int e = tid; e < TC_ROWS * a.in_pad; e += 128) {
      const int r = e / a.in_pad, k = e % a.in_pad;
      const int gr = row0 + r;
      const float v = (gr < a.n && k < a.in_dim) ? a.X[(size_t)gr * a.in_dim + k] : 0.f;
      *reinterpret_cast<__nv_bfloat16 *>(sA + canon_off(r, k, a.in_pad)) = __float2bfloat16(v);
    }
    float yacc = 0.f;
    for (int l = 0; l < a.depth; ++l) {
      const int K = l == 0 ? a.in_pad : TC_N;
      // this layer's packed weights (N 256 x K) into shared memory
      {
        const uint4 *src = reinterpret_cast<const uint4 *>(a.W[l]);
        uint4 *dst = reinterpret_cast<uint4 *>(sB);
        const int n16 = TC_N * K * 2 / 16;
        for (int e = tid; e < n16; e += 128) dst[e] = __ldg(&src[e]);
      }
      asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
      if (tid == 0) {
        const uint32_t idesc = idesc_bf16(TC_ROWS, TC_N);
        const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
        const uint32_t sbo = (uint32_t)(K >> 3) * 128u;
        for (int k = 0; k < K / 16; ++k) {
          const uint64_t ad = smem_desc(a0 + (uint32_t)k * 256u, 128u, sbo);
          const uint64_t bd = smem_desc(b0 + (uint32_t)k * 256u, 128u, sbo);
          mma_issue(tmem, ad, bd, idesc, k > 0 ? 1u : 0u);
        }
        asm volatile(
            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                mbar_a)
            : "memory");
      }
      const bool ok = mbar_wait(mbar_a, phase);
      phase ^= 1u;
      if (!ok) {
        s_fail = 1;
        atomicExch(a.err, 1);
      }
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
      __syncthreads();
      if (s_fail) break;
      // epilogue: row r = 32*warp + lane of the tile, 256 columns
      const int r = warp * 32 + lane;
      const float *bl = a.bias[l];
      const bool last = (l == a.depth - 1);
      for (int cb = 0; cb < TC_N / 32; ++cb) {
        uint32_t v[32];
        AXX_TMEM_LD32(tmem + lane_base + (uint32_t)(cb * 32), v);
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
        if (last) {
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int col = cb * 32 + j;
            const float z = __uint_as_float(v[j]) + __ldg(&bl[col]);
            const float h = z / (1.f + __expf(-z));
            yacc = fmaf(h, __ldg(&a.w_out[col]), yacc);
          }
        } else {
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            __align__(16) __nv_bfloat16 hb[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
              const int col = cb * 32 + q * 8 + j;
              const float z = __uint_as_float(v[q * 8 + j]) + __ldg(&bl[col]);
              hb[j] = __float2bfloat16(z / (1.f + __expf(-z)));
            }
            *reinterpret_cast<uint4 *>(sA + canon_off(r, cb * 32 + q * 8, TC_N)) =
                *reinterpret_cast<const uint4 *>(hb);
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
      __syncthreads();
    }
    if (!s_fail) {
      const int gr = row0 + warp * 32 + lane;
      if (gr < a.n) a.y[gr] = yacc + __ldg(a.b_out);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TC_N));
}

// Packs W [256][in] (FP32 master, row-major) into the canonical BF16 layout
// with K = in_pad columns (zero padding).
__global__ void pack_tc_kernel(const float *__restrict__ W, __nv_bfloat16 *__restrict__ out,
                               int in, int in_pad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= TC_N * in_pad) return;
  const int n = i / in_pad, k = i % in_pad;
  const float v = k < in ? W[(size_t)n * in + k] : 0.f;
  *reinterpret_cast<__nv_bfloat16 *>(reinterpret_cast<unsigned char *>(out) +
                                     canon_off(n, k, in_pad)) = __float2bfloat16(v);
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
  const int grid = std::min(ntiles, m->ctx->nsm);
  mlp_tc_kernel<<<grid, 128, TC_SMEM, m->ctx->stream>>>(a);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    m->ctx->err = std::string("mlp_tc_kernel: ") + cudaGetErrorString(e);
    return AXX_ERR_CUDA;
  }
  return AXX_OK;
}
