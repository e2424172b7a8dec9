// mlp_gemm_tc.cu -- the surrogate's training GEMMs on the 5th-generation
// tensor cores.
//
//   C[m][n] (+)= sum_k A(m,k) B(k,n),  A(m,k) = A[m*sam + k*sak],
//                                      B(k,n) = B[k*sbk + n*sbn],
// BF16 operands, FP32 accumulation in TMEM.  One CTA of 128 threads per
// 128 x NT output tile (NT = N rounded up to a multiple of 16, at most 256):
//   * all four warps copy 64-column K chunks of A (128 rows) and B (NT rows)
//     into shared memory in the canonical K-major layout without swizzle,
//     whatever the operands' strides (a row stride along k copies 16-byte
//     core-matrix rows whole; otherwise element by element, coalesced along
//     the unit-stride index), double-buffered;
//   * thread 0 issues the chunk's tcgen05.mma (kind::f16, M 128, N NT, K 16
//     each) and commits them to the chunk's stage mbarrier, which releases the
//     stage for the chunk after next;
//   * after the last chunk, warp w reads TMEM lanes 32w.. (one output row per
//     thread) with tcgen05.ld and stores (or adds) the FP32 row.
// blockIdx.z takes the K range [z kc, (z+1) kc) and writes C + z cz: split-K
// partials for the weight gradients (K = the batch), summed afterwards in a
// fixed order, so results do not depend on scheduling.  Every mbarrier wait
// is bounded (2 s of %globaltimer); a wait that runs out sets *err, skips the
// remaining work and still frees the TMEM.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "mlp_internal.h"
#include "tc_ptx.cuh"

namespace axx {

constexpr int GTC_ROWS = 128;
constexpr int GTC_KC = 64;  // K columns per chunk
constexpr int GTC_THREADS = 128;
constexpr int GTC_A_BYTES = GTC_ROWS * GTC_KC * 2;  // 16 KB
constexpr unsigned long long GTC_WAIT_NS = 2000000000ull;

struct GemmTcArgs {
  int M, N, K;
  const __nv_bfloat16 *A;
  long long sam, sak;
  const __nv_bfloat16 *B;
  long long sbk, sbn;
  float *C;
  long long ldc;
  int accumulate;
  int kc;          // K columns per split (blockIdx.z)
  long long cz;    // C offset between splits
  int nt;          // tile width along N: a multiple of 16, <= 256
  int tcols;       // TMEM columns allocated: a power of two >= max(32, nt)
  int *err;
};

// Copies rows [r0, r0 + rows) x K columns [k0, k0 + 64) of X(r, k) =
// X[r*sr + k*sk] into the canonical tile at `dst` (K = 64), zero outside
// [0, R) x [k0, ke).
__device__ __forceinline__ void load_chunk(unsigned char *dst, const __nv_bfloat16 *X,
                                           long long sr, long long sk, int r0, int rows, int R,
                                           int k0, int ke, int tid) {
  const __nv_bfloat16 zero = __float2bfloat16(0.f);
  const bool vec = sk == 1 && (sr & 7) == 0 && ((reinterpret_cast<uintptr_t>(X) & 15) == 0);
  if (vec) {
    // 8 consecutive k of one row: one 16-byte core-matrix row
    for (int e = tid; e < rows * (GTC_KC / 8); e += GTC_THREADS) {
      const int r = e / (GTC_KC / 8), k8 = (e % (GTC_KC / 8)) * 8;
      const int gr = r0 + r, gk = k0 + k8;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (gr < R && gk + 8 <= ke) {
        v = __ldg(reinterpret_cast<const uint4 *>(X + (size_t)gr * sr + gk));
      } else if (gr < R && gk < ke) {
        __align__(16) __nv_bfloat16 t[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) t[j] = gk + j < ke ? X[(size_t)gr * sr + gk + j] : zero;
        v = *reinterpret_cast<const uint4 *>(t);
      }
      *reinterpret_cast<uint4 *>(dst + canon_off(r, k8, GTC_KC)) = v;
    }
  } else {
    // element by element, the unit-stride index fastest across the threads
    const bool r_fast = sr == 1;
    for (int e = tid; e < rows * GTC_KC; e += GTC_THREADS) {
      const int r = r_fast ? e % rows : e / GTC_KC, k = r_fast ? e / rows : e % GTC_KC;
      const int gr = r0 + r, gk = k0 + k;
      const __nv_bfloat16 v = (gr < R && gk < ke) ? X[(size_t)gr * sr + (size_t)gk * sk] : zero;
      *reinterpret_cast<__nv_bfloat16 *>(dst + canon_off(r, k, GTC_KC)) = v;
    }
  }
}

__global__ void __launch_bounds__(GTC_THREADS, 1) gemm_tc_kernel(const __grid_constant__ GemmTcArgs g) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ uint32_t s_tmem;
  __shared__ volatile int s_fail;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nt = g.nt;
  const int m0 = blockIdx.y * GTC_ROWS, n0 = blockIdx.x * nt;
  const int kb = blockIdx.z * g.kc, ke = min(g.K, kb + g.kc);
  const int nq = ke > kb ? (ke - kb + GTC_KC - 1) / GTC_KC : 0;
  const uint32_t stage_bytes = (uint32_t)(GTC_A_BYTES + nt * GTC_KC * 2);
  const uint32_t bar0 = smem_u32(&bars[0]);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     smem_u32(&s_tmem)),
                 "r"(g.tcols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
  }
  if (tid == 0) {
    s_fail = 0;
    mbar_init(bar0, 1);
    mbar_init(bar0 + 8u, 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
  const uint32_t tmem = s_tmem;
  const uint32_t idesc = idesc_bf16(GTC_ROWS, nt);
  bool ok = true;
  int committed = 0;  // chunks whose MMAs thread 0 committed
  for (int q = 0; q < nq && ok; ++q) {
    const int st = q & 1;
    unsigned char *sa = smem + (size_t)st * stage_bytes;
    unsigned char *sb = sa + GTC_A_BYTES;
    if (q >= 2) {
      // the MMAs of chunk q - 2 read this stage
      const bool got = mbar_wait(bar0 + 8u * (uint32_t)st, (uint32_t)((q - 2) >> 1) & 1u, &s_fail,
                                 GTC_WAIT_NS);
      if (!__syncthreads_and(got)) {
        ok = false;
        break;
      }
    }
    const int k0 = kb + q * GTC_KC;
    load_chunk(sa, g.A, g.sam, g.sak, m0, GTC_ROWS, g.M, k0, ke, tid);
    load_chunk(sb, g.B, g.sbn, g.sbk, n0, nt, g.N, k0, ke, tid);
    // the generic-proxy stores become visible to the tensor cores' reads
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
      const int steps = (min(GTC_KC, ke - k0) + 15) / 16;
      const uint32_t a0 = smem_u32(sa), b0 = smem_u32(sb);
      const uint32_t sbo = (uint32_t)(GTC_KC >> 3) * 128u;
      for (int kk = 0; kk < steps; ++kk) {
        const uint64_t ad = smem_desc(a0 + (uint32_t)kk * 256u, 128u, sbo);
        const uint64_t bd = smem_desc(b0 + (uint32_t)kk * 256u, 128u, sbo);
        mma_issue(tmem, ad, bd, idesc, (q > 0 || kk > 0) ? 1u : 0u);
      }
      mma_commit(bar0 + 8u * (uint32_t)st);
      committed = q + 1;
    }
  }
  if (ok && nq > 0) {
    // the last chunk's commit arrives when every MMA before it is done
    const int q = nq - 1;
    ok = mbar_wait(bar0 + 8u * (uint32_t)(q & 1), (uint32_t)(q >> 1) & 1u, &s_fail, GTC_WAIT_NS);
    ok = __syncthreads_and(ok);
  }
  if (!ok) {
    s_fail = 1;
    if (tid == 0) atomicExch(g.err, 1);
    // MMAs still in flight finish before the TMEM and the stages go
    if (tid == 0 && committed > 0) {
      const int q = committed - 1;
      mbar_wait(bar0 + 8u * (uint32_t)(q & 1), (uint32_t)(q >> 1) & 1u, nullptr, GTC_WAIT_NS);
    }
  } else {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
    // epilogue: row m0 + 32 warp + lane
    const int m = m0 + warp * 32 + lane;
    float *C = g.C + (size_t)blockIdx.z * g.cz;
    const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
    for (int cb = 0; cb < nt; cb += 32) {
      uint32_t v[32];
      const int w = min(32, nt - cb);
      if (nq == 0) {
#pragma unroll
        for (int j = 0; j < 32; ++j) v[j] = 0u;
      } else if (w == 32) {
        AXX_TMEM_LD32(trow + (uint32_t)cb, v);
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      } else {
        AXX_TMEM_LD16(trow + (uint32_t)cb, v);
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      }
      if (m < g.M) {
        float *row = C + (size_t)m * g.ldc + n0 + cb;
        const int lim = min(w, g.N - n0 - cb);
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          if (j < lim) {
            const float x = __uint_as_float(v[j]);
            row[j] = g.accumulate ? row[j] + x : x;
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                 "r"(g.tcols));
}

// Sums the split-K partials part[z][m][n] (z ascending: a fixed order) into C.
__global__ void splitk_sum_kernel(const float *__restrict__ part, int splits, int M, int N,
                                  float *__restrict__ C, long long ldc) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)M * N) return;
  const int m = (int)(i / N), n = (int)(i % N);
  float s = 0.f;
  for (int z = 0; z < splits; ++z) s += part[(long long)z * M * N + i];
  C[m * ldc + n] = s;
}

static size_t gemm_tc_smem(int nt) { return 2 * (size_t)(GTC_A_BYTES + nt * GTC_KC * 2); }

cudaError_t gemm_tc_init() {
  return cudaFuncSetAttribute(gemm_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)gemm_tc_smem(256));
}

void gemm_bf16(cudaStream_t s, int M, int N, int K, const __nv_bfloat16 *A, long long sam,
               long long sak, const __nv_bfloat16 *B, long long sbk, long long sbn, float *C,
               long long ldc, bool accumulate, float *part, int *err) {
  GemmTcArgs g{};
  g.M = M;
  g.N = N;
  g.K = K;
  g.A = A;
  g.sam = sam;
  g.sak = sak;
  g.B = B;
  g.sbk = sbk;
  g.sbn = sbn;
  g.err = err;
  g.nt = std::min(256, (N + 15) / 16 * 16);
  g.tcols = 32;
  while (g.tcols < g.nt) g.tcols <<= 1;
  dim3 grid((N + g.nt - 1) / g.nt, (M + GTC_ROWS - 1) / GTC_ROWS, 1);
  // a long reduction over few output tiles (the weight gradients: K = batch)
  // splits K across CTAs into partials, summed in a fixed order after
  const int tiles = (int)(grid.x * grid.y);
  int splits = 1;
  if (part && !accumulate)
    while (splits < kMaxSplitK && tiles * splits < 128 && K / (splits * 2) >= 2 * GTC_KC)
      splits *= 2;
  const size_t smem = gemm_tc_smem(g.nt);
  if (splits == 1) {
    g.C = C;
    g.ldc = ldc;
    g.accumulate = accumulate ? 1 : 0;
    g.kc = K;
    g.cz = 0;
    gemm_tc_kernel<<<grid, GTC_THREADS, smem, s>>>(g);
    return;
  }
  g.kc = ((K + splits - 1) / splits + GTC_KC - 1) / GTC_KC * GTC_KC;
  g.C = part;
  g.ldc = N;
  g.accumulate = 0;
  g.cz = (long long)M * N;
  grid.z = splits;
  gemm_tc_kernel<<<grid, GTC_THREADS, smem, s>>>(g);
  splitk_sum_kernel<<<(int)(((long long)M * N + 255) / 256), 256, 0, s>>>(part, splits, M, N, C,
                                                                          ldc);
}

}  // namespace axx
