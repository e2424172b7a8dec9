// tc_ptx.cuh -- inline-PTX building blocks of the tcgen05 kernels (sm_103a):
// shared-memory matrix descriptors for the canonical K-major layout without
// swizzle, the kind::f16 instruction descriptor, MMA issue and commit,
// mbarriers with bounded waits, bulk copies and TMEM loads.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace axx {

// Byte offset of element (row, k) in the canonical K-major no-swizzle layout
// of a tile with K columns: 8-row x 16-byte core matrices, core (row/8, k/8)
// at ((row/8) * K/8 + k/8) * 128.
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

// Arrives on mbar once every tcgen05 operation this thread issued before is
// complete.
__device__ __forceinline__ void mma_commit(uint32_t mbar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
      : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(mbar), "r"(count));
}

__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mbar), "r"(bytes)
               : "memory");
}

// Global -> shared bulk copy (16-byte aligned, size a multiple of 16) whose
// completion is counted on mbar's transaction bytes.
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes,
                                         uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::
          "r"(dst),
      "l"(src), "r"(bytes), "r"(mbar)
      : "memory");
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
  return t;
}

// Suspend-time hint of the mbarrier waits (ns): a waiting thread is woken at
// least this often, so it resumes soon after the phase completes (measured:
// the default hint left the inference kernel's MMA issue 8 % slower).
constexpr uint32_t kMbarSuspendNs = 32;

// Waits for the phase of parity `parity` to complete.  Gives up (false) when
// *fail is set by another role or after limit_ns of wall-clock time.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, volatile int *fail,
                                          unsigned long long limit_ns) {
  unsigned long long t0 = 0;
  for (uint32_t it = 0;; ++it) {
    uint32_t done;
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
        "selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity), "r"(kMbarSuspendNs)
        : "memory");
    if (done) return true;
    if ((it & 63u) == 0u) {
      if (fail && *fail) return false;
      const unsigned long long t = global_ns();
      if (t0 == 0) t0 = t;
      else if (t - t0 > limit_ns) return false;
    }
  }
}

}  // namespace axx

// 32 consecutive FP32 columns of this warp's 32 TMEM lanes (one row per
// thread).
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

// 16 consecutive FP32 columns of this warp's 32 TMEM lanes.
#define AXX_TMEM_LD16(taddr, r)                                                              \
  asm volatile(                                                                              \
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13," \
      "%14,%15}, [%16];\n"                                                                   \
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),  \
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),           \
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])                                                \
      : "r"(taddr))
