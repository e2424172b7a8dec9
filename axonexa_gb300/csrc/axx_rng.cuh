// axx_rng.cuh -- counter-based randomness and direction math of the walker.
//
// Philox4x32-10 is written from its published description (Salmon, Moraes,
// Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11): ten
// rounds of two 32x32->64 multiplies with a Weyl-sequence key schedule.
//
// Stream layout.  Walker w under seed s draws 32-bit word k of its stream as
//   Philox4x32-10(key = (s_lo, s_hi), counter = (k/4, 0, w_lo, w_hi))[k % 4],
// i.e. the same sequence as cuRAND's Philox4_32_10 device generator after
// curand_init(s, w, 0).  Word 0 is never used: the walk consumes words 1, 2,
// 3, ... in exactly the order the reference consumes curand_uniform() calls
// (src/kernels/kernelLattice.cuh:36,52-53; src/kernels/boundaryCheck.cuh:95),
// so three start-position draws are followed by step draws that always sit in
// aligned pairs (4,5), (6,7), (8,9), ...  A word x becomes the uniform
// ((x >> 9) + 1/2) * 2^-23, exactly representable in FP32 and FP64, in (0, 1).
//
// Direction.  The reference draws phi = 2*pi*u1, theta = acos(2*u2 - 1)
// (kernelLattice.cuh:52-57).  Here cos(theta) = 2*u2 - 1 is exact,
// sin(theta) = sqrt(1 - cos^2) (same value, no acos), and sin/cos(2*pi*u1)
// come from a quadrant reduction of u1 (exact) and Taylor polynomials of
// sin(2*pi*f), cos(2*pi*f) on |f| <= 1/8 (truncation error < 2e-9).  Every
// operation is +, -, *, fma or sqrt with IEEE rounding, so a host build of
// the same sequence gives bit-identical results.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define AXX_HD __host__ __device__ __forceinline__
#else
#define AXX_HD inline
#endif

#if !defined(__CUDA_ARCH__)
#include <cmath>
#include <cstring>
#endif

namespace axx {

struct Words4 {
  uint32_t x, y, z, w;
};

AXX_HD uint32_t mulhi32(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32);
#endif
}

// Philox4x32 with 10 rounds.  Multipliers and Weyl increments are the
// constants given in the SC'11 paper.
AXX_HD Words4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                             uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = mulhi32(M0, c0), lo0 = M0 * c0;
    const uint32_t hi1 = mulhi32(M1, c2), lo1 = M1 * c2;
    const uint32_t n0 = hi1 ^ c1 ^ k0;
    const uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += W0;
    k1 += W1;
  }
  Words4 o;
  o.x = c0;
  o.y = c1;
  o.z = c2;
  o.w = c3;
  return o;
}

AXX_HD int float_bits(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_int(f);
#else
  int i;
  std::memcpy(&i, &f, 4);
  return i;
#endif
}

AXX_HD float word_to_uniform(uint32_t x) {
  // (k + 1/2) * 2^-23 with k = x >> 9: exact in FP32.
#if defined(__CUDA_ARCH__)
  // without an int-to-float conversion: the bits of 1 + k 2^-23 minus
  // (1 - 2^-24), exact by Sterbenz's lemma (both operands lie in [1/2, 2])
  return __uint_as_float((x >> 9) | 0x3F800000u) - 0.999999940395355224609375f;
#else
  return (float)(x >> 9) * 1.1920928955078125e-07f + 5.9604644775390625e-08f;
#endif
}

// Sequential per-walker stream over Philox blocks.
struct Stream {
  uint32_t k0, k1, w_lo, w_hi;
  uint32_t blk;  // index of the block held in b0..b3
  uint32_t b0, b1, b2, b3;
  int pos;       // next word inside the held block (0..4)

  AXX_HD void init(uint64_t seed, uint64_t walker, uint32_t first_word) {
    k0 = (uint32_t)seed;
    k1 = (uint32_t)(seed >> 32);
    w_lo = (uint32_t)walker;
    w_hi = (uint32_t)(walker >> 32);
    blk = first_word >> 2;
    load();
    pos = (int)(first_word & 3u);
  }
  AXX_HD void load() {
    const Words4 o = philox4x32_10(blk, 0u, w_lo, w_hi, k0, k1);
    b0 = o.x;
    b1 = o.y;
    b2 = o.z;
    b3 = o.w;
  }
  AXX_HD uint32_t next_word() {
    if (pos == 4) {
      ++blk;
      load();
      pos = 0;
    }
    const uint32_t v = (pos == 0) ? b0 : (pos == 1) ? b1 : (pos == 2) ? b2 : b3;
    ++pos;
    return v;
  }
  AXX_HD float next() { return word_to_uniform(next_word()); }
  // Two consecutive uniforms; cheap when the position is even.
  AXX_HD void next2(float &u1, float &u2) {
    if ((pos & 1) == 0) {
      if (pos == 4) {
        ++blk;
        load();
        pos = 0;
      }
      const bool lo = (pos == 0);
      u1 = word_to_uniform(lo ? b0 : b2);
      u2 = word_to_uniform(lo ? b1 : b3);
      pos += 2;
    } else {
      u1 = next();
      u2 = next();
    }
  }
  AXX_HD uint32_t words_used() const { return blk * 4u + (uint32_t)pos; }
};

#if defined(__CUDACC__)
// Device stream with the key schedule precomputed: rk0[r] = seed_lo + r*W0,
// rk1[r] = seed_hi + r*W1 (mod 2^32) come from the kernel parameters, the
// product of the constant counter word (the walker id) with M1 in round 1
// is computed once per walker, and each 32x32 multiply is one 64-bit
// product.  Outputs are identical to philox4x32_10 above.
struct DevStream {
  uint32_t w_lo, w_hi, r1_hi, r1_lo;  // walker id; M1 * w_lo of round 1
  uint32_t blk;
  uint32_t b0, b1, b2, b3;
  int pos;

  template <class KP>
  __device__ __forceinline__ void init(const KP &P, uint64_t walker, uint32_t first_word) {
    w_lo = (uint32_t)walker;
    w_hi = (uint32_t)(walker >> 32);
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * w_lo;
    r1_hi = (uint32_t)(p1 >> 32);
    r1_lo = (uint32_t)p1;
    blk = first_word >> 2;
    load(P);
    pos = (int)(first_word & 3u);
  }
  template <class KP>
  __device__ __forceinline__ void load(const KP &P) {
    // round 1 (counter words c1 = 0, c2 = w_lo, c3 = w_hi)
    const uint64_t p0 = (uint64_t)0xD2511F53u * blk;
    uint32_t c0 = r1_hi ^ P.rk0[0];
    uint32_t c1 = r1_lo;
    uint32_t c2 = (uint32_t)(p0 >> 32) ^ w_hi ^ P.rk1[0];
    uint32_t c3 = (uint32_t)p0;
#pragma unroll
    for (int r = 1; r < 10; ++r) {
      const uint64_t q0 = (uint64_t)0xD2511F53u * c0;
      const uint64_t q1 = (uint64_t)0xCD9E8D57u * c2;
      const uint32_t n0 = (uint32_t)(q1 >> 32) ^ c1 ^ P.rk0[r];
      const uint32_t n2 = (uint32_t)(q0 >> 32) ^ c3 ^ P.rk1[r];
      c0 = n0;
      c1 = (uint32_t)q1;
      c2 = n2;
      c3 = (uint32_t)q0;
    }
    b0 = c0;
    b1 = c1;
    b2 = c2;
    b3 = c3;
  }
  template <class KP>
  __device__ __forceinline__ uint32_t next_word(const KP &P) {
    if (pos == 4) {
      ++blk;
      load(P);
      pos = 0;
    }
    const uint32_t v = (pos == 0) ? b0 : (pos == 1) ? b1 : (pos == 2) ? b2 : b3;
    ++pos;
    return v;
  }
  template <class KP>
  __device__ __forceinline__ float next(const KP &P) {
    return word_to_uniform(next_word(P));
  }
  // The words at pos and pos + 1 need at most one new block (pos 3: the held
  // block's last word, then the next block's first; pos 4: the next block's
  // first two), so a warp whose lanes sit at different positions (permeable
  // walks draw one word per wall hit) runs at most one block load per move.
  template <class KP>
  __device__ __forceinline__ void next2(const KP &P, float &u1, float &u2) {
    const int p0 = pos;
    const uint32_t last = b3;
    if (p0 >= 3) {
      ++blk;
      load(P);
    }
    const uint32_t w1 = (p0 == 1) ? b1 : (p0 == 2) ? b2 : (p0 == 3) ? last : b0;
    const uint32_t w2 = (p0 == 1) ? b2 : (p0 == 2) ? b3 : (p0 == 3) ? b0 : b1;
    u1 = word_to_uniform(w1);
    u2 = word_to_uniform(w2);
    pos = (p0 >= 3) ? p0 - 2 : p0 + 2;
  }
  // next2, except that a move whose two words end the held block loads the
  // next one at once (pos 2: the block's last two words; pos 3: the last
  // word, then the next block's first; pos 4: the next block's first two):
  // after the move's draws at least one word is held, so a permeable wall
  // hit's draw (one word) needs no block load inside the divergent boundary
  // loop unless the move hits more than once.  Same words, same positions.
  template <class KP>
  __device__ __forceinline__ void next2_eager(const KP &P, float &u1, float &u2) {
    const int p0 = pos;
    const uint32_t o2 = b2, o3 = b3;
    if (p0 >= 2) {
      ++blk;
      load(P);
    }
    const uint32_t w1 = (p0 == 0) ? b0 : (p0 == 1) ? b1 : (p0 == 2) ? o2 : (p0 == 3) ? o3 : b0;
    const uint32_t w2 = (p0 == 0) ? b1 : (p0 == 1) ? b2 : (p0 == 2) ? o3 : (p0 == 3) ? b0 : b1;
    u1 = word_to_uniform(w1);
    u2 = word_to_uniform(w2);
    pos = (p0 < 2) ? p0 + 2 : p0 - 2;
  }
  __device__ __forceinline__ uint32_t words_used() const { return blk * 4u + (uint32_t)pos; }
};
#endif

AXX_HD float fma_f(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return std::fmaf(a, b, c);
#endif
}

AXX_HD float sqrt_f(float a) {
#if defined(__CUDA_ARCH__)
  return __fsqrt_rn(a);
#else
  return std::sqrt(a);
#endif
}

AXX_HD float div_f(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fdiv_rn(a, b);
#else
  return a / b;
#endif
}

AXX_HD float rint_f(float a) {
#if defined(__CUDA_ARCH__)
  return rintf(a);
#else
  return std::nearbyint(a);
#endif
}

// sin(2*pi*u) and cos(2*pi*u) for u in (0, 1).
AXX_HD void sincos_2pi(float u, float &s, float &c) {
  const float q = rint_f(u * 4.0f);          // quadrant 0..4, u*4 exact
  const float f = fma_f(q, -0.25f, u);        // exact, |f| <= 1/8
  const float f2 = f * f;
  // Taylor coefficients (2*pi)^k / k! with alternating signs, rounded to FP32.
  float ps = fma_f(f2, 0x1.5078340p+5f, -0x1.32d2ccp+6f);
  ps = fma_f(f2, ps, 0x1.466bc6p+6f);
  ps = fma_f(f2, ps, -0x1.4abbcep+5f);
  ps = fma_f(f2, ps, 0x1.921fb6p+2f);
  const float sn = f * ps;
  float pc = fma_f(f2, -0x1.a6d1f2p+4f, 0x1.e1f506p+5f);
  pc = fma_f(f2, pc, -0x1.55d3c8p+6f);
  pc = fma_f(f2, pc, 0x1.03c1f0p+6f);
  pc = fma_f(f2, pc, -0x1.3bd3ccp+4f);
  const float cs = fma_f(f2, pc, 1.0f);
  const int qi = float_bits(q + 12582912.0f) & 3;  // q in 0..4, exact
  // rotate by qi quarter turns
  const float s1 = (qi & 1) ? cs : sn;
  const float c1 = (qi & 1) ? sn : cs;
  s = (qi & 2) ? -s1 : s1;
  c = ((qi + 1) & 2) ? -c1 : c1;
}

// Unit step direction from two uniforms (see the header comment).
AXX_HD void direction(float u1, float u2, float &dx, float &dy, float &dz) {
  float sp, cp;
  sincos_2pi(u1, sp, cp);
  const float z = fma_f(2.0f, u2, -1.0f);
  const float st = sqrt_f(fma_f(-z, z, 1.0f));
  dx = st * cp;
  dy = st * sp;
  dz = z;
}

}  // namespace axx
