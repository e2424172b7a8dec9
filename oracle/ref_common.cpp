// ref_common.cpp -- stand-ins shared by every build of ref_shim.cpp.
// TEST INFRASTRUCTURE ONLY (part of oracle/_ref).
#include <cstdint>

#include "oracle.h"

struct ShimDim3 {
  unsigned x, y, z;
};
thread_local ShimDim3 threadIdx, blockIdx, blockDim;
thread_local uint32_t shim_last_word;

// Word k of the stream of (seed, walker): Philox4x32-10 with key = seed and
// counter = (k/4, 0, walker).
uint32_t shim_stream_word(uint64_t seed, uint64_t walker, uint32_t k) {
  const uint32_t ctr[4] = {k >> 2, 0u, (uint32_t)walker, (uint32_t)(walker >> 32)};
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t out[4];
  orc_philox4x32_10(ctr, key, out);
  return out[k & 3u];
}
