// ctx_internal.h -- the context record behind the opaque axx_ctx handle.
#pragma once
#include <cuda_runtime.h>

#include <string>

struct axx_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[8] = {};
  std::string err;
  int nsm = 0, ccmaj = 0, ccmin = 0;
  size_t gmem = 0;
  volatile int *abort_host = nullptr;
  int *abort_dev = nullptr;
  // bytes the walk entry points copied between host and device on this
  // context (plan tables up, sums and counters down)
  unsigned long long h2d_bytes = 0, d2h_bytes = 0;
};
