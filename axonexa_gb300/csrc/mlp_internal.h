// mlp_internal.h -- the record behind the opaque axx_mlp handle.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <vector>

#include "ctx_internal.h"

struct axx_mlp {
  axx_ctx *ctx = nullptr;
  int in_dim = 0, in_pad = 0, width = 0, depth = 0;
  long long nparam = 0;
  std::vector<long long> w_off, b_off;  // parameter layout (floats)
  float *params = nullptr, *grad = nullptr, *am = nullptr, *av = nullptr;  // FP32, device
  __nv_bfloat16 *wb_all = nullptr;    // BF16 weights [out][in_pad] per hidden layer
  std::vector<__nv_bfloat16 *> Wb;
  __nv_bfloat16 *wtc = nullptr;       // BF16 weights in the tensor-core operand layout
  std::vector<__nv_bfloat16 *> Wtc;
  int *tc_error = nullptr;            // device flag set by a timed-out wait
  long long adam_t = 0;
  // training batch buffers
  void *work = nullptr;
  int cap = 0;
  __nv_bfloat16 *Xb = nullptr, *H = nullptr, *dZb = nullptr;
  float *tb = nullptr, *yb = nullptr, *dy = nullptr, *Cb = nullptr, *Z = nullptr, *dH = nullptr,
        *dZ = nullptr, *loss = nullptr;
  float *kpart = nullptr;  // split-K partials of the weight-gradient GEMMs
  // inference from host memory: device copies of the queries and outputs
  // (grown on demand, kept between calls), and the copy streams and events
  // of the chunk pipeline (queries of chunk i+1 cross while chunk i runs)
  static constexpr int kMaxChunks = 4;
  float *io = nullptr;
  long long io_rows = 0;
  cudaStream_t s_in = nullptr, s_out = nullptr;
  cudaEvent_t ev_start = nullptr, ev_in[kMaxChunks] = {}, ev_done[kMaxChunks] = {};
  float *weight(int l) const { return params + w_off[l]; }
  float *bias(int l) const { return params + b_off[l]; }
  float *grad_weight(int l) const { return grad + w_off[l]; }
  float *grad_bias(int l) const { return grad + b_off[l]; }
};

namespace axx {
constexpr int kMaxSplitK = 16;
// C[m*ldc + n] (+)= sum_k A[m*sam + k*sak] B[k*sbk + n*sbn] on the tcgen05
// tensor cores (mlp_gemm_tc.cu).  part: scratch for split-K partials
// (kMaxSplitK * M * N floats), or null; err: device flag set by a timed-out
// completion wait.
void gemm_bf16(cudaStream_t s, int M, int N, int K, const __nv_bfloat16 *A, long long sam,
               long long sak, const __nv_bfloat16 *B, long long sbk, long long sbn, float *C,
               long long ldc, bool accumulate, float *part, int *err);
// Raises the GEMM kernel's dynamic shared-memory limit (once per process).
cudaError_t gemm_tc_init();
}  // namespace axx

// tensor-core inference (mlp_tc.cu)
cudaError_t mlp_tc_init(axx_mlp *m);
void mlp_tc_free(axx_mlp *m);
// Rows one wave of the persistent inference kernel covers on this device.
long long mlp_tc_rows_per_wave(const axx_mlp *m);
void mlp_pack_tc(axx_mlp *m);
