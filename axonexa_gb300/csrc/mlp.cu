// mlp.cu -- the learned surrogate's network: MLP in -> depth x width (SiLU)
// -> 1, trained with hand-written BF16 tensor-core GEMMs (tcgen05.mma with
// TMEM accumulators, mlp_gemm_tc.cu) and Adam; inference runs the fused
// tcgen05 kernel of mlp_tc.cu.
//
// Training step for a batch of B rows (weights W_l are [out][in] row-major):
//   forward   Z_l = A_l W_l^T + b_l, H_l = silu(Z_l) (A_0 = X, A_l = H_{l-1}),
//             y = H_last w_out + b_out
//   loss      mean (y - t)^2
//   backward  dy = 2 (y - t) / B; dW_out = H_last^T dy; dH_last = dy w_out^T;
//             dZ_l = dH_l * silu'(Z_l); dW_l = dZ_l^T A_l; db_l = sum_b dZ_l;
//             dH_{l-1} = dZ_l W_l
//   update    Adam (beta1 0.9, beta2 0.999, eps 1e-8) on FP32 master weights,
//             then BF16 copies of the weights for the next GEMMs.
// GEMM operands are BF16 (activations, weights, dZ); accumulation and the
// elementwise work are FP32.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/axx.h"
#include "axx_rng.cuh"
#include "ctx_internal.h"
#include "mlp_internal.h"

namespace axx {

// ---- elementwise kernels ----------------------------------------------------
__device__ __forceinline__ float sigmoid_f(float z) { return 1.0f / (1.0f + __expf(-z)); }

// Gathers a batch: rows idx[b] (or b when idx is null) of the FP32 inputs into
// the BF16 operand [B][in_pad] (zero padded) and the targets.
__global__ void gather_kernel(const float *__restrict__ X, const float *__restrict__ y, int n,
                              int in_dim, int in_pad, int B, uint64_t seed, uint32_t step,
                              int random, __nv_bfloat16 *__restrict__ Xb, float *__restrict__ tb) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  int row = b;
  if (random) {
    const Words4 w = philox4x32_10(step, (uint32_t)b, 0x5EEDu, 0u, (uint32_t)seed,
                                   (uint32_t)(seed >> 32));
    row = (int)(((uint64_t)w.x * (uint64_t)n) >> 32);
  }
  for (int k = 0; k < in_pad; ++k)
    Xb[(size_t)b * in_pad + k] = __float2bfloat16(k < in_dim ? X[(size_t)row * in_dim + k] : 0.f);
  if (tb) tb[b] = y ? y[row] : 0.f;
}

// Z = C + bias (kept in FP32), H = silu(Z) in BF16.
__global__ void bias_silu_kernel(const float *__restrict__ C, const float *__restrict__ bias,
                                 float *__restrict__ Z, __nv_bfloat16 *__restrict__ H, int B,
                                 int N) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)B * N) return;
  const float z = C[i] + bias[i % N];
  Z[i] = z;
  H[i] = __float2bfloat16(z * sigmoid_f(z));
}

// y[b] = sum_j H[b][j] w[j] + b0 (the scalar output layer, FP32).
__global__ void out_dot_kernel(const __nv_bfloat16 *__restrict__ H, const float *__restrict__ w,
                               const float *__restrict__ b0, float *__restrict__ y, int B, int N) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= B) return;
  float s = 0.f;
  for (int j = lane; j < N; j += 32) s += __bfloat162float(H[(size_t)warp * N + j]) * w[j];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) y[warp] = s + b0[0];
}

// dy = 2 (y - t) / B; loss += sum (y - t)^2 / B.
__global__ void loss_grad_kernel(const float *__restrict__ y, const float *__restrict__ t,
                                 float *__restrict__ dy, float *__restrict__ loss, int B) {
  __shared__ float red[256];
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  float e = 0.f;
  if (b < B) {
    const float d = y[b] - t[b];
    dy[b] = 2.f * d / (float)B;
    e = d * d / (float)B;
  }
  red[threadIdx.x] = e;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(loss, red[0]);
}

// Output layer backward: dW_out[j] = sum_b dy[b] H[b][j] (one block per j),
// db_out = sum_b dy[b]; dH[b][j] = dy[b] w[j].
__global__ void out_backward_kernel(const float *__restrict__ dy, const __nv_bfloat16 *__restrict__ H,
                                    const float *__restrict__ w, float *__restrict__ dW,
                                    float *__restrict__ db, float *__restrict__ dH, int B, int N) {
  __shared__ float red[256];
  const int j = blockIdx.x;
  float s = 0.f, sb = 0.f;
  for (int b = threadIdx.x; b < B; b += blockDim.x) {
    s += dy[b] * __bfloat162float(H[(size_t)b * N + j]);
    sb += dy[b];
    dH[(size_t)b * N + j] = dy[b] * w[j];
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int k = 128; k > 0; k >>= 1) {
    if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) dW[j] = red[0];
  if (j == 0) {
    __syncthreads();
    red[threadIdx.x] = sb;
    __syncthreads();
    for (int k = 128; k > 0; k >>= 1) {
      if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
      __syncthreads();
    }
    if (threadIdx.x == 0) db[0] = red[0];
  }
}

// dZ = dH * silu'(Z), kept in FP32 and BF16.
__global__ void silu_backward_kernel(const float *__restrict__ dH, const float *__restrict__ Z,
                                     float *__restrict__ dZ, __nv_bfloat16 *__restrict__ dZb,
                                     long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float z = Z[i], s = sigmoid_f(z);
  const float d = dH[i] * s * (1.f + z * (1.f - s));
  dZ[i] = d;
  dZb[i] = __float2bfloat16(d);
}

// db[j] = sum_b dZ[b][j] (one block per j).
__global__ void colsum_kernel(const float *__restrict__ dZ, float *__restrict__ db, int B, int N) {
  __shared__ float red[256];
  const int j = blockIdx.x;
  float s = 0.f;
  for (int b = threadIdx.x; b < B; b += blockDim.x) s += dZ[(size_t)b * N + j];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int k = 128; k > 0; k >>= 1) {
    if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) db[j] = red[0];
}

// Adam on the FP32 master parameters (bias-corrected step size lr_t).
__global__ void adam_kernel(float *__restrict__ p, const float *__restrict__ g,
                            float *__restrict__ m, float *__restrict__ v, long long n, float lr_t,
                            float b1, float b2, float eps) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr_t * mi / (sqrtf(vi) + eps);
}

// BF16 copy of a weight matrix [out][in] into [out][in_pad] (zero padded).
__global__ void weights_bf16_kernel(const float *__restrict__ W, __nv_bfloat16 *__restrict__ Wb,
                                    int out, int in, int in_pad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= out * in_pad) return;
  const int o = i / in_pad, k = i % in_pad;
  Wb[i] = __float2bfloat16(k < in ? W[(size_t)o * in + k] : 0.f);
}

__global__ void zero_kernel(float *p, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = 0.f;
}

static int blocks(long long n, int t = 256) { return (int)((n + t - 1) / t); }

}  // namespace axx

using namespace axx;

// ---- host side ---------------------------------------------------------------

namespace {

struct SplitMix64 {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
};

axx_status mfail(axx_ctx *ctx, axx_status s, const std::string &m) {
  if (ctx) ctx->err = m;
  return s;
}

axx_status mcuda(axx_ctx *ctx, cudaError_t e, const char *where) {
  if (ctx) ctx->err = std::string(where) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? AXX_ERR_OUT_OF_MEMORY : AXX_ERR_CUDA;
}

}  // namespace

// Ensures batch buffers for B rows.
static cudaError_t mlp_reserve(axx_mlp *m, int B) {
  if (B <= m->cap) return cudaSuccess;
  if (m->work) cudaFree(m->work);
  m->work = nullptr;
  m->cap = 0;
  const int W = m->width, L = m->depth;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off = (off + bytes + 255) & ~(size_t)255;
    return o;
  };
  const size_t oXb = take((size_t)B * m->in_pad * 2), oT = take((size_t)B * 4),
               oY = take((size_t)B * 4), oDy = take((size_t)B * 4), oC = take((size_t)B * W * 4),
               oZ = take((size_t)L * B * W * 4), oH = take((size_t)L * B * W * 2),
               oDH = take((size_t)B * W * 4), oDZ = take((size_t)B * W * 4),
               oDZb = take((size_t)B * W * 2), oLoss = take(16),
               oKp = take((size_t)kMaxSplitK * W * W * 4);
  cudaError_t e = cudaMalloc(&m->work, off);
  if (e != cudaSuccess) return e;
  char *b = (char *)m->work;
  m->Xb = (__nv_bfloat16 *)(b + oXb);
  m->tb = (float *)(b + oT);
  m->yb = (float *)(b + oY);
  m->dy = (float *)(b + oDy);
  m->Cb = (float *)(b + oC);
  m->kpart = (float *)(b + oKp);
  m->Z = (float *)(b + oZ);
  m->H = (__nv_bfloat16 *)(b + oH);
  m->dH = (float *)(b + oDH);
  m->dZ = (float *)(b + oDZ);
  m->dZb = (__nv_bfloat16 *)(b + oDZb);
  m->loss = (float *)(b + oLoss);
  m->cap = B;
  return cudaSuccess;
}

// Forward of a gathered batch (Xb, B rows) with the mma.sync GEMMs; y into yb.
void mlp_forward_train(axx_mlp *m, int B) {
  cudaStream_t s = m->ctx->stream;
  const int W = m->width;
  for (int l = 0; l < m->depth; ++l) {
    const int in = l == 0 ? m->in_pad : W;
    const __nv_bfloat16 *A = l == 0 ? m->Xb : m->H + (size_t)(l - 1) * B * W;
    gemm_bf16(s, B, W, in, A, in, 1, m->Wb[l], 1, in, m->Cb, W, false, nullptr, m->tc_error);
    bias_silu_kernel<<<blocks((long long)B * W), 256, 0, s>>>(
        m->Cb, m->bias(l), m->Z + (size_t)l * B * W, m->H + (size_t)l * B * W, B, W);
  }
  out_dot_kernel<<<blocks((long long)B * 32), 256, 0, s>>>(
      m->H + (size_t)(m->depth - 1) * B * W, m->weight(m->depth), m->bias(m->depth), m->yb, B, W);
}

// Backward of the batch into m->grad (FP32, params layout); loss into m->loss.
void mlp_backward(axx_mlp *m, int B) {
  cudaStream_t s = m->ctx->stream;
  const int W = m->width, L = m->depth;
  cudaMemsetAsync(m->loss, 0, 4, s);
  loss_grad_kernel<<<blocks(B), 256, 0, s>>>(m->yb, m->tb, m->dy, m->loss, B);
  out_backward_kernel<<<W, 256, 0, s>>>(m->dy, m->H + (size_t)(L - 1) * B * W, m->weight(L),
                                        m->grad_weight(L), m->grad_bias(L), m->dH, B, W);
  for (int l = L - 1; l >= 0; --l) {
    const int in = l == 0 ? m->in_pad : W;
    const int in_true = l == 0 ? m->in_dim : W;
    silu_backward_kernel<<<blocks((long long)B * W), 256, 0, s>>>(
        m->dH, m->Z + (size_t)l * B * W, m->dZ, m->dZb, (long long)B * W);
    colsum_kernel<<<W, 256, 0, s>>>(m->dZ, m->grad_bias(l), B, W);
    // dW_l[n][k] = sum_b dZ[b][n] A[b][k]  (M = W rows n, N = in_true columns k, K = B)
    const __nv_bfloat16 *A = l == 0 ? m->Xb : m->H + (size_t)(l - 1) * B * W;
    gemm_bf16(s, W, in_true, B, m->dZb, 1, W, A, in, 1, m->grad_weight(l), in_true, false,
              m->kpart, m->tc_error);
    if (l > 0) {
      // dH_{l-1}[b][k] = sum_n dZ[b][n] W_l[n][k]
      gemm_bf16(s, B, W, W, m->dZb, W, 1, m->Wb[l], W, 1, m->dH, W, false, nullptr,
                m->tc_error);
    }
  }
}

void mlp_refresh_bf16(axx_mlp *m) {
  cudaStream_t s = m->ctx->stream;
  for (int l = 0; l < m->depth; ++l) {
    const int in = l == 0 ? m->in_dim : m->width, pad = l == 0 ? m->in_pad : m->width;
    weights_bf16_kernel<<<blocks((long long)m->width * pad), 256, 0, s>>>(
        m->weight(l), m->Wb[l], m->width, in, pad);
  }
  mlp_pack_tc(m);
}

extern "C" axx_status axx_mlp_create(axx_ctx *ctx, int in_dim, int width, int depth,
                                     uint64_t seed, axx_mlp **out) {
  if (!ctx || !out) return AXX_ERR_INVALID_ARG;
  *out = nullptr;
  if (in_dim < 1 || in_dim > 64 || width != 256 || depth < 1 || depth > 8)
    return mfail(ctx, AXX_ERR_UNSUPPORTED, "the MLP supports in_dim <= 64, width 256, depth 1-8");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return mcuda(ctx, e, "cudaSetDevice");
  auto *m = new axx_mlp();
  m->ctx = ctx;
  m->in_dim = in_dim;
  m->in_pad = (in_dim + 15) / 16 * 16;
  m->width = width;
  m->depth = depth;
  // parameter layout: per layer W [out][in] then b [out]; layers 0..depth
  long long off = 0;
  for (int l = 0; l <= depth; ++l) {
    const int in = l == 0 ? in_dim : width, outd = l == depth ? 1 : width;
    m->w_off.push_back(off);
    off += (long long)outd * in;
    m->b_off.push_back(off);
    off += outd;
  }
  m->nparam = off;
  std::vector<float> h((size_t)off);
  SplitMix64 rng{seed ^ 0x51A7E5EEDull};
  for (int l = 0; l <= depth; ++l) {
    const int in = l == 0 ? in_dim : width, outd = l == depth ? 1 : width;
    const double bound = 1.0 / std::sqrt((double)in);
    for (long long i = 0; i < (long long)outd * in; ++i)
      h[m->w_off[l] + i] = (float)((2.0 * rng.uniform() - 1.0) * bound);
    for (int i = 0; i < outd; ++i) h[m->b_off[l] + i] = (float)((2.0 * rng.uniform() - 1.0) * bound);
  }
  e = cudaMalloc(&m->params, (size_t)off * 4 * 4);  // params, grad, adam m, adam v
  if (e == cudaSuccess) {
    m->grad = m->params + off;
    m->am = m->grad + off;
    m->av = m->am + off;
    e = cudaMemcpy(m->params, h.data(), (size_t)off * 4, cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) e = cudaMemset(m->am, 0, (size_t)off * 4 * 2);
  size_t wb = 0;
  for (int l = 0; l < depth; ++l) wb += (size_t)width * (l == 0 ? m->in_pad : width);
  if (e == cudaSuccess) e = cudaMalloc(&m->wb_all, wb * 2);
  if (e == cudaSuccess) {
    size_t o = 0;
    for (int l = 0; l < depth; ++l) {
      m->Wb.push_back(m->wb_all + o);
      o += (size_t)width * (l == 0 ? m->in_pad : width);
    }
    e = mlp_tc_init(m);
  }
  if (e == cudaSuccess) e = gemm_tc_init();
  if (e != cudaSuccess) {
    axx_mlp_destroy(m);
    return mcuda(ctx, e, "axx_mlp_create");
  }
  mlp_refresh_bf16(m);
  e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    axx_mlp_destroy(m);
    return mcuda(ctx, e, "axx_mlp_create");
  }
  *out = m;
  return AXX_OK;
}

static void predict_io_free(axx_mlp *m);

extern "C" axx_status axx_mlp_destroy(axx_mlp *m) {
  if (!m) return AXX_OK;
  if (m->ctx) cudaStreamSynchronize(m->ctx->stream);
  predict_io_free(m);
  if (m->params) cudaFree(m->params);
  if (m->wb_all) cudaFree(m->wb_all);
  if (m->work) cudaFree(m->work);
  mlp_tc_free(m);
  delete m;
  return AXX_OK;
}

extern "C" axx_status axx_mlp_num_params(const axx_mlp *m, int64_t *n) {
  if (!m || !n) return AXX_ERR_INVALID_ARG;
  *n = m->nparam;
  return AXX_OK;
}

extern "C" axx_status axx_mlp_get_params(axx_mlp *m, float *params) {
  if (!m || !params) return AXX_ERR_INVALID_ARG;
  cudaError_t e = cudaStreamSynchronize(m->ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpy(params, m->params, (size_t)m->nparam * 4, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return mcuda(m->ctx, e, "axx_mlp_get_params");
  return AXX_OK;
}

extern "C" axx_status axx_mlp_set_params(axx_mlp *m, const float *params) {
  if (!m || !params) return AXX_ERR_INVALID_ARG;
  cudaError_t e = cudaMemcpy(m->params, params, (size_t)m->nparam * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    mlp_refresh_bf16(m);
    e = cudaStreamSynchronize(m->ctx->stream);
  }
  if (e != cudaSuccess) return mcuda(m->ctx, e, "axx_mlp_set_params");
  return AXX_OK;
}

// AXX_ERR_TIMEOUT (and the flag cleared) when a tensor-core completion wait
// of the work just synchronised ran out.
static axx_status tc_status(axx_mlp *m) {
  int tc_err = 0;
  const cudaError_t e = cudaMemcpy(&tc_err, m->tc_error, 4, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return mcuda(m->ctx, e, "reading the tensor-core error flag");
  if (!tc_err) return AXX_OK;
  cudaMemset(m->tc_error, 0, 4);
  return mfail(m->ctx, AXX_ERR_TIMEOUT, "a tensor-core completion wait ran out");
}

static cudaError_t upload_xy(axx_mlp *m, const float *X, const float *y, int n, float **dX,
                             float **dy) {
  cudaError_t e = cudaMalloc(dX, (size_t)n * m->in_dim * 4);
  if (e == cudaSuccess) e = cudaMalloc(dy, (size_t)n * 4);
  if (e == cudaSuccess) e = cudaMemcpy(*dX, X, (size_t)n * m->in_dim * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && y) e = cudaMemcpy(*dy, y, (size_t)n * 4, cudaMemcpyHostToDevice);
  return e;
}

extern "C" axx_status axx_mlp_gradients(axx_mlp *m, const float *X, const float *y, int n,
                                        float *grads, float *loss) {
  if (!m || !X || !y || !grads || n < 1) return AXX_ERR_INVALID_ARG;
  float *dX = nullptr, *dY = nullptr;
  cudaError_t e = mlp_reserve(m, n);
  if (e == cudaSuccess) e = upload_xy(m, X, y, n, &dX, &dY);
  if (e == cudaSuccess) {
    cudaStream_t s = m->ctx->stream;
    gather_kernel<<<blocks(n), 256, 0, s>>>(dX, dY, n, m->in_dim, m->in_pad, n, 0, 0, 0, m->Xb,
                                            m->tb);
    mlp_forward_train(m, n);
    mlp_backward(m, n);
    e = cudaStreamSynchronize(s);
  }
  if (e == cudaSuccess) e = cudaMemcpy(grads, m->grad, (size_t)m->nparam * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && loss) e = cudaMemcpy(loss, m->loss, 4, cudaMemcpyDeviceToHost);
  if (dX) cudaFree(dX);
  if (dY) cudaFree(dY);
  if (e != cudaSuccess) return mcuda(m->ctx, e, "axx_mlp_gradients");
  return tc_status(m);
}

extern "C" axx_status axx_mlp_train(axx_mlp *m, const float *X, const float *y, int n, int batch,
                                    int steps, float lr, uint64_t seed, float *loss_out) {
  if (!m || !X || !y || n < 1 || batch < 1 || steps < 0 || !(lr > 0.f)) return AXX_ERR_INVALID_ARG;
  float *dX = nullptr, *dY = nullptr, *dL = nullptr;
  cudaError_t e = mlp_reserve(m, batch);
  if (e == cudaSuccess) e = upload_xy(m, X, y, n, &dX, &dY);
  if (e == cudaSuccess && loss_out && steps > 0) e = cudaMalloc(&dL, (size_t)steps * 4);
  cudaStream_t s = m->ctx->stream;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int t = 0; t < steps && e == cudaSuccess; ++t) {
    gather_kernel<<<blocks(batch), 256, 0, s>>>(dX, dY, n, m->in_dim, m->in_pad, batch, seed,
                                                (uint32_t)t, 1, m->Xb, m->tb);
    mlp_forward_train(m, batch);
    mlp_backward(m, batch);
    if (dL) cudaMemcpyAsync(dL + t, m->loss, 4, cudaMemcpyDeviceToDevice, s);
    ++m->adam_t;
    const double c1 = 1.0 - std::pow(0.9, (double)m->adam_t),
                 c2 = 1.0 - std::pow(0.999, (double)m->adam_t);
    const float lr_t = (float)(lr * std::sqrt(c2) / c1);
    adam_kernel<<<blocks(m->nparam), 256, 0, s>>>(m->params, m->grad, m->am, m->av, m->nparam,
                                                  lr_t, b1, b2, eps);
    mlp_refresh_bf16(m);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess && dL) e = cudaMemcpy(loss_out, dL, (size_t)steps * 4, cudaMemcpyDeviceToHost);
  if (dX) cudaFree(dX);
  if (dY) cudaFree(dY);
  if (dL) cudaFree(dL);
  if (e != cudaSuccess) return mcuda(m->ctx, e, "axx_mlp_train");
  return tc_status(m);
}

// The device buffers, streams and events of inference from host memory,
// made at the first call and kept (the buffers grown when a call needs more
// rows; every earlier call has drained its streams before returning).
static cudaError_t predict_io(axx_mlp *m, long long n) {
  cudaError_t e = cudaSuccess;
  auto event = [&](cudaEvent_t &ev) {
    if (e == cudaSuccess && !ev) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  };
  if (!m->s_in) e = cudaStreamCreateWithFlags(&m->s_in, cudaStreamNonBlocking);
  if (e == cudaSuccess && !m->s_out) e = cudaStreamCreateWithFlags(&m->s_out, cudaStreamNonBlocking);
  event(m->ev_start);
  for (int i = 0; i < axx_mlp::kMaxChunks; ++i) {
    event(m->ev_in[i]);
    event(m->ev_done[i]);
  }
  if (e == cudaSuccess && n > m->io_rows) {
    if (m->io) cudaFree(m->io);
    m->io = nullptr;
    m->io_rows = 0;
    e = cudaMalloc(&m->io, (size_t)n * (m->in_dim + 1) * 4);
    if (e == cudaSuccess) m->io_rows = n;
  }
  return e;
}

static void predict_io_free(axx_mlp *m) {
  if (m->io) cudaFree(m->io);
  if (m->s_in) cudaStreamDestroy(m->s_in);
  if (m->s_out) cudaStreamDestroy(m->s_out);
  if (m->ev_start) cudaEventDestroy(m->ev_start);
  for (int i = 0; i < axx_mlp::kMaxChunks; ++i) {
    if (m->ev_in[i]) cudaEventDestroy(m->ev_in[i]);
    if (m->ev_done[i]) cudaEventDestroy(m->ev_done[i]);
  }
}

// Inference from host memory as a pipeline of up to four chunks (whole waves
// of the persistent kernel, about a quarter of the rows each): chunk i's
// queries cross on one copy stream while chunk i-1 runs on the context's
// stream, and the outputs come back on another copy stream.  The rows of a
// chunk are computed exactly as in one launch over all rows (every row is
// independent), so the outputs equal axx_mlp_predict_device's bit for bit.
extern "C" axx_status axx_mlp_predict(axx_mlp *m, const float *X, int n, float *y) {
  if (!m || !X || !y || n < 0) return AXX_ERR_INVALID_ARG;
  if (n == 0) return AXX_OK;
  cudaError_t e = predict_io(m, n);
  if (e != cudaSuccess) return mcuda(m->ctx, e, "axx_mlp_predict");
  const cudaStream_t s = m->ctx->stream;
  const long long wave = mlp_tc_rows_per_wave(m), d = m->in_dim;
  const long long chunk = ((n + axx_mlp::kMaxChunks - 1) / axx_mlp::kMaxChunks + wave - 1) / wave * wave;
  const int nch = (int)((n + chunk - 1) / chunk);
  float *dX = m->io, *dY = m->io + (size_t)n * d;
  axx_status st = AXX_OK;
  // the copy streams start after the work already queued on the context
  e = cudaEventRecord(m->ev_start, s);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(m->s_in, m->ev_start, 0);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(m->s_out, m->ev_start, 0);
  int queued = 0;
  for (int i = 0; i < nch && e == cudaSuccess && st == AXX_OK; ++i) {
    const long long r0 = i * chunk, rn = std::min<long long>(chunk, n - r0);
    e = cudaMemcpyAsync(dX + r0 * d, X + r0 * d, (size_t)(rn * d) * 4, cudaMemcpyHostToDevice,
                        m->s_in);
    if (e == cudaSuccess) e = cudaEventRecord(m->ev_in[i], m->s_in);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, m->ev_in[i], 0);
    if (e == cudaSuccess) st = axx_mlp_predict_device(m, dX + r0 * d, (int)rn, dY + r0);
    if (e == cudaSuccess && st == AXX_OK) e = cudaEventRecord(m->ev_done[i], s);
    if (e == cudaSuccess && st == AXX_OK) ++queued;
  }
  // the outputs once every chunk is queued (a copy into pageable memory
  // returns only when it has completed)
  for (int i = 0; i < queued && e == cudaSuccess; ++i) {
    const long long r0 = i * chunk, rn = std::min<long long>(chunk, n - r0);
    e = cudaStreamWaitEvent(m->s_out, m->ev_done[i], 0);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(y + r0, dY + r0, (size_t)rn * 4, cudaMemcpyDeviceToHost, m->s_out);
  }
  // drain all three streams whatever happened: no copy may still touch the
  // caller's memory after the return
  const cudaError_t e_in = cudaStreamSynchronize(m->s_in);
  const cudaError_t e_run = cudaStreamSynchronize(s);
  const cudaError_t e_out = cudaStreamSynchronize(m->s_out);
  if (e == cudaSuccess) e = e_in != cudaSuccess ? e_in : (e_run != cudaSuccess ? e_run : e_out);
  int tc_err = 0;
  if (e == cudaSuccess && st == AXX_OK) e = cudaMemcpy(&tc_err, m->tc_error, 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && st == AXX_OK && tc_err) {
    cudaMemset(m->tc_error, 0, 4);
    st = mfail(m->ctx, AXX_ERR_TIMEOUT, "a tensor-core completion wait ran out");
  }
  if (st != AXX_OK) return st;
  if (e != cudaSuccess) return mcuda(m->ctx, e, "axx_mlp_predict");
  return AXX_OK;
}

extern "C" axx_status axx_mlp_flops_per_row(const axx_mlp *m, double *flops) {
  if (!m || !flops) return AXX_ERR_INVALID_ARG;
  double f = 2.0 * m->in_dim * m->width + 2.0 * m->width;
  f += (m->depth - 1) * 2.0 * m->width * m->width;
  *flops = f;
  return AXX_OK;
}
