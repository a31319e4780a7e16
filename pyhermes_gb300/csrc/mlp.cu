// Small fully connected network (the learned importance-sampling proposal of
// the Monte Carlo 3PCF): forward, backward, MSE gradient and Adam, written as
// plain CUDA kernels.  No reference counterpart (the reference samples
// triangle centres uniformly, corr3pcf_kernels.py:66-140); the estimator that
// uses it stays unbiased through importance weights.
//
// Parameters are one float32 array: for each layer l, W_l [in_l][out_l]
// (row-major) then b_l [out_l].  Hidden layers use tanh, the last layer is
// linear.  Widths are <= 128.  Inference can read bfloat16 copies of the
// weights (float32 accumulation).
#include <cuda_bf16.h>

#include "hermes_common.cuh"

namespace {

using hermes::fail;

constexpr int kMaxWidth = 128;
constexpr int kMaxLayers = 8;
constexpr int kRows = 32;  // rows per CTA in the dense kernels

struct Dims {
  int n_layers;
  int d[kMaxLayers + 1];
};

__device__ __forceinline__ float act_fwd(float z, bool tanh_act) { return tanh_act ? tanhf(z) : z; }

// Y[b][n] = act(sum_k X[b][k] W[k][n] + bias[n]); 256 threads, kRows rows per CTA.
template <typename WT>
__global__ void __launch_bounds__(256)
dense_fwd_kernel(const float* __restrict__ X, int64_t B, int K, int N, const WT* __restrict__ W,
                 const WT* __restrict__ bias, bool tanh_act, float* __restrict__ Y) {
  extern __shared__ float dsm[];
  float* sW = dsm;               // K * N
  float* sX = sW + K * N;        // kRows * K
  float* sb = sX + kRows * K;    // N
  for (int i = threadIdx.x; i < K * N; i += blockDim.x) sW[i] = (float)W[i];
  for (int i = threadIdx.x; i < N; i += blockDim.x) sb[i] = (float)bias[i];
  const int64_t r0 = (int64_t)blockIdx.x * kRows;
  for (int i = threadIdx.x; i < kRows * K; i += blockDim.x) {
    const int64_t r = r0 + i / K;
    sX[i] = r < B ? X[r * K + i % K] : 0.f;
  }
  __syncthreads();
  const int row = threadIdx.x >> 3, lane8 = threadIdx.x & 7;
  const int64_t r = r0 + row;
  float acc[kMaxWidth / 8];
#pragma unroll
  for (int j = 0; j < kMaxWidth / 8; ++j) acc[j] = 0.f;
  for (int k = 0; k < K; ++k) {
    const float xv = sX[row * K + k];
#pragma unroll
    for (int j = 0; j < kMaxWidth / 8; ++j) {
      const int c = lane8 + 8 * j;
      if (c < N) acc[j] = fmaf(xv, sW[k * N + c], acc[j]);
    }
  }
  if (r < B) {
#pragma unroll
    for (int j = 0; j < kMaxWidth / 8; ++j) {
      const int c = lane8 + 8 * j;
      if (c < N) Y[r * N + c] = act_fwd(acc[j] + sb[c], tanh_act);
    }
  }
}

// dZ = dY * act'(.) (tanh' = 1 - Y^2) written to dZ; dX = dZ W^T.
__global__ void __launch_bounds__(256)
dense_bwd_data_kernel(const float* __restrict__ dY, const float* __restrict__ Y, int64_t B, int K, int N,
                      const float* __restrict__ W, bool tanh_act, float* __restrict__ dZ, float* __restrict__ dX) {
  extern __shared__ float dsm[];
  float* sW = dsm;          // K * N
  float* sZ = sW + K * N;   // kRows * N
  for (int i = threadIdx.x; i < K * N; i += blockDim.x) sW[i] = W[i];
  const int64_t r0 = (int64_t)blockIdx.x * kRows;
  for (int i = threadIdx.x; i < kRows * N; i += blockDim.x) {
    const int64_t r = r0 + i / N;
    float z = 0.f;
    if (r < B) {
      const int64_t g = r * N + i % N;
      z = dY[g];
      if (tanh_act) {
        const float y = Y[g];
        z *= 1.f - y * y;
      }
      dZ[g] = z;
    }
    sZ[i] = z;
  }
  __syncthreads();
  if (!dX) return;
  const int row = threadIdx.x >> 3, lane8 = threadIdx.x & 7;
  const int64_t r = r0 + row;
  float acc[kMaxWidth / 8];
#pragma unroll
  for (int j = 0; j < kMaxWidth / 8; ++j) acc[j] = 0.f;
  for (int n = 0; n < N; ++n) {
    const float zv = sZ[row * N + n];
#pragma unroll
    for (int j = 0; j < kMaxWidth / 8; ++j) {
      const int k = lane8 + 8 * j;
      if (k < K) acc[j] = fmaf(zv, sW[k * N + n], acc[j]);
    }
  }
  if (r < B) {
#pragma unroll
    for (int j = 0; j < kMaxWidth / 8; ++j) {
      const int k = lane8 + 8 * j;
      if (k < K) dX[r * K + k] = acc[j];
    }
  }
}

// dW[k][n] += sum_b X[b][k] dZ[b][n], db[n] += sum_b dZ[b][n] over a chunk of rows.
constexpr int kWChunk = 256;
__global__ void __launch_bounds__(256)
dense_bwd_weight_kernel(const float* __restrict__ X, const float* __restrict__ dZ, int64_t B, int K, int N,
                        float* __restrict__ dW, float* __restrict__ db) {
  __shared__ float sX[32 * kMaxWidth];
  __shared__ float sZ[32 * kMaxWidth];
  const int pairs = K * N;
  float acc[64];
#pragma unroll
  for (int j = 0; j < 64; ++j) acc[j] = 0.f;
  float bacc = 0.f;
  const int64_t c0 = (int64_t)blockIdx.x * kWChunk;
  for (int64_t s = c0; s < c0 + kWChunk && s < B; s += 32) {
    __syncthreads();
    for (int i = threadIdx.x; i < 32 * K; i += blockDim.x) {
      const int64_t r = s + i / K;
      sX[i] = (r < B && r < c0 + kWChunk) ? X[r * K + i % K] : 0.f;
    }
    for (int i = threadIdx.x; i < 32 * N; i += blockDim.x) {
      const int64_t r = s + i / N;
      sZ[i] = (r < B && r < c0 + kWChunk) ? dZ[r * N + i % N] : 0.f;
    }
    __syncthreads();
    for (int rr = 0; rr < 32; ++rr) {
#pragma unroll
      for (int j = 0; j < 64; ++j) {
        const int p = threadIdx.x + 256 * j;
        if (p < pairs) acc[j] = fmaf(sX[rr * K + p / N], sZ[rr * N + p % N], acc[j]);
      }
      if (threadIdx.x < N) bacc += sZ[rr * N + threadIdx.x];
    }
  }
#pragma unroll
  for (int j = 0; j < 64; ++j) {
    const int p = threadIdx.x + 256 * j;
    if (p < pairs) atomicAdd(&dW[p], acc[j]);
  }
  if (threadIdx.x < N) atomicAdd(&db[threadIdx.x], bacc);
}

__global__ void mse_grad_kernel(const float* __restrict__ y, const float* __restrict__ t, int64_t n,
                                float* __restrict__ dy, double* __restrict__ partial) {
  double acc = 0.0;
  const float inv = 2.f / (float)n;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float d = y[i] - t[i];
    dy[i] = inv * d;
    acc += (double)d * (double)d;
  }
  __shared__ double sh[256];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(partial, sh[0]);
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, int64_t n, float lr, float b1, float b2, float eps, float c1,
                            float c2) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

__global__ void to_bf16_kernel(const float* __restrict__ p, int64_t n, __nv_bfloat16* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = __float2bfloat16_rn(p[i]);
}

int check_dims(const int32_t* dims, int n_layers, Dims* d, int64_t* n_params) {
  if (!dims || n_layers < 1 || n_layers > kMaxLayers) return fail(HERMES_ERR_INVALID, "mlp: n_layers=%d", n_layers);
  d->n_layers = n_layers;
  int64_t np = 0;
  for (int i = 0; i <= n_layers; ++i) {
    if (dims[i] < 1 || dims[i] > kMaxWidth) return fail(HERMES_ERR_INVALID, "mlp: width %d outside [1,%d]", dims[i], kMaxWidth);
    d->d[i] = dims[i];
    if (i > 0) np += (int64_t)dims[i - 1] * dims[i] + dims[i];
  }
  *n_params = np;
  return HERMES_OK;
}

int grid_rows(int64_t B) { return (int)((B + kRows - 1) / kRows); }

size_t fwd_smem(int K, int N) { return sizeof(float) * ((size_t)K * N + (size_t)kRows * K + N); }
size_t bwd_smem(int K, int N) { return sizeof(float) * ((size_t)K * N + (size_t)kRows * N); }

int set_smem_limits() {
  static bool done = false;
  if (done) return HERMES_OK;
  const int big = (int)(sizeof(float) * (kMaxWidth * kMaxWidth + kRows * kMaxWidth + kMaxWidth));
  HERMES_CUDA_TRY(cudaFuncSetAttribute(dense_fwd_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  HERMES_CUDA_TRY(cudaFuncSetAttribute(dense_fwd_kernel<__nv_bfloat16>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  HERMES_CUDA_TRY(cudaFuncSetAttribute(dense_bwd_data_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  done = true;
  return HERMES_OK;
}

}  // namespace

extern "C" int hermes_mlp_param_count(const int32_t* dims, int n_layers, int64_t* n_params) {
  Dims d;
  if (!n_params) return fail(HERMES_ERR_INVALID, "mlp: n_params is NULL");
  return check_dims(dims, n_layers, &d, n_params);
}

extern "C" int hermes_mlp_forward(const float* params, const void* params_bf16, const int32_t* dims, int n_layers,
                                  const float* x, int64_t batch, float* acts, void* stream) {
  Dims d;
  int64_t np = 0;
  int rc = check_dims(dims, n_layers, &d, &np);
  if (rc) return rc;
  if ((!params && !params_bf16) || !x || !acts) return fail(HERMES_ERR_INVALID, "mlp_forward: NULL argument");
  if (batch <= 0) return HERMES_OK;
  if (batch > (1LL << 31) / kMaxWidth) return fail(HERMES_ERR_INVALID, "mlp_forward: batch too large");
  cudaStream_t s = hermes::as_stream(stream);
  rc = set_smem_limits();
  if (rc) return rc;
  const float* in = x;
  float* out = acts;
  int64_t off = 0;
  for (int l = 0; l < n_layers; ++l) {
    const int K = d.d[l], N = d.d[l + 1];
    const bool tanh_act = l + 1 < n_layers;
    if (params_bf16) {
      const __nv_bfloat16* pw = static_cast<const __nv_bfloat16*>(params_bf16) + off;
      dense_fwd_kernel<__nv_bfloat16><<<grid_rows(batch), 256, fwd_smem(K, N), s>>>(in, batch, K, N, pw, pw + (int64_t)K * N,
                                                                       tanh_act, out);
    } else {
      const float* pw = params + off;
      dense_fwd_kernel<float><<<grid_rows(batch), 256, fwd_smem(K, N), s>>>(in, batch, K, N, pw, pw + (int64_t)K * N, tanh_act,
                                                              out);
    }
    HERMES_LAUNCH_CHECK("dense_fwd_kernel");
    off += (int64_t)K * N + N;
    in = out;
    out += batch * N;
  }
  return HERMES_OK;
}

extern "C" int hermes_mlp_backward(const float* params, const int32_t* dims, int n_layers, const float* x,
                                   int64_t batch, const float* acts, const float* dy, float* grads, float* scratch,
                                   void* stream) {
  Dims d;
  int64_t np = 0;
  int rc = check_dims(dims, n_layers, &d, &np);
  if (rc) return rc;
  if (!params || !x || !acts || !dy || !grads || !scratch) return fail(HERMES_ERR_INVALID, "mlp_backward: NULL argument");
  if (batch <= 0) return HERMES_OK;
  cudaStream_t s = hermes::as_stream(stream);
  rc = set_smem_limits();
  if (rc) return rc;
  HERMES_CUDA_TRY(cudaMemsetAsync(grads, 0, sizeof(float) * np, s));
  // offsets of each layer's parameters and activations
  int64_t poff[kMaxLayers], aoff[kMaxLayers];
  int64_t p = 0, a = 0;
  for (int l = 0; l < n_layers; ++l) {
    poff[l] = p;
    aoff[l] = a;
    p += (int64_t)d.d[l] * d.d[l + 1] + d.d[l + 1];
    a += batch * d.d[l + 1];
  }
  // scratch: two ping-pong buffers of batch * 128 floats (dZ and dX)
  float* bufZ = scratch;
  float* bufX = scratch + batch * kMaxWidth;
  float* bufY = scratch + 2 * batch * kMaxWidth;
  const float* cur_dy = dy;
  for (int l = n_layers - 1; l >= 0; --l) {
    const int K = d.d[l], N = d.d[l + 1];
    const bool tanh_act = l + 1 < n_layers;
    const float* Yl = acts + aoff[l];
    const float* Xl = l == 0 ? x : acts + aoff[l - 1];
    float* dX = l == 0 ? nullptr : bufX;
    dense_bwd_data_kernel<<<grid_rows(batch), 256, bwd_smem(K, N), s>>>(cur_dy, Yl, batch, K, N, params + poff[l], tanh_act,
                                                           bufZ, dX);
    HERMES_LAUNCH_CHECK("dense_bwd_data_kernel");
    const int wg = (int)((batch + kWChunk - 1) / kWChunk);
    dense_bwd_weight_kernel<<<wg, 256, 0, s>>>(Xl, bufZ, batch, K, N, grads + poff[l], grads + poff[l] + (int64_t)K * N);
    HERMES_LAUNCH_CHECK("dense_bwd_weight_kernel");
    if (dX) {
      // the next (lower) layer's dY is this dX; move it out of the way of bufX
      float* t = bufY;
      bufY = bufX;
      bufX = t;
      cur_dy = bufY;
    }
  }
  return HERMES_OK;
}

extern "C" int hermes_mlp_scratch_floats(int64_t batch, int64_t* n) {
  if (!n) return fail(HERMES_ERR_INVALID, "n is NULL");
  *n = 3 * batch * kMaxWidth;
  return HERMES_OK;
}

extern "C" int hermes_mse_grad(const float* y, const float* target, int64_t n, float* dy, double* loss_out,
                               double* scratch, void* stream) {
  if (!y || !target || !dy || !loss_out || !scratch) return fail(HERMES_ERR_INVALID, "mse_grad: NULL argument");
  cudaStream_t s = hermes::as_stream(stream);
  HERMES_CUDA_TRY(cudaMemsetAsync(scratch, 0, sizeof(double), s));
  if (n > 0) {
    mse_grad_kernel<<<256, 256, 0, s>>>(y, target, n, dy, scratch);
    HERMES_LAUNCH_CHECK("mse_grad_kernel");
  }
  HERMES_CUDA_TRY(cudaMemcpyAsync(loss_out, scratch, sizeof(double), cudaMemcpyDeviceToHost, s));
  HERMES_CUDA_TRY(cudaStreamSynchronize(s));
  *loss_out = n > 0 ? *loss_out / (double)n : 0.0;
  return HERMES_OK;
}

extern "C" int hermes_adam_step(float* params, const float* grads, float* m, float* v, int64_t n, float lr, float b1,
                                float b2, float eps, int step, void* stream) {
  if (!params || !grads || !m || !v || step < 1) return fail(HERMES_ERR_INVALID, "adam: bad argument");
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  adam_kernel<<<256, 256, 0, hermes::as_stream(stream)>>>(params, grads, m, v, n, lr, b1, b2, eps, c1, c2);
  HERMES_LAUNCH_CHECK("adam_kernel");
  return HERMES_OK;
}

extern "C" int hermes_to_bf16(const float* in, int64_t n, void* out, void* stream) {
  if (!in || !out) return fail(HERMES_ERR_INVALID, "to_bf16: NULL argument");
  to_bf16_kernel<<<256, 256, 0, hermes::as_stream(stream)>>>(in, n, static_cast<__nv_bfloat16*>(out));
  HERMES_LAUNCH_CHECK("to_bf16_kernel");
  return HERMES_OK;
}
