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

// Poisson deviance of predictions y = log(mu) against non-negative targets
// t: loss = mean(exp(y) - t y), dy = (exp(y) - t) / n.  Its minimiser is
// y = log E[t | input], the log of a conditional mean, where a squared error
// on log t would give E[log t | input].  y is clamped to <= 30 in exp.
__global__ void poisson_grad_kernel(const float* __restrict__ y, const float* __restrict__ t, int64_t n,
                                    float* __restrict__ dy, double* __restrict__ partial) {
  double acc = 0.0;
  const float inv = 1.f / (float)n;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float e = expf(fminf(y[i], 30.f));
    dy[i] = inv * (e - t[i]);
    acc += (double)e - (double)t[i] * (double)y[i];
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

// ---- inference on the tensor cores ----------------------------------------------
// For networks dims = (d0 <= 16, 128, ..., 128, 1): the first layer (K = d0)
// and the last (128 -> 1) on the CUDA cores, every 128 x 128 hidden layer as
// one tcgen05.mma GEMM per tile of 128 rows: A = the tile's activations
// (BF16, M = 128 rows x K = 128), B = the layer's weights W[k][n] (BF16,
// N = 128 x K = 128), D in tensor memory (FP32, 128 lanes x 128 columns);
// bias and tanh applied on the way back (tcgen05.ld), the result written as
// the next layer's A.  Both operands are MN-major in 128B-swizzled shared
// memory (8-row atoms of 1 KB along K; two 64-element atom columns 16 KB
// apart along M or N), K advancing by 16 per MMA.  One persistent CTA per SM
// keeps every hidden layer's weights in shared memory and walks the tiles.
#include "tc_common.cuh"

namespace {

namespace mi {
constexpr int kWidth = 128;
constexpr int kMaxIn = 16;
constexpr int kMaxTc = 4;                       // hidden 128 x 128 layers
constexpr int kAtomCol = 128 * 128;             // 128 K rows x 128 B
constexpr int kMat = 2 * kAtomCol;              // one 128 x 128 BF16 operand
constexpr int kThreads = 256;
constexpr uint32_t kIdesc = hermes::tc::idesc_bf16_f32(128, 128, true, true);

__host__ __device__ constexpr size_t smem_bytes(int n_tc) {
  return 1024 + (size_t)(n_tc + 1) * kMat + sizeof(float) * (kMaxIn * kWidth + (kMaxTc + 2) * kWidth + kWidth +
                                                              128 * kMaxIn + 2 * 128) + 128;
}
}  // namespace mi

struct MlpTcArgs {
  const float* params;
  const float* x;
  float* y;
  int64_t batch;
  int d0, n_tc;
  int64_t off_w[kMaxLayers], off_b[kMaxLayers];
  int* status;
};

// Byte offset of element (mn, k) in an MN-major 128B-swizzled BF16 operand.
__device__ __forceinline__ uint32_t mi_off(int mn, int k) {
  return (uint32_t)(mn >> 6) * mi::kAtomCol + (uint32_t)(k >> 3) * 1024u +
         hermes::tc::sw128_offset((uint32_t)(k & 7), (uint32_t)((mn & 63) >> 3)) + (uint32_t)(mn & 7) * 2u;
}

__device__ __forceinline__ void mi_put(unsigned char* op, int mn, int k, float v) {
  *reinterpret_cast<__nv_bfloat16*>(op + mi_off(mn, k)) = __float2bfloat16_rn(v);
}

__global__ void __launch_bounds__(mi::kThreads, 1) mlp_infer_tc_kernel(MlpTcArgs A) {
  namespace tc = hermes::tc;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char* base = smem_raw + ((1024u - (tc::smem_u32(smem_raw) & 1023u)) & 1023u);
  unsigned char* wop = base;                                    // [n_tc][kMat] hidden weights
  unsigned char* aop = wop + (size_t)A.n_tc * mi::kMat;         // activations of the tile
  float* w1 = reinterpret_cast<float*>(aop + mi::kMat);         // [d0][128]
  float* bias = w1 + mi::kMaxIn * mi::kWidth;                   // [n_tc + 1][128], then the last bias
  float* wl = bias + (mi::kMaxTc + 2) * mi::kWidth;             // [128] last layer
  float* xt = wl + mi::kWidth;                                  // [128][d0]
  float* red = xt + 128 * mi::kMaxIn;                           // [2][128]
  uint64_t* bar = reinterpret_cast<uint64_t*>(red + 2 * 128);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar + 1);
  int* s_abort = reinterpret_cast<int*>(tmem_slot + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int d0 = A.d0, n_tc = A.n_tc;
  const float* P = A.params;
  // weights: hidden layers as BF16 operands, the rest as float
  for (int l = 0; l < n_tc; ++l) {
    const float* W = P + A.off_w[l + 1];
    unsigned char* op = wop + (size_t)l * mi::kMat;
    for (int i = tid; i < mi::kWidth * mi::kWidth; i += mi::kThreads) {
      const int k = i >> 7, n = i & 127;
      mi_put(op, n, k, W[i]);
    }
  }
  for (int i = tid; i < d0 * mi::kWidth; i += mi::kThreads) w1[i] = P[A.off_w[0] + i];
  for (int l = 0; l <= n_tc; ++l)
    for (int i = tid; i < mi::kWidth; i += mi::kThreads) bias[l * mi::kWidth + i] = P[A.off_b[l] + i];
  for (int i = tid; i < mi::kWidth; i += mi::kThreads) wl[i] = P[A.off_w[n_tc + 1] + i];
  const float b_last = P[A.off_b[n_tc + 1]];
  if (tid == 0) {
    tc::mbar_init(bar, 1);
    tc::mbar_fence_init();
    *s_abort = 0;
  }
  if (warp == 0) tc::tmem_alloc(tmem_slot, 128);
  tc::fence_proxy_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t sw = tc::smem_u32(wop), sa = tc::smem_u32(aop);
  uint32_t phase = 0;
  const int64_t ntiles = (A.batch + 127) / 128;
  // epilogue mapping: lane quarter (rows) and column half
  const int quarter = warp & 3, chalf = warp >> 2;
  const int erow = quarter * 32 + lane;

  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int64_t r0 = t * 128;
    for (int i = tid; i < 128 * d0; i += mi::kThreads) {
      const int64_t r = r0 + i / d0;
      xt[i] = r < A.batch ? A.x[r * d0 + i % d0] : 0.f;
    }
    __syncthreads();
    {  // layer 0 on the CUDA cores: row m, outputs [64 h, 64 h + 64)
      const int m = tid & 127, h = tid >> 7;
      float xv[mi::kMaxIn];
#pragma unroll
      for (int k = 0; k < mi::kMaxIn; ++k) xv[k] = k < d0 ? xt[m * d0 + k] : 0.f;
      for (int j = 0; j < 64; ++j) {
        const int n = 64 * h + j;
        float z = bias[n];
#pragma unroll
        for (int k = 0; k < mi::kMaxIn; ++k)
          if (k < d0) z = fmaf(xv[k], w1[k * mi::kWidth + n], z);
        mi_put(aop, m, n, tanhf(z));
      }
    }
    tc::fence_proxy_async_smem();
    __syncthreads();
    for (int l = 0; l < n_tc; ++l) {
      if (tid == 0) {
        tc::tc_fence_after();
#pragma unroll
        for (int kk = 0; kk < 8; ++kk) {
          const uint64_t ad = tc::smem_desc(sa + kk * 2048, mi::kAtomCol, 1024, tc::kLayoutSw128);
          const uint64_t bd = tc::smem_desc(sw + (uint32_t)l * mi::kMat + kk * 2048, mi::kAtomCol, 1024,
                                            tc::kLayoutSw128);
          tc::mma_bf16(tmem, ad, bd, mi::kIdesc, kk > 0);
        }
        tc::mma_commit(bar);
      }
      if (!tc::mbar_wait(bar, phase)) *s_abort = 1;
      phase ^= 1u;
      tc::tc_fence_after();
      const float* bl = bias + (l + 1) * mi::kWidth;
      float part = 0.f;
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        float d[32];
        const int c0 = chalf * 64 + j * 32;
        tc::tmem_ld_32x32b_x32(tmem + ((uint32_t)(quarter * 32) << 16) + c0, d);
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          const float v = tanhf(d[i] + bl[c0 + i]);
          if (l + 1 < n_tc) mi_put(aop, erow, c0 + i, v);
          else part = fmaf(v, wl[c0 + i], part);
        }
      }
      if (l + 1 == n_tc) red[chalf * 128 + erow] = part;
      tc::fence_proxy_async_smem();
      tc::tc_fence_before();
      __syncthreads();
      if (*s_abort) break;
    }
    if (*s_abort) break;
    if (tid < 128 && r0 + tid < A.batch) A.y[r0 + tid] = red[tid] + red[128 + tid] + b_last;
    __syncthreads();  // xt / red / aop idle before the next tile
  }
  if (*s_abort && tid == 0 && A.status) atomicExch(A.status, 1);
  __syncthreads();
  if (warp == 0) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, 128);
  }
}

}  // namespace

extern "C" int hermes_mlp_infer_tc(const float* params, const int32_t* dims, int n_layers, const float* x,
                                   int64_t batch, float* y, int* status, void* stream) {
  if (!params || !dims || !x || !y || !status) return fail(HERMES_ERR_INVALID, "mlp_infer_tc: NULL argument");
  if (n_layers < 3 || n_layers - 2 > mi::kMaxTc)
    return fail(HERMES_ERR_UNSUPPORTED, "mlp_infer_tc: needs 3..%d layers", mi::kMaxTc + 2);
  if (dims[0] < 1 || dims[0] > mi::kMaxIn || dims[n_layers] != 1)
    return fail(HERMES_ERR_UNSUPPORTED, "mlp_infer_tc: needs 1..%d inputs and one output", mi::kMaxIn);
  for (int l = 1; l < n_layers; ++l)
    if (dims[l] != mi::kWidth) return fail(HERMES_ERR_UNSUPPORTED, "mlp_infer_tc: hidden widths must be 128");
  if (batch < 0) return fail(HERMES_ERR_INVALID, "mlp_infer_tc: batch < 0");
  cudaStream_t s = hermes::as_stream(stream);
  HERMES_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), s));
  if (batch == 0) return HERMES_OK;
  MlpTcArgs A;
  A.params = params;
  A.x = x;
  A.y = y;
  A.batch = batch;
  A.d0 = dims[0];
  A.n_tc = n_layers - 2;
  A.status = status;
  int64_t off = 0;
  for (int l = 0; l < n_layers; ++l) {
    A.off_w[l] = off;
    off += (int64_t)dims[l] * dims[l + 1];
    A.off_b[l] = off;
    off += dims[l + 1];
  }
  const size_t smem = mi::smem_bytes(A.n_tc);
  static bool smem_set[64] = {false};
  int dev = 0, nsm = 148;
  HERMES_CUDA_TRY(cudaGetDevice(&dev));
  HERMES_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  if (dev < 0 || dev >= 64 || !smem_set[dev]) {  // once per device, before any stream capture
    HERMES_CUDA_TRY(cudaFuncSetAttribute(mlp_infer_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)mi::smem_bytes(mi::kMaxTc)));
    if (dev >= 0 && dev < 64) smem_set[dev] = true;
  }
  const int64_t ntiles = (batch + 127) / 128;
  const int grid = (int)(ntiles < nsm ? ntiles : nsm);
  mlp_infer_tc_kernel<<<grid, mi::kThreads, smem, s>>>(A);
  HERMES_LAUNCH_CHECK("mlp_infer_tc_kernel");
  return HERMES_OK;
}

extern "C" int hermes_poisson_grad(const float* y, const float* target, int64_t n, float* dy, double* loss_out,
                                   double* scratch, void* stream) {
  if (!y || !target || !dy || !loss_out || !scratch) return fail(HERMES_ERR_INVALID, "poisson_grad: NULL argument");
  cudaStream_t s = hermes::as_stream(stream);
  HERMES_CUDA_TRY(cudaMemsetAsync(scratch, 0, sizeof(double), s));
  if (n > 0) {
    poisson_grad_kernel<<<256, 256, 0, s>>>(y, target, n, dy, scratch);
    HERMES_LAUNCH_CHECK("poisson_grad_kernel");
  }
  HERMES_CUDA_TRY(cudaMemcpyAsync(loss_out, scratch, sizeof(double), cudaMemcpyDeviceToHost, s));
  HERMES_CUDA_TRY(cudaStreamSynchronize(s));
  *loss_out = n > 0 ? *loss_out / (double)n : 0.0;
  return HERMES_OK;
}
