// Generic multi-bin pair-product pass (Parseval): the kernel template and its
// per-NP launchers.  Each NP (spectrum pairs handled together) is
// instantiated in its own translation unit (pair_products_np1.cu ..
// pair_products_np4.cu): the kernel inlines the full window evaluation four
// times, so one unit holding all four took most of the library's build time.
#pragma once

#include "hermes_common.cuh"
#include "window_eval.cuh"

namespace hermes {

constexpr int kPPThreads = 256;
constexpr int kPPModesPerThread = 16;
constexpr int kMaxPairs = 4;
constexpr int kBinsPerGroup = 4;

struct PPArgs {
  const float2* si[kMaxPairs];  // first spectrum of pair p
  const float2* sj[kMaxPairs];  // second spectrum of pair p
  int n_pairs;
  int L;
  int bw, np;
  int n_bins;
  int exclude_k0;
  int complex_k;  // any bin with a complex kernel
};

// grid.x: mode blocks; grid.y: bin groups.  partial[(blockIdx.x * n_bins + b) * n_pairs + p].
// NP = number of (i, j) spectrum pairs handled together (compile-time).
template <int NP>
__global__ void __launch_bounds__(kPPThreads, 2)
pair_products_kernel(PPArgs a, const WinDev* __restrict__ wins, const double* __restrict__ pd,
                     double* __restrict__ partial, double* __restrict__ k0) {
  extern __shared__ float P[];
  __shared__ double red[kPPThreads / 32][kBinsPerGroup * NP];
  for (int i = threadIdx.x; i < a.np; i += blockDim.x) P[i] = (float)pd[i];
  __syncthreads();
  const int L = a.L, H = L / 2 + 1;
  const long long total = (long long)L * L * H;
  const int b0 = blockIdx.y * kBinsPerGroup;
  const int nb = min(kBinsPerGroup, a.n_bins - b0);
  if (blockIdx.x == 0 && threadIdx.x < nb) k0[b0 + threadIdx.x] = (double)kernel_value(wins[b0 + threadIdx.x], 0, 0, 0, L, P, a.bw).x;
  double acc[kBinsPerGroup][NP];
#pragma unroll
  for (int b = 0; b < kBinsPerGroup; ++b)
#pragma unroll
    for (int p = 0; p < NP; ++p) acc[b][p] = 0.0;

  const long long base = (long long)blockIdx.x * kPPThreads * kPPModesPerThread;
  float fac[kBinsPerGroup][NP];
#pragma unroll
  for (int b = 0; b < kBinsPerGroup; ++b)
#pragma unroll
    for (int p = 0; p < NP; ++p) fac[b][p] = 0.f;
  for (int it = 0; it < kPPModesPerThread; ++it) {
    const long long m = base + (long long)it * kPPThreads + threadIdx.x;
    if (m >= total) break;
    const int z = (int)(m % H);
    const long long r = m / H;
    const int y = (int)(r % L), x = (int)(r / L);
    if (a.exclude_k0 && m == 0) continue;
    const float wgt = (z == 0 || z == L / 2) ? 1.f : 2.f;
    float tr[NP], ti[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      if (true) {
        const float2 u = a.si[p][m], v = a.sj[p][m];
        tr[p] = wgt * (u.x * v.x + u.y * v.y);   // Re(u conj v)
        ti[p] = wgt * (u.y * v.x - u.x * v.y);   // Im(u conj v)
      } else {
        tr[p] = 0.f;
        ti[p] = 0.f;
      }
    }
#pragma unroll
    for (int b = 0; b < kBinsPerGroup; ++b) {
      if (b < nb) {
        const float2 K = kernel_value(wins[b0 + b], x, y, z, L, P, a.bw);
#pragma unroll
        for (int p = 0; p < NP; ++p)
          fac[b][p] += tr[p] * K.x - ti[p] * K.y;
      }
    }
    if ((it & 3) == 3) {  // fold float32 partials into float64 every 4 modes
#pragma unroll
      for (int b = 0; b < kBinsPerGroup; ++b)
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          acc[b][p] += (double)fac[b][p];
          fac[b][p] = 0.f;
        }
    }
  }
#pragma unroll
  for (int b = 0; b < kBinsPerGroup; ++b)
#pragma unroll
    for (int p = 0; p < NP; ++p) acc[b][p] += (double)fac[b][p];

  // block reduction (fixed order -> deterministic)
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int b = 0; b < kBinsPerGroup; ++b)
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      double v = acc[b][p];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) red[wid][b * NP + p] = v;
    }
  __syncthreads();
  if (threadIdx.x < nb * NP) {
    const int b = threadIdx.x / NP, p = threadIdx.x % NP;
    double s = 0.0;
    for (int w = 0; w < kPPThreads / 32; ++w) s += red[w][b * NP + p];
    partial[((long long)blockIdx.x * a.n_bins + b0 + b) * a.n_pairs + p] = s;
  }
}

#define HERMES_PP_LAUNCHER(NP)                                                                                 \
  cudaError_t launch_pair_products_##NP(dim3 grid, size_t smem, cudaStream_t s, const PPArgs& a,           \
                                          const WinDev* wins, const double* pd, double* partial, double* k0)
HERMES_PP_LAUNCHER(1);
HERMES_PP_LAUNCHER(2);
HERMES_PP_LAUNCHER(3);
HERMES_PP_LAUNCHER(4);

}  // namespace hermes
