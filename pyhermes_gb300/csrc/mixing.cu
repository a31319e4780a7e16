// Edge-correction mixing solve for 3PCF multipoles, float64 on the GPU.
//
// Restates pyhermes/utils/special_functions.py:366-409 for every (r12, r13)
// sample at once: M = B0 (I + F) with
//   F[0][l] = f_l / (2l + 1)                      (l >= 1)
//   F[k][l] = sum_{l' >= 1} G(l, l', k) f_{l'}    (k >= 1),   f = B / B0,
// cond_2(M) (numpy.linalg.cond) and C = M^{-1} A (numpy.linalg.solve).
// One warp per sample.  The solve is LU with partial pivoting (first row of
// largest |pivot|, as LAPACK's idamax) and back substitution; the condition
// number is sigma_max / sigma_min from a one-sided Jacobi SVD (Hestenes'
// method: rotate column pairs until they are mutually orthogonal, then the
// singular values are the column norms).  Reductions run in a fixed lane
// order, so results are deterministic.
#include "hermes_common.cuh"

namespace {

using hermes::fail;

constexpr int kMaxN = 32;       // lmax + 1 <= 32
constexpr int kLd = kMaxN + 1;  // padded row length in shared memory
constexpr int kJacobiSweeps = 60;

// Butterfly sum: every lane ends with the same value (each step adds the same
// pair of operands on both partner lanes).
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void __launch_bounds__(32)
mixing_kernel(const double* __restrict__ A, const double* __restrict__ B, const double* __restrict__ gaunt,
              int n, double* __restrict__ C, double* __restrict__ m_out, double* __restrict__ cond_out) {
  __shared__ double M[kMaxN * kLd];
  __shared__ double U[kMaxN * kLd];
  __shared__ double f[kMaxN];
  __shared__ double rhs[kMaxN];
  __shared__ double x[kMaxN];
  const int sys = blockIdx.x, lane = threadIdx.x;
  const double b0 = B[(long long)sys * n];
  if (lane < n) {
    f[lane] = B[(long long)sys * n + lane] / b0;
    rhs[lane] = A[(long long)sys * n + lane];
  }
  __syncwarp();
  if (lane < n) {  // lane = column l
    const int l = lane;
    for (int k = 0; k < n; ++k) {
      double v = 0.0;
      if (k == 0) {
        if (l >= 1) v = f[l] / (2.0 * l + 1.0);
      } else {
        for (int lp = 1; lp < n; ++lp) v += gaunt[((long long)k * n + l) * n + lp] * f[lp];
      }
      if (k == l) v += 1.0;
      v *= b0;
      M[k * kLd + l] = v;
      U[k * kLd + l] = v;
      if (m_out) m_out[((long long)sys * n + k) * n + l] = v;
    }
  }
  __syncwarp();

  // ---- cond_2 by one-sided Jacobi on the columns of U (lane = row) --------
  for (int sweep = 0; sweep < kJacobiSweeps; ++sweep) {
    int rotated = 0;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double up = lane < n ? U[lane * kLd + p] : 0.0;
        const double uq = lane < n ? U[lane * kLd + q] : 0.0;
        const double alpha = warp_sum(up * up), beta = warp_sum(uq * uq), gamma = warp_sum(up * uq);
        if (gamma != 0.0 && fabs(gamma) > 1e-15 * sqrt(alpha * beta)) {
          rotated = 1;
          const double zeta = (beta - alpha) / (2.0 * gamma);
          const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
          const double c = 1.0 / sqrt(1.0 + t * t), s = c * t;
          if (lane < n) {
            U[lane * kLd + p] = c * up - s * uq;
            U[lane * kLd + q] = s * up + c * uq;
          }
        }
        __syncwarp();
      }
    if (!rotated) break;
  }
  double smax = 0.0, smin = 0.0;
  for (int j = 0; j < n; ++j) {
    const double u = lane < n ? U[lane * kLd + j] : 0.0;
    const double sj = sqrt(warp_sum(u * u));
    if (j == 0 || sj > smax) smax = sj;
    if (j == 0 || sj < smin) smin = sj;
  }

  // ---- LU with partial pivoting (lane = row), then back substitution ------
  for (int k = 0; k < n; ++k) {
    double best = (lane >= k && lane < n) ? fabs(M[lane * kLd + k]) : -1.0;
    int bi = lane;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ob > best || (ob == best && oi < bi)) {
        best = ob;
        bi = oi;
      }
    }
    const int piv = bi;
    if (piv != k && lane < n) {  // lane = column for the row swap
      const double t = M[k * kLd + lane];
      M[k * kLd + lane] = M[piv * kLd + lane];
      M[piv * kLd + lane] = t;
    }
    if (piv != k && lane == 0) {
      const double t = rhs[k];
      rhs[k] = rhs[piv];
      rhs[piv] = t;
    }
    __syncwarp();
    const double pk = M[k * kLd + k];
    if (lane > k && lane < n) {
      const double fi = M[lane * kLd + k] / pk;
      for (int j = k + 1; j < n; ++j) M[lane * kLd + j] -= fi * M[k * kLd + j];
      rhs[lane] -= fi * rhs[k];
      M[lane * kLd + k] = 0.0;
    }
    __syncwarp();
  }
  if (lane == 0) {
    for (int i = n - 1; i >= 0; --i) {
      double s = rhs[i];
      for (int j = i + 1; j < n; ++j) s -= M[i * kLd + j] * x[j];
      x[i] = s / M[i * kLd + i];
    }
  }
  __syncwarp();
  if (lane < n) C[(long long)sys * n + lane] = x[lane];
  if (lane == 0 && cond_out) cond_out[sys] = smin > 0.0 ? smax / smin : INFINITY;
}

}  // namespace

extern "C" int hermes_mixing_solve(const double* A, const double* B, const double* gaunt, int n_sys, int n,
                                   double* zeta_out, double* m_out, double* cond_out, void* stream) {
  if (n_sys < 0) return fail(HERMES_ERR_INVALID, "mixing_solve: n_sys=%d", n_sys);
  if (n < 1 || n > kMaxN) return fail(HERMES_ERR_INVALID, "mixing_solve: n=%d outside [1,%d]", n, kMaxN);
  if (n_sys == 0) return HERMES_OK;
  if (!A || !B || !gaunt || !zeta_out) return fail(HERMES_ERR_INVALID, "mixing_solve: NULL argument");
  cudaStream_t s = hermes::as_stream(stream);
  mixing_kernel<<<n_sys, 32, 0, s>>>(A, B, gaunt, n, zeta_out, m_out, cond_out);
  HERMES_LAUNCH_CHECK("mixing_kernel");
  return HERMES_OK;
}
