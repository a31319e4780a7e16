// The scaling function's precomputes on the device: the Fourier power
// |phi_hat(k)|^2 every window and multipole kernel weights its images with
// (utils/wavelet_grid.py:94-118, fourier_power_spectrum) and the triple
// overlap matrix Gamma of the 3PCF contraction
// (utils/corr3pcf_multipoles.py:22-30, cal_gamma), float64, with the
// reference's expressions: arg = (-2 pi k) x, term = (phi dx) cos/sin(arg),
// Gamma[l1][l2] = sum_j phi[j] phi[j - l1 res] phi[j - l2 res] / res (cyclic).
#include "hermes_common.cuh"

namespace {

using hermes::fail;

constexpr int kPhiThreads = 256;

// (re, im) block sums in a fixed order (deterministic).
__device__ __forceinline__ double2 block_sum2(double re, double im) {
  __shared__ double sr[kPhiThreads / 32], si[kPhiThreads / 32];
  for (int o = 16; o > 0; o >>= 1) {
    re += __shfl_xor_sync(0xffffffffu, re, o);
    im += __shfl_xor_sync(0xffffffffu, im, o);
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) {
    sr[w] = re;
    si[w] = im;
  }
  __syncthreads();
  double2 out = make_double2(0.0, 0.0);
  if (threadIdx.x == 0)
    for (int i = 0; i < kPhiThreads / 32; ++i) {
      out.x += sr[i];
      out.y += si[i];
    }
  __syncthreads();
  return out;
}

__global__ void __launch_bounds__(kPhiThreads)
phi_power_kernel(const double* __restrict__ phi, int n, double dx, double dk, int kc, double* __restrict__ out) {
  const double two_pi = 6.283185307179586;
  for (int kn = blockIdx.x; kn <= kc; kn += gridDim.x) {
    const double mk = -two_pi * ((double)kn * dk);
    double re = 0.0, im = 0.0;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
      double s, c;
      sincos(mk * ((double)j * dx), &s, &c);
      const double a = phi[j] * dx;
      re = fma(a, c, re);
      im = fma(a, s, im);
    }
    const double2 t = block_sum2(re, im);
    if (threadIdx.x == 0) out[kn] = t.x * t.x + t.y * t.y;
  }
}

// one warp per (l1, l2)
__global__ void phi_gamma_kernel(const double* __restrict__ phi, int n, int support, int res,
                                 double* __restrict__ gamma) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (w >= support * support) return;
  const int l1 = w / support, l2 = w - l1 * support;
  double acc = 0.0;
  for (int j = lane; j < n; j += 32) {
    const int j1 = ((j - l1 * res) % n + n) % n, j2 = ((j - l2 * res) % n + n) % n;
    acc = fma(phi[j] * phi[j1], phi[j2], acc);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) gamma[w] = acc / (double)res;
}

}  // namespace

extern "C" int hermes_phi_prepare(const double* phi, int n_phi, int phi_res, int L, int bandwidth,
                                  double* power_out, double* gamma_out, void* stream) {
  if (!phi) return fail(HERMES_ERR_INVALID, "phi_prepare: phi is NULL");
  if (phi_res < 1 || n_phi < phi_res || n_phi % phi_res)
    return fail(HERMES_ERR_INVALID, "phi_prepare: n_phi=%d must be a positive multiple of phi_res=%d", n_phi, phi_res);
  const int support = n_phi / phi_res;
  if (gamma_out && support * support > 32)  // one warp per entry, one block
    return fail(HERMES_ERR_INVALID, "phi_prepare: support %d too large for gamma", support);
  cudaStream_t s = hermes::as_stream(stream);
  if (power_out) {
    if (L < 1 || bandwidth < 1 || (long long)L * bandwidth > (1 << 24))
      return fail(HERMES_ERR_INVALID, "phi_prepare: L=%d, bandwidth=%d", L, bandwidth);
    const int kc = L * bandwidth;
    const double dx = ((double)n_phi / (double)phi_res) / (double)n_phi;  // as the reference: (n/res)/n
    const double dk = (double)bandwidth / (double)kc;
    const int grid = kc + 1 < 4096 ? kc + 1 : 4096;
    phi_power_kernel<<<grid, kPhiThreads, 0, s>>>(phi, n_phi, dx, dk, kc, power_out);
    HERMES_LAUNCH_CHECK("phi_power_kernel");
  }
  if (gamma_out) {
    phi_gamma_kernel<<<1, 32 * support * support, 0, s>>>(phi, n_phi, support, phi_res, gamma_out);
    HERMES_LAUNCH_CHECK("phi_gamma_kernel");
  }
  return HERMES_OK;
}
