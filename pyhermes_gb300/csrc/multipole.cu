// Spherical-harmonic 3PCF multipoles on one GB300.
//
// Reference (pyhermes/utils/corr3pcf_multipoles.py:460-579, per (r12, r13)
// sample, per (l, m)): build two complex full-FFT windows
// K_lm(k) = sum_{8 images} |phi_hat|^2 j_l(2 pi |k| R) Y_lm(khat)
// (utils/radial_multipole_windows.py:128-183), two complex FFT convolutions,
// then the triple-product contraction
//   S_m = 4 pi / L^3 sum_x eps1(x) sum_{l1,l2} Gamma3(l1,l2) a2(x-l1) a3(x-l2).
//
// Here, per (l, m), for all radial bins at once:
//   mp_jl_table_kernel   j_l(2 pi sqrt(n2) R_b / L) tabulated over the integer
//                        |k|^2 grid (float32, double-float phase)
//   mp_prepass_*_kernel  eps_hat(k) K_lm^b(k) / L^3 for every bin b, Y_lm
//                        shared by the bins, written as a batch of spectra;
//                        one window evaluation serves k, its x- and
//                        y-reflections and their inversions
//   cuFFT (batched C2C)  -> a_lm^b(x) for every bin, one contiguous field per
//                        bin (cuFFT is far slower on strided batches)
//   mp_interleave_kernel bin-major -> bin-interleaved [cell][16], so one
//                        cell's bins are one 128-byte row for the contraction
//   mp_contract_kernel   S[b2,b3] = sum_y a2^{b2}(y) G^{b3}(y) with
//                        G(y) = sum_{l1,l2} Gamma3 eps1(y+l1) a3(y+l1-l2), an
//                        x-marching separable pair stencil (see the kernel)
//   mp_reduce_kernel     float64 cross-block reduction
// The identity S = sum_y a2(y) G3(y) is the reference sum with y = x - l1.
// mp_plain_kernel is the reference-form contraction of one (a2, a3) pair
// (the per-sample path the batched engine is measured against).
#include <cufft.h>

#include <algorithm>
#include <atomic>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include <cudaTypedefs.h>

#include "hermes_common.cuh"
#include "tc_common.cuh"
#include "window_eval.cuh"

namespace hermes {
int get_plan_c2c_batch(int J, int batch, cufftHandle* out);
int get_plan_c2c_lines(int J, int fields, cufftHandle* out);
int fft512_strided_inverse(float2* data, int nf, int axis, cudaStream_t s);
int prepare_window(const hermes_window_t& in, int L, WinDev* out);
}

namespace {

using hermes::df_frac;
using hermes::df_mul;
using hermes::df_sqrt_int;
using hermes::fail;

constexpr int kMaxBins = 16;
constexpr int kBinStride = 16;  // interleaved field layout [cell][kBinStride]
constexpr float kFourPiInvSqrt = 0.28209479177387814f;  // 1/sqrt(4 pi)

// ---- spherical Bessel j_l in float32 --------------------------------------
// Follows pyhermes/utils/special_functions.py:49-128 (series for small x,
// Miller downward recurrence for x < l+1, upward recurrence otherwise); x is
// given as a double-float multiple of 2 pi so sin/cos are exact-phase.
__device__ float sph_jl_f32(int l, float xh, float xl) {
  const float x = hermes::kTwoPi * (xh + xl);
  if (x == 0.f) return l == 0 ? 1.f : 0.f;
  const float ax = fabsf(x);
  const float x2 = x * x;
  if (ax <= 5.0e-2f || (l == 1 && ax < 1.f)) {
    if (l == 0) return 1.f - x2 / 6.f + x2 * x2 / 120.f;
    if (l == 1 && ax > 5.0e-2f)
      return x * (1.f / 3.f - x2 * (1.f / 30.f - x2 * (1.f / 840.f - x2 * (1.f / 45360.f - x2 / 3991680.f))));
    float denom = 1.f, xp = 1.f;
    for (int n = 1; n <= l; ++n) {
      denom *= 2.f * n + 1.f;
      xp *= x;
    }
    return (xp / denom) * (1.f - x2 / (2.f * (2.f * l + 3.f)) + x2 * x2 / (8.f * (2.f * l + 3.f) * (2.f * l + 5.f)));
  }
  float s, c;
  sincospif(2.f * df_frac(xh, xl), &s, &c);
  const float j0 = s / x;
  if (l == 0) return j0;
  const float j1 = s / x2 - c / x;
  if (l == 1) return j1;
  if (ax < l + 1.f) {
    const int n_stop = l + 40;
    float jp1 = 0.f, jcur = 1.f, jt = 0.f, jd0 = 0.f, jd1 = 0.f;
    const float inv = 1.f / x;
    for (int n = n_stop; n > 0; --n) {
      const float jm1 = (2.f * n + 1.f) * inv * jcur - jp1;
      if (n - 1 == l) jt = jm1;
      if (n - 1 == 1) jd1 = jm1;
      if (n - 1 == 0) jd0 = jm1;
      jp1 = jcur;
      jcur = jm1;
      if (fabsf(jcur) > 1.0e30f) {
        jp1 *= 1.0e-30f; jcur *= 1.0e-30f; jt *= 1.0e-30f; jd0 *= 1.0e-30f; jd1 *= 1.0e-30f;
      }
    }
    if (fabsf(jd0) >= fabsf(jd1) || jd1 == 0.f) return jt * (j0 / jd0);
    return jt * (j1 / jd1);
  }
  float jm1 = j0, jc = j1;
  for (int e = 1; e < l; ++e) {
    const float jn = (2.f * e + 1.f) / x * jc - jm1;
    jm1 = jc;
    jc = jn;
  }
  return jc;
}

// T[n2 * kBinStride + b] = j_l(2 pi sqrt(n2) R_b / L), n2 = 0 .. n2max (rows
// padded to 16 floats so one image's bins are four float4 loads).
struct RhoArgs {
  float v[2 * kMaxBins];  // R_b / L as double-float (hi, lo) pairs
};

// Radii travel as a kernel argument (no host-to-device copy), so the fields
// call can be captured into a CUDA graph.
__global__ void mp_jl_table_kernel(float* __restrict__ T, int n2max, RhoArgs rho,
                                   int nb, int l) {
  const long long total = (long long)(n2max + 1) * kBinStride;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int n2 = (int)(i / kBinStride), b = (int)(i % kBinStride);
    if (b >= nb) {
      T[i] = 0.f;
      continue;
    }
    float nh, nl, xh, xl;
    df_sqrt_int(n2, nh, nl);
    df_mul(nh, nl, rho.v[2 * b], rho.v[2 * b + 1], xh, xl);
    T[i] = sph_jl_f32(l, xh, xl);
  }
}

// T[n2 * 16 + b] = U_b(|k|) for isotropic window transfers (sphere, gaussian,
// shell, thick_shell, gaussian_shell; the analytic monopole profiles of
// radial_multipole_windows.py:60-128), k = sqrt(n2) / L.  The window
// descriptors are staged in shared memory.
struct IsoWins {
  hermes::WinDev w[kMaxBins];
};
__global__ void mp_iso_table_kernel(float* __restrict__ T, int n2max, IsoWins wins, int nb) {
  __shared__ hermes::WinDev sw[kMaxBins];
  if (threadIdx.x < kMaxBins) sw[threadIdx.x] = wins.w[threadIdx.x];
  __syncthreads();
  const long long total = (long long)(n2max + 1) * kBinStride;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int n2 = (int)(i / kBinStride), b = (int)(i % kBinStride);
    float v = 0.f;
    if (b < nb) {
      bool ok;
      v = hermes::window_iso_n2(sw[b], n2, &ok).x * sw[b].scale;
      if (!ok) v = __int_as_float(0x7fc00000);
    }
    T[i] = v;
  }
}

// T[n2 * 16 + b] = U_b(k) from uniform tables over k in [0, kmax_b] (n_b
// points; physical k = sqrt(n2) * k_scale), with the local cubic of
// radial_multipole_windows.py:186-210 (linear in the first and last
// interval, clamped outside), float64.
struct TabArgs {
  long long off[kMaxBins];
  int n[kMaxBins];
  double kmax[kMaxBins];
  double k_scale;  // grid_to_physical / L
};
__global__ void mp_tab_table_kernel(float* __restrict__ T, int n2max, const double* __restrict__ tables, TabArgs ta,
                                    int nb) {
  __shared__ long long soff[kMaxBins];
  __shared__ int sn[kMaxBins];
  __shared__ double skm[kMaxBins];
  if (threadIdx.x < kMaxBins) {
    soff[threadIdx.x] = ta.off[threadIdx.x];
    sn[threadIdx.x] = ta.n[threadIdx.x];
    skm[threadIdx.x] = ta.kmax[threadIdx.x];
  }
  __syncthreads();
  const long long total = (long long)(n2max + 1) * kBinStride;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int n2 = (int)(i / kBinStride), b = (int)(i % kBinStride);
    double v = 0.0;
    if (b < nb) {
      const double* t = tables + soff[b];
      const int n = sn[b];
      const double km = skm[b];
      const double k = sqrt((double)n2) * ta.k_scale;
      if (k <= 0.0) {
        v = t[0];
      } else if (k >= km) {
        v = t[n - 1];
      } else {
        const double idx = k * (double)(n - 1) / km;
        const int lo = (int)idx;
        const double f = idx - (double)lo;
        if (lo == 0 || lo >= n - 2) {
          v = t[lo] * (1.0 - f) + t[lo + 1] * f;
        } else {
          const double p0 = t[lo - 1], p1 = t[lo], p2 = t[lo + 1], p3 = t[lo + 2];
          const double f2 = f * f, f3 = f2 * f;
          v = 0.5 * (2.0 * p1 + (-p0 + p2) * f + (2.0 * p0 - 5.0 * p1 + 4.0 * p2 - p3) * f2 +
                     (-p0 + 3.0 * p1 - 3.0 * p2 + p3) * f3);
        }
      }
    }
    T[i] = (float)v;
  }
}

constexpr int kMaxEll = 40;
struct YlmConst {
  int l, m;          // m >= 0 here; negative m handled by the caller's flag
  float norm;        // sqrt((2l+1)/(4pi) (l-m)!/(l+m)!)
  float pmm;         // (-1)^m (2m-1)!!
  int neg_m;         // requested m < 0
  float neg_sign;    // (-1)^|m|
  float norm_lo;     // pairs (m = 0, degrees l - 1 and l): norm of degree l - 1
  // upward recurrence P_e = ca[e] ct P_{e-1} - cb[e] P_{e-2}, e = m+2 .. l:
  // ca = (2e-1)/(e-m), cb = (e+m-1)/(e-m) (float64 on the host, then float)
  float ca[kMaxEll + 1], cb[kMaxEll + 1];
};

// Y_lm(k) for integer frequency indices (a, b, c) != 0: with
// w = (a + i b)/|k| = sin(theta) e^{i phi} and c' = c/|k| = cos(theta),
// Y = norm * Q_l^m(c') * w^m where Q = P_l^m / sin^m (same recurrence as
// special_functions.py:273-304 with the sin^m factor moved into w^m).
__device__ __forceinline__ float2 ylm_at(const YlmConst& Y, int a, int b, int c, int n2) {
  if (n2 == 0) return make_float2((Y.l == 0 && Y.m == 0) ? kFourPiInvSqrt : 0.f, 0.f);
  const float rk = rsqrtf((float)n2);
  const float ct = (float)c * rk;
  const float wr = (float)a * rk, wi = (float)b * rk;
  float pr = 1.f, pi = 0.f;
  for (int i = 0; i < Y.m; ++i) {
    const float t = pr * wr - pi * wi;
    pi = pr * wi + pi * wr;
    pr = t;
  }
  float q;
  const float pmm = Y.pmm;
  if (Y.l == Y.m) {
    q = pmm;
  } else {
    float pmmp1 = ct * (2.f * Y.m + 1.f) * pmm;
    if (Y.l == Y.m + 1) {
      q = pmmp1;
    } else {
      float p2 = pmm, p1 = pmmp1, pl = 0.f;
      for (int e = Y.m + 2; e <= Y.l; ++e) {
        pl = Y.ca[e] * ct * p1 - Y.cb[e] * p2;
        p2 = p1;
        p1 = pl;
      }
      q = pl;
    }
  }
  float yr = Y.norm * q * pr, yi = Y.norm * q * pi;
  if (Y.neg_m) {
    yr = Y.neg_sign * yr;
    yi = -Y.neg_sign * yi;
  }
  return make_float2(yr, yi);
}

// (Y_{l-1,0}(k), Y_{l,0}(k)) for Y made for (l, 0) with norm_lo set: one
// Legendre recurrence gives both degrees, each the same float value
// ylm_at gives for it alone.
__device__ __forceinline__ float2 ylm_pair_at(const YlmConst& Y, int c, int n2) {
  if (n2 == 0) return make_float2(Y.l == 1 ? kFourPiInvSqrt : 0.f, 0.f);
  const float ct = (float)c * rsqrtf((float)n2);
  float p2 = 1.f, p1 = ct;  // P_0, P_1
  for (int e = 2; e <= Y.l; ++e) {
    const float pl = Y.ca[e] * ct * p1 - Y.cb[e] * p2;
    p2 = p1;
    p1 = pl;
  }
  return make_float2(Y.norm_lo * p2, Y.norm * p1);
}

// acc[b] = K_lm^b(x, y, z) = sum over the 8 images (a, b', c) (each axis
// index i in {i - L, i}) of Pphi(|a|) Pphi(|b'|) Pphi(|c|) j_l(|k|) Y_lm(k).
// kPair: acc[b] = (K_{l-1,0}^b, K_{l,0}^b) from the tables T4 (degree
// l - 1) and T4b (degree l), Y made for (l, 0) with norm_lo.
template <int NB4, bool kPair = false>
__device__ __forceinline__ void mp_window_sum(int x, int y, int z, int L, const float* __restrict__ P,
                                              const float4* __restrict__ T4, const float4* __restrict__ T4b,
                                              const YlmConst& Y, float2 (&acc)[4 * NB4]) {
#pragma unroll
  for (int b = 0; b < 4 * NB4; ++b) acc[b] = make_float2(0.f, 0.f);
  const int ia[2] = {x - L, x}, ib[2] = {y - L, y}, ic[2] = {z - L, z};
  const float pa[2] = {P[L - x], P[x]}, pb[2] = {P[L - y], P[y]}, pc[2] = {P[L - z], P[z]};
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        const int n2 = ia[i] * ia[i] + ib[j] * ib[j] + ic[k] * ic[k];
        const float pw = pa[i] * pb[j] * pc[k];
        const float2 yv = kPair ? ylm_pair_at(Y, ic[k], n2) : ylm_at(Y, ia[i], ib[j], ic[k], n2);
        const float2 yw = make_float2(pw * yv.x, pw * yv.y);  // (Re, Im) of P Y, one paired FMA per bin
        const float4* tr = T4 + (long long)n2 * (kBinStride / 4);
        if (kPair) {
          const float4* trb = T4b + (long long)n2 * (kBinStride / 4);
#pragma unroll
          for (int q = 0; q < NB4; ++q) {
            const float4 ja = __ldg(tr + q), jb = __ldg(trb + q);
            acc[4 * q + 0] = __ffma2_rn(make_float2(ja.x, jb.x), yw, acc[4 * q + 0]);
            acc[4 * q + 1] = __ffma2_rn(make_float2(ja.y, jb.y), yw, acc[4 * q + 1]);
            acc[4 * q + 2] = __ffma2_rn(make_float2(ja.z, jb.z), yw, acc[4 * q + 2]);
            acc[4 * q + 3] = __ffma2_rn(make_float2(ja.w, jb.w), yw, acc[4 * q + 3]);
          }
        } else {
#pragma unroll
          for (int q = 0; q < NB4; ++q) {
            const float4 jl = __ldg(tr + q);
            acc[4 * q + 0] = __ffma2_rn(make_float2(jl.x, jl.x), yw, acc[4 * q + 0]);
            acc[4 * q + 1] = __ffma2_rn(make_float2(jl.y, jl.y), yw, acc[4 * q + 1]);
            acc[4 * q + 2] = __ffma2_rn(make_float2(jl.z, jl.z), yw, acc[4 * q + 2]);
            acc[4 * q + 3] = __ffma2_rn(make_float2(jl.w, jl.w), yw, acc[4 * q + 3]);
          }
        }
      }
}

// out[b * L^3 + k] = eps_hat(k) * K_lm^b(k) / L^3 on the full FFT grid, from
// the half spectrum of a real field, in two kernels that together write
// every mode once.  Symmetries used (the float32 recurrences are
// sign-symmetric, so each holds exactly in the computed values):
//   inversion   eps_hat(-k) = conj eps_hat(k); K(-k) = (-1)^l K(k) when the
//               image set of -k is the negated image set of k, i.e. off the
//               x = 0 and y = 0 lines and for z != 0 (z = 0 has images
//               {-L, 0} against {0, L});
//   x-reflection (x, y, z) -> (L - x, y, z): K -> (-1)^m conj K
//               (Y_lm(-a, b, c) = (-1)^m conj Y_lm(a, b, c));
//   y-reflection (x, y, z) -> (x, L - y, z): K -> conj K
// for x, y not in {0, L/2} (where a reflected line is itself or its image
// set is not reflected).

// Interior: one thread per (x, y, z), 1 <= x, y < L/2, z in [0, L/2]; one
// window evaluation serves the four reflected lines (x, y), (L-x, y),
// (x, L-y), (L-x, L-y) at z and, for z not 0 or L/2, their inversions at
// L - z (the inversion of line a is line 3 - a).
//
// kPair: the window is K_{l-1,0} + K_{l,0} for odd l (Y made for (l, 0)
// with norm_lo, tables T4 for l - 1 and T4b for l).  Both terms are real and
// reflection-symmetric; under inversion the even one keeps its sign and the
// odd one flips it, so -k gets K_{l-1,0} - K_{l,0}.  The inverse FFT then
// gives a_{l-1,0} + a_{l,0}: the real field a_{l-1,0} in the real part and
// a_{l,0}, which is imaginary, in the imaginary part.
template <int NB4, bool kPair = false>
__global__ void __launch_bounds__(256)
mp_prepass_quad_kernel(const float2* __restrict__ half, int J, const float* __restrict__ P,
                       const float4* __restrict__ T4, const float4* __restrict__ T4b, YlmConst Y, int nb,
                       float2* __restrict__ out, float inv_n) {
  constexpr int NB = 4 * NB4;
  const int L = 1 << J, H = L / 2 + 1, Q1 = L / 2 - 1;
  const long long N = 1LL << (3 * J);
  const long long W = (long long)Q1 * Q1 * H;
  const float lsign = (Y.l & 1) ? -1.f : 1.f, msign = (Y.m & 1) ? -1.f : 1.f;
  for (long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x; w < W;
       w += (long long)gridDim.x * blockDim.x) {
    const int z = (int)(w % H), li = (int)(w / H);
    const int x = 1 + li / Q1, y = 1 + li % Q1;
    float2 acc[NB];
    mp_window_sum<NB4, kPair>(x, y, z, L, P, T4, T4b, Y, acc);
    const bool mirror = z != 0 && z != L / 2;
    if (kPair) {
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        const int xa = (a & 1) ? L - x : x, ya = (a & 2) ? L - y : y;
        const float2 e = half[((long long)xa * L + ya) * H + z];
        const float er = e.x * inv_n, ei = e.y * inv_n;
        const long long idx = ((long long)xa * L + ya) * L + z;
#pragma unroll
        for (int b = 0; b < NB; ++b) {
          if (b < nb) {
            const float k = acc[b].x + acc[b].y;
            out[b * N + idx] = make_float2(er * k, ei * k);
          }
        }
        if (mirror) {
          const long long idm = ((long long)(L - xa) * L + (L - ya)) * L + (L - z);
#pragma unroll
          for (int b = 0; b < NB; ++b) {
            if (b < nb) {
              const float k = acc[b].x - acc[b].y;
              out[b * N + idm] = make_float2(er * k, -ei * k);  // conj(eps_hat(k)) K(-k) / L^3
            }
          }
        }
      }
      continue;
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const int xa = (a & 1) ? L - x : x, ya = (a & 2) ? L - y : y;
      const float cr = (a & 1) ? msign : 1.f;                           // K_a = cr Re K + i ci Im K
      const float ci = (a == 1) ? -msign : (a == 2 ? -1.f : ((a == 3) ? msign : 1.f));
      const float2 e = half[((long long)xa * L + ya) * H + z];
      const float er = e.x * inv_n, ei = e.y * inv_n;
      const long long idx = ((long long)xa * L + ya) * L + z;
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        if (b < nb) {
          const float kr = cr * acc[b].x, ki = ci * acc[b].y;
          out[b * N + idx] = make_float2(er * kr - ei * ki, er * ki + ei * kr);
        }
      }
      if (mirror) {
        const long long idm = ((long long)(L - xa) * L + (L - ya)) * L + (L - z);
        const float mr = er, mi = -ei;  // conj(eps_hat(k)) / L^3
#pragma unroll
        for (int b = 0; b < NB; ++b) {
          if (b < nb) {
            const float kr = lsign * cr * acc[b].x, ki = lsign * ci * acc[b].y;
            out[b * N + idm] = make_float2(mr * kr - mi * ki, mr * ki + mi * kr);
          }
        }
      }
    }
  }
}

// Edge lines, x in {0, L/2} or y in {0, L/2} (4L - 4 lines): one thread per
// half-spectrum mode, which also writes its inversion when z is not 0 or
// L/2, evaluating it on the x = 0 and y = 0 lines.
template <int NB4, bool kPair = false>
__global__ void __launch_bounds__(256)
mp_prepass_edge_kernel(const float2* __restrict__ half, int J, const float* __restrict__ P,
                       const float4* __restrict__ T4, const float4* __restrict__ T4b, YlmConst Y, int nb,
                       float2* __restrict__ out, float inv_n) {
  constexpr int NB = 4 * NB4;
  const int L = 1 << J, H = L / 2 + 1, Lm = L - 1;
  const long long N = 1LL << (3 * J);
  const long long W = (long long)(4 * L - 4) * H;
  const float lsign = (Y.l & 1) ? -1.f : 1.f;
  for (long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x; w < W;
       w += (long long)gridDim.x * blockDim.x) {
    const int z = (int)(w % H), bi = (int)(w / H);
    int x, y;
    if (bi < 2 * L) {  // x in {0, L/2}, any y
      x = bi < L ? 0 : L / 2;
      y = bi & Lm;
    } else {           // y in {0, L/2}, x not in {0, L/2}
      const int t = bi - 2 * L;
      y = t < L - 2 ? 0 : L / 2;
      x = (t < L - 2 ? t : t - (L - 2)) + 1;
      if (x >= L / 2) ++x;
    }
    const float2 e = half[((long long)x * L + y) * H + z];
    float2 acc[NB];
    mp_window_sum<NB4, kPair>(x, y, z, L, P, T4, T4b, Y, acc);
    const float er = e.x * inv_n, ei = e.y * inv_n;
    const long long idx = ((long long)x * L + y) * L + z;
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      if (b < nb) {
        if (kPair) {
          const float k = acc[b].x + acc[b].y;
          out[b * N + idx] = make_float2(er * k, ei * k);
        } else {
          out[b * N + idx] = make_float2(er * acc[b].x - ei * acc[b].y, er * acc[b].y + ei * acc[b].x);
        }
      }
    }
    if (z == 0 || z == L / 2) continue;
    const int xm = (L - x) & Lm, ym = (L - y) & Lm, zm = L - z;
    if (x == 0 || y == 0) {
      mp_window_sum<NB4, kPair>(xm, ym, zm, L, P, T4, T4b, Y, acc);
    } else if (kPair) {  // K_{l-1,0} keeps its sign under inversion, K_{l,0} flips it
#pragma unroll
      for (int b = 0; b < NB; ++b) acc[b].y = -acc[b].y;
    } else {
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        acc[b].x *= lsign;
        acc[b].y *= lsign;
      }
    }
    const float mr = e.x * inv_n, mi = -(e.y * inv_n);  // conj(eps_hat(k)) / L^3
    const long long idm = ((long long)xm * L + ym) * L + zm;
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      if (b < nb) {
        if (kPair) {
          const float k = acc[b].x + acc[b].y;
          out[b * N + idm] = make_float2(mr * k, mi * k);
        } else {
          out[b * N + idm] = make_float2(mr * acc[b].x - mi * acc[b].y, mr * acc[b].y + mi * acc[b].x);
        }
      }
    }
  }
}

// dst[c * 16 + b] = src[b * N + c] for b < nb, 0 for nb <= b < 16.  A block
// moves 128 cells: coalesced per-bin reads into a padded shared tile, then
// 16 KB of contiguous 16-byte writes.
constexpr int kIlCells = 128;
__global__ void __launch_bounds__(256)
mp_interleave_kernel(const float2* __restrict__ src, int nb, long long N, float2* __restrict__ dst) {
  __shared__ float2 tile[kIlCells][kBinStride + 1];
  const int tid = threadIdx.x;
  for (long long c0 = (long long)blockIdx.x * kIlCells; c0 < N; c0 += (long long)gridDim.x * kIlCells) {
    for (int i = tid; i < kIlCells * kBinStride; i += blockDim.x) {
      const int b = i / kIlCells, c = i % kIlCells;
      tile[c][b] = b < nb ? src[(long long)b * N + c0 + c] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    float4* d4 = reinterpret_cast<float4*>(dst + c0 * kBinStride);
    for (int i = tid; i < kIlCells * kBinStride / 2; i += blockDim.x) {
      const int c = i >> 3, q = i & 7;
      d4[i] = make_float4(tile[c][2 * q].x, tile[c][2 * q].y, tile[c][2 * q + 1].x, tile[c][2 * q + 1].y);
    }
    __syncthreads();
  }
}

// ---- contraction: ε-weighted pair stencil + bin x bin product ----------------
// With Gamma3 = Gx (x) Gy (x) Gz and x_e = y_x + l1x, delta = l2x:
//   G(y)  = sum_{l1x, delta} Gx[l1x][delta] T_delta(y_x + l1x; y_y, y_z)
//   T_d(x_e; c) = sum_{u in [-2,2]^2} V_u(x_e; c) a3(x_e - d, c + u)
//   V_u(x_e; c) = sum_{l1y, l1z} Gy[l1y][l1y-uy] Gz[l1z][l1z-uz] eps1(x_e, c + l1)
// (terms with l1 - u outside [0,2] vanish).  V is bin independent, so a CTA
// computes it once per x-plane for its 8x8 column tile and every bin lane
// reuses it.  The CTA marches along x over a chunk of CX planes: plane x_a of
// a3 (12x12 cells x 16 bins, 128-byte rows) is staged with cp.async, T_d for
// d = 0..2 comes from that one plane, and G(x_a - 2) is complete after the
// step and is multiplied into S[b2][b3] += a2^{b2} G^{b3}.
// Thread mapping: lane & 15 = bin b3, each half-warp owns 2x2 columns.
// Per cell and bin: 75 + 9 complex*real FMAs for G, 16 complex FMAs for S.
namespace ct {
constexpr int TY = 8, TZ = 8;              // column tile (y, z)
constexpr int HY = TY + 4, HZ = TZ + 4;    // a3 plane region (halo 2)
constexpr int EY = TY + 2, EZ = TZ + 2;    // eps plane region (halo +2)
constexpr int kCols = TY * TZ;
constexpr int kGroups = kCols / 4;         // 2x2 column groups
constexpr int kThreads = kGroups * 16;     // 256
constexpr int kVRow = 8;                   // floats per (column, uy) row of V; 5 used
constexpr int kVCol = 5 * kVRow + 4;       // floats per column (pad: conflict-free V stores)
constexpr int kVPlane = kCols * kVCol;
constexpr int kA3Plane = HY * HZ * kBinStride;  // float2
constexpr int kA2Stride = kBinStride + 2;       // float2 per cell (pad: no bank conflicts)
constexpr int kA2Plane = kCols * kA2Stride;
constexpr int kEpsPlane = EY * EZ;
constexpr int kMaxCX = 64;  // default x-chunk below L = 256
// a3 planes x2, a2 planes x3, V ring x3, eps planes x2, one G plane, float64 S
constexpr size_t kSmem = sizeof(float2) * (2 * kA3Plane + 3 * kA2Plane + kA2Plane) +
                         sizeof(float) * (3 * kVPlane + 2 * kEpsPlane) + sizeof(double) * 2 * kMaxBins * kMaxBins;
}  // namespace ct

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

struct GammaC {
  float g[9];  // Gamma[l1][l2], row-major
};

struct ContractArgs {
  const float* eps1;
  const float2* f2;
  const float2* src3;
  int s2, s3;        // field strides (kBinStride, or 1 for a single bin)
  long long bstride; // bin-major fields (tensor-core kernel): float2 stride between bins
  int nb3s;          // bin-major fields: bins of the a3 source to stage
  int conj_src;      // a3 = sign * conj(src3)
  float sign;
  int packed;        // tensor-core kernel: S = (sum Re a2 Re G, sum Im a2 Im G), not a2 G
  int J, CX;
  GammaC gm;
  double* partial;   // [gridDim.x][16][16][2]
  int* status;       // first bounded wait that gave up (tensor-core kernel), else 0
};

// a3 plane x_a (region rows y0-2.., cols z0-2..) -> buf [cell][16] float2.
__device__ __forceinline__ void ct_stage_a3(const float2* __restrict__ src3, int s3, float2* buf, int xa, int y0, int z0, int L, int Lm) {
  const long long xb = (long long)(xa & Lm) * L;
  if (s3 == kBinStride) {
    for (int c = threadIdx.x; c < ct::HY * ct::HZ * 8; c += ct::kThreads) {
      const int cell = c >> 3, ch = c & 7;
      const int hy = cell / ct::HZ, hz = cell - hy * ct::HZ;
      const long long g = ((xb + ((y0 - 2 + hy) & Lm)) * L + ((z0 - 2 + hz) & Lm)) * kBinStride + 2 * ch;
      cp_async16(buf + cell * kBinStride + 2 * ch, src3 + g);
    }
  } else {  // single bin: slot 0 holds the value, other slots zero
    for (int c = threadIdx.x; c < ct::HY * ct::HZ * kBinStride; c += ct::kThreads) {
      const int cell = c >> 4, bb = c & 15;
      const int hy = cell / ct::HZ, hz = cell - hy * ct::HZ;
      float2 v = make_float2(0.f, 0.f);
      if (bb == 0) v = src3[(xb + ((y0 - 2 + hy) & Lm)) * L + ((z0 - 2 + hz) & Lm)];
      buf[c] = v;
    }
  }
}

// a2 plane x (the tile's 8x8 columns) -> buf [col][kA2Stride] float2.
__device__ __forceinline__ void ct_stage_a2(const float2* __restrict__ f2, int s2, float2* buf, int x, int y0, int z0, int L, int Lm) {
  const long long xb = (long long)(x & Lm) * L;
  if (s2 == kBinStride) {
    for (int c = threadIdx.x; c < ct::kCols * 8; c += ct::kThreads) {
      const int col = c >> 3, ch = c & 7;
      const int cy = col / ct::TZ, cz = col - cy * ct::TZ;
      const long long g = ((xb + y0 + cy) * L + z0 + cz) * kBinStride + 2 * ch;
      cp_async16(buf + col * ct::kA2Stride + 2 * ch, f2 + g);
    }
  } else {
    for (int c = threadIdx.x; c < ct::kCols * kBinStride; c += ct::kThreads) {
      const int col = c >> 4, bb = c & 15;
      const int cy = col / ct::TZ, cz = col - cy * ct::TZ;
      float2 v = make_float2(0.f, 0.f);
      if (bb == 0) v = f2[(xb + y0 + cy) * L + z0 + cz];
      buf[col * ct::kA2Stride + bb] = v;
    }
  }
}

__device__ __forceinline__ void ct_stage_eps(const float* __restrict__ eps1, float* buf, int xe, int y0, int z0, int L, int Lm) {
  const long long xb = (long long)(xe & Lm) * L;
  for (int c = threadIdx.x; c < ct::kEpsPlane; c += ct::kThreads) {
    const int ey = c / ct::EZ, ez = c - ey * ct::EZ;
    cp_async4(buf + c, eps1 + (xb + ((y0 + ey) & Lm)) * L + ((z0 + ez) & Lm));
  }
}

// V plane from a staged eps plane: V[col][uy+2][uz+2].  Four threads per
// column; w[a][l1] = Gamma[l1][l1 - a + 2] (0 outside [0,2]) in shared memory.
// Each thread filters the column's 3x3 eps neighbourhood along z for the five
// uz, then along y for its uy rows (uy+2 = part, and 4 for part 0).
__device__ __forceinline__ void ct_compute_v(const float* __restrict__ w, const float* __restrict__ e,
                                             float* __restrict__ v) {
  const int col = threadIdx.x >> 2, part = threadIdx.x & 3;
  const int cy = col / ct::TZ, cz = col - cy * ct::TZ;
  float ev[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) ev[i][j] = e[(cy + i) * ct::EZ + cz + j];
  float ez[3][5];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int a = 0; a < 5; ++a) ez[i][a] = fmaf(w[a * 3 + 2], ev[i][2], fmaf(w[a * 3 + 1], ev[i][1], w[a * 3] * ev[i][0]));
#pragma unroll
  for (int rep = 0; rep < 2; ++rep) {
    const int ay = rep == 0 ? part : 4;
    if (rep == 1 && part != 0) break;
    const float w0 = w[ay * 3], w1 = w[ay * 3 + 1], w2 = w[ay * 3 + 2];
    float o[5];
#pragma unroll
    for (int a = 0; a < 5; ++a) o[a] = fmaf(w2, ez[2][a], fmaf(w1, ez[1][a], w0 * ez[0][a]));
    float* dst = v + col * ct::kVCol + ay * ct::kVRow;
    *reinterpret_cast<float4*>(dst) = make_float4(o[0], o[1], o[2], o[3]);
    dst[4] = o[4];
  }
}

__global__ void __launch_bounds__(ct::kThreads, 2) mp_contract_kernel(ContractArgs A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* abuf = reinterpret_cast<float2*>(smem_raw);     // [2][kA3Plane]
  float2* a2buf = abuf + 2 * ct::kA3Plane;                // [3][kA2Plane]
  float2* gpl = a2buf + 3 * ct::kA2Plane;                 // [kCols][kA2Stride] completed G plane
  double* dacc = reinterpret_cast<double*>(gpl + ct::kA2Plane);  // [16][16][2]
  float* vring = reinterpret_cast<float*>(dacc + 2 * kMaxBins * kMaxBins);  // [3][kVPlane]
  float* epsb = vring + 3 * ct::kVPlane;                  // [2][kEpsPlane]
  const int J = A.J, L = 1 << J, Lm = L - 1, CX = A.CX;
  const int tid = threadIdx.x;
  // stencil mapping: lane & 15 = bin, half-warp = 2x2 column group
  const int b = tid & 15;
  const int grp = tid >> 4;
  const int cy = 2 * (grp / (ct::TZ / 2)), cz = 2 * (grp % (ct::TZ / 2));
  // product mapping: warp -> b2 quad (w >> 1), lane >> 2 -> b3 pair, cells 8k + slice
  const int bq = tid >> 6, b3p = (tid >> 2) & 7;
  const int slice = ((tid >> 5) & 1) * 4 + (tid & 3);
  const int nty = L / ct::TY, ntz = L / ct::TZ;
  const int n_items = (L / CX) * nty * ntz;
  const int nsteps = CX + 4;
  __shared__ float gsm[15];    // V-pass weights w[a][l1] = Gamma[l1][l1 - a + 2]
  if (tid == 0) {
#pragma unroll
    for (int a = 0; a < 5; ++a)
#pragma unroll
      for (int l1 = 0; l1 < 3; ++l1) {
        const int l2 = l1 - a + 2;  // static indices keep A in parameter space
        gsm[a * 3 + l1] = (l2 >= 0 && l2 <= 2) ? A.gm.g[l1 * 3 + (l2 < 0 ? 0 : (l2 > 2 ? 2 : l2))] : 0.f;
      }
  }
  for (int i = tid; i < 2 * kMaxBins * kMaxBins; i += ct::kThreads) dacc[i] = 0.0;
  __syncthreads();

  for (int item = blockIdx.x; item < n_items; item += gridDim.x) {
    const int tz = item % ntz, ty = (item / ntz) % nty, xc = item / (ntz * nty);
    const int x0 = xc * CX, y0 = ty * ct::TY, z0 = tz * ct::TZ;
    // prologue: V(x0-2), V(x0-1) into ring slots 0, 1; first a3 plane; eps plane x0
    ct_stage_eps(A.eps1, epsb, x0 - 2, y0, z0, L, Lm);
    ct_stage_eps(A.eps1, epsb + ct::kEpsPlane, x0 - 1, y0, z0, L, Lm);
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
    ct_compute_v(gsm, epsb, vring);
    ct_compute_v(gsm, epsb + ct::kEpsPlane, vring + ct::kVPlane);
    __syncthreads();
    ct_stage_a3(A.src3, A.s3, abuf, x0 - 2, y0, z0, L, Lm);
    ct_stage_eps(A.eps1, epsb, x0, y0, z0, L, Lm);
    cp_async_commit();

    float2 G[5][4];
    float2 S[8];  // S[4 bq + i][2 b3p + j] at i * 2 + j
#pragma unroll
    for (int q = 0; q < 5; ++q)
#pragma unroll
      for (int c = 0; c < 4; ++c) G[q][c] = make_float2(0.f, 0.f);
#pragma unroll
    for (int q = 0; q < 8; ++q) S[q] = make_float2(0.f, 0.f);

    for (int st = 0; st < nsteps; ++st) {
      const int xa = x0 - 2 + st;
      // (1) prefetch: a3 plane xa+1, eps plane xa+3, a2 plane of the next step's product.
      // Readers of the overwritten buffers finished before the previous step's
      // third barrier (a3, eps) or before this step's first barrier of the step
      // before (a2, three buffers).
      if (st + 1 < nsteps) {
        ct_stage_a3(A.src3, A.s3, abuf + ((st + 1) & 1) * ct::kA3Plane, xa + 1, y0, z0, L, Lm);
        ct_stage_eps(A.eps1, epsb + ((st + 1) & 1) * ct::kEpsPlane, xa + 3, y0, z0, L, Lm);
        if (st + 1 >= 4) ct_stage_a2(A.f2, A.s2, a2buf + ((st + 1) % 3) * ct::kA2Plane, xa - 1, y0, z0, L, Lm);
      }
      cp_async_commit();
      cp_async_wait<1>();
      __syncthreads();
      // (2) V(xa + 2) from eps plane xa + 2
      ct_compute_v(gsm, epsb + (st & 1) * ct::kEpsPlane, vring + ((st + 2) % 3) * ct::kVPlane);
      __syncthreads();
      // (3) T_d(xa + d) for this group's 2x2 columns, bin b
      {
        const float2* ap = abuf + (st & 1) * ct::kA3Plane;
        const float* vp0 = vring + (st % 3) * ct::kVPlane;
        const float* vp1 = vring + ((st + 1) % 3) * ct::kVPlane;
        const float* vp2 = vring + ((st + 2) % 3) * ct::kVPlane;
        float2 T[3][4];
#pragma unroll
        for (int d = 0; d < 3; ++d)
#pragma unroll
          for (int c = 0; c < 4; ++c) T[d][c] = make_float2(0.f, 0.f);
#pragma unroll
        for (int r = 0; r < 6; ++r) {
          float2 av[6];
#pragma unroll
          for (int k = 0; k < 6; ++k) av[k] = ap[((cy + r) * ct::HZ + cz + k) * kBinStride + b];
#pragma unroll
          for (int dy = 0; dy < 2; ++dy) {
            const int uy = r - 2 - dy;
            if (uy < -2 || uy > 2) continue;
#pragma unroll
            for (int dz = 0; dz < 2; ++dz) {
              const int voff = ((cy + dy) * ct::TZ + cz + dz) * ct::kVCol + (uy + 2) * ct::kVRow;
#pragma unroll
              for (int d = 0; d < 3; ++d) {
                const float* vp = (d == 0 ? vp0 : (d == 1 ? vp1 : vp2)) + voff;
                const float4 v4 = *reinterpret_cast<const float4*>(vp);
                const float v5 = vp[4];
                float2 t = T[d][dy * 2 + dz];
                t = __ffma2_rn(make_float2(v4.x, v4.x), av[dz], t);
                t = __ffma2_rn(make_float2(v4.y, v4.y), av[dz + 1], t);
                t = __ffma2_rn(make_float2(v4.z, v4.z), av[dz + 2], t);
                t = __ffma2_rn(make_float2(v4.w, v4.w), av[dz + 3], t);
                t = __ffma2_rn(make_float2(v5, v5), av[dz + 4], t);
                T[d][dy * 2 + dz] = t;
              }
            }
          }
        }
        // (4) G(xa + d - l1x) += Gx[l1x][d] T_d; ring slot q <-> x = xa - 2 + q
#pragma unroll
        for (int d = 0; d < 3; ++d)
#pragma unroll
          for (int l1x = 0; l1x < 3; ++l1x) {
            const float gx = A.gm.g[l1x * 3 + d];
#pragma unroll
            for (int c = 0; c < 4; ++c) G[d - l1x + 2][c] = __ffma2_rn(make_float2(gx, gx), T[d][c], G[d - l1x + 2][c]);
          }
      }
      // (5) G(xa - 2) is complete: publish it, then S[b2][b3] += a2^{b2} G^{b3}
      const bool full = st >= 4;
      if (full) {
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          float2 g = G[0][c];
          if (A.conj_src) g = make_float2(A.sign * g.x, -A.sign * g.y);
          gpl[((cy + (c >> 1)) * ct::TZ + cz + (c & 1)) * ct::kA2Stride + b] = g;
        }
      }
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int c = 0; c < 4; ++c) G[q][c] = G[q + 1][c];
#pragma unroll
      for (int c = 0; c < 4; ++c) G[4][c] = make_float2(0.f, 0.f);
      __syncthreads();
      if (full) {
        const float2* a2p = a2buf + (st % 3) * ct::kA2Plane;
#pragma unroll 2
        for (int k = 0; k < ct::kCols / 8; ++k) {
          const int cell = 8 * k + slice;
          const float4* ar = reinterpret_cast<const float4*>(a2p + cell * ct::kA2Stride + 4 * bq);
          const float4 a01 = ar[0], a23 = ar[1];
          const float4 gg = *reinterpret_cast<const float4*>(gpl + cell * ct::kA2Stride + 2 * b3p);
          const float2 g0 = make_float2(gg.x, gg.y), g1 = make_float2(gg.z, gg.w);
          const float2 h0 = make_float2(-gg.y, gg.x), h1 = make_float2(-gg.w, gg.z);  // i g
          const float ar_[4] = {a01.x, a01.z, a23.x, a23.z}, ai_[4] = {a01.y, a01.w, a23.y, a23.w};
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const float2 re = make_float2(ar_[i], ar_[i]), im = make_float2(ai_[i], ai_[i]);
            S[2 * i] = __ffma2_rn(im, h0, __ffma2_rn(re, g0, S[2 * i]));
            S[2 * i + 1] = __ffma2_rn(im, h1, __ffma2_rn(re, g1, S[2 * i + 1]));
          }
        }
      }
    }
    cp_async_wait<0>();
    // fixed-order reduction of the eight cell slices (lanes, then the warp
    // pair in two ordered passes), float64 per CTA
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      S[q].x += __shfl_xor_sync(0xffffffffu, S[q].x, 1);
      S[q].y += __shfl_xor_sync(0xffffffffu, S[q].y, 1);
      S[q].x += __shfl_xor_sync(0xffffffffu, S[q].x, 2);
      S[q].y += __shfl_xor_sync(0xffffffffu, S[q].y, 2);
    }
#pragma unroll
    for (int round = 0; round < 2; ++round) {
      if ((tid & 3) == 0 && ((tid >> 5) & 1) == round) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int o = ((4 * bq + (q >> 1)) * kMaxBins + 2 * b3p + (q & 1)) * 2;
          dacc[o] += (double)S[q].x;
          dacc[o + 1] += (double)S[q].y;
        }
      }
      __syncthreads();  // pass 1 after pass 0; all buffers idle before the next item
    }
  }
  for (int i = tid; i < 2 * kMaxBins * kMaxBins; i += ct::kThreads)
    A.partial[(long long)blockIdx.x * 2 * kMaxBins * kMaxBins + i] = dacc[i];
}

// ---- h form of the per-plane stencil ------------------------------------------
//   T_d(c) = sum_{uy in [-2,2]} sum_{l1z in [0,2]} h_{uy,l1z}(x_e; c) Rz_{l1z}(x_a; c_y + uy, c_z)
//   h_{uy,l1z}(c) = sum_{l1y} Gamma[l1y][l1y-uy] eps1(x_e, c_y + l1y, c_z + l1z)   (bin independent)
//   Rz_{l1z}(y, z) = sum_{l2z} Gamma[l1z][l2z] a3(x_a, y, z + l1z - l2z)           (fixed z filter)
// This is the V form above with its z sum split through the separable Gamma:
// 15 weights per column and plane instead of 25, and per (column, uy, plane)
// 3 FMAs instead of 5 (plus the 9-FMA z filter per row, shared by the planes).
namespace hf {
constexpr int kHCol = 20;                      // floats per column: [5 uy][4] (3 used)
constexpr int kHPlane = ct::kCols * kHCol;
}  // namespace hf

// h plane from a staged eps plane: H[col][uy+2][l1z].  Four threads per
// column; thread `part` writes uy + 2 = part (and 4 for part 0).
__device__ __forceinline__ void ct_compute_h(const float* __restrict__ w, const float* __restrict__ e,
                                             float* __restrict__ h) {
  const int col = threadIdx.x >> 2, part = threadIdx.x & 3;
  const int cy = col / ct::TZ, cz = col - cy * ct::TZ;
  float ev[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) ev[i][j] = e[(cy + i) * ct::EZ + cz + j];
#pragma unroll
  for (int rep = 0; rep < 2; ++rep) {
    const int ay = rep == 0 ? part : 4;
    if (rep == 1 && part != 0) break;
    const float w0 = w[ay * 3], w1 = w[ay * 3 + 1], w2 = w[ay * 3 + 2];
    float o[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) o[j] = fmaf(w2, ev[2][j], fmaf(w1, ev[1][j], w0 * ev[0][j]));
    *reinterpret_cast<float4*>(h + col * hf::kHCol + ay * 4) = make_float4(o[0], o[1], o[2], 0.f);
  }
}

// ---- contraction with the bin x bin product on the tensor cores -------------
// The stencil runs on the CUDA cores in FP32 (the h form); the product
// S[b2][b3] += sum_cells a2^{b2} G^{b3} of every completed plane runs as one
// tcgen05.mma GEMM (kind::f16, BF16 operands, FP32 accumulate) with the
// accumulator in tensor memory, in the BF16x3 split: every FP32 operand value
// v = hi + mid + lo with hi = bf16(v), mid = bf16(v - hi),
// lo = bf16(v - hi - mid) (~24 significant bits: the FP32 value to rounding).
//   A (M = 128 x K = 64 cells): rows m = s*32 + 2*b2 + part of a2, s = 0, 1,
//     2 for hi, mid, lo, part = re / im; rows 96..127 are padding (unused);
//   B (N = 96 x K = 64 cells): columns n = s*32 + 2*b3 + part of G;
//   D[m][n] = sum_cells A[m] B[n] (FP32 in TMEM, 128 lanes x 96 columns).
// Summed over (s, s'), D gives the four real products of a2 x G per bin pair
// from all nine partial products.  Both operands are MN-major in
// 128B-swizzled shared memory: per cell one 128-byte row holding (hi, mid)
// (64 BF16) in atom column 0 and one holding (lo, padding) in atom column 1
// (8 KB further), 8-row atoms of 1 KB, K advancing by whole atoms.  The a2
// plane arrives by TMA (4-D tensor map over the [x][y][z][16 bins] fields,
// box 32 floats x 8 z x 8 y x 1 x) one step ahead; threads split it.  A
// plane's MMAs (4 x K = 16) are issued by one thread after the block barrier
// that follows the operand writes and run while the CUDA cores compute the
// next plane's stencil; their tcgen05.commit arrives on an mbarrier that the
// next overwrite of the operand buffers waits on.  At the end of a work item
// the accumulator is read back (tcgen05.ld) and added in float64 in a fixed
// order per bin pair.
namespace tcc {
constexpr int kAtomCol = 64 * 128;                         // one atom column: 64 cells x 128 B
constexpr int kOpBytes = 2 * kAtomCol;                     // (hi, mid) + (lo, pad) atom columns
constexpr int kRawBytes = 64 * kBinStride * 8;             // TMA a2 plane: 64 cells x 16 complex
constexpr int kTmemCols = 128;                             // D: 96 columns used
constexpr int kN = 96;
// a3 plane buffer: [cell][16] (bin-interleaved fields) or [16][kA3P]
// (bin-major fields).  kA3P = 146: rows stay 16-byte aligned, so a plane is
// staged with 16-byte copies and a thread reads two cells of its bin with
// one 16-byte load; the 16 bins of one cell start 4 banks apart, so a
// quarter-warp's 16-byte loads cover all 32 banks once (no conflict).
constexpr int kA3P = ct::HY * ct::HZ + 2;
constexpr int kA3Buf = kBinStride * kA3P;
static_assert(kA3Buf >= ct::kA3Plane, "a3 buffer");
constexpr uint32_t kIdesc = hermes::tc::idesc_bf16_f32(128, kN, true, true);
// 1 KB slack for the runtime 1024-byte alignment of the swizzled operands
constexpr size_t kSmem = 1024 + 2 * kOpBytes + 2 * kRawBytes + sizeof(float2) * 2 * kA3Buf +
                         sizeof(float) * (3 * hf::kHPlane + 2 * ct::kEpsPlane) +
                         sizeof(double) * 2 * kMaxBins * kMaxBins + 128;
}  // namespace tcc

// (lower half, upper half) -> packed BF16x2, round to nearest even
__device__ __forceinline__ uint32_t pack_bf16x2(float lo_half, float hi_half) {
  uint32_t r;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;\n" : "=r"(r) : "f"(hi_half), "f"(lo_half));
  return r;
}
__device__ __forceinline__ float bf16_lo(uint32_t p) { return __uint_as_float(p << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t p) { return __uint_as_float(p & 0xFFFF0000u); }

// BF16x3 split of a pair (x, y): packed hi, mid and lo pairs.
__device__ __forceinline__ void split3(float x, float y, uint32_t& h, uint32_t& m, uint32_t& l) {
  h = pack_bf16x2(x, y);
  const float rx = x - bf16_lo(h), ry = y - bf16_hi(h);
  m = pack_bf16x2(rx, ry);
  l = pack_bf16x2(rx - bf16_lo(m), ry - bf16_hi(m));
}

// Writes (re, im) of one bin into a swizzled operand, row `cell`: hi at
// element 2b and mid at 32 + 2b of atom column 0, lo at 2b of atom column 1.
__device__ __forceinline__ void tc_put_pair(unsigned char* op, int cell, int b, float re, float im) {
  uint32_t h, m, l;
  split3(re, im, h, m, l);
  const uint32_t row = (cell >> 3) * 1024, r = cell & 7, byte = (b & 3) * 4;
  *reinterpret_cast<uint32_t*>(op + row + hermes::tc::sw128_offset(r, b >> 2) + byte) = h;
  *reinterpret_cast<uint32_t*>(op + row + hermes::tc::sw128_offset(r, 4 + (b >> 2)) + byte) = m;
  *reinterpret_cast<uint32_t*>(op + tcc::kAtomCol + row + hermes::tc::sw128_offset(r, b >> 2) + byte) = l;
}

// a3 plane x_a from bin-major fields (bin b at src3 + b * bstride) -> buf
// [16][kA3P] float2; bins nb3 .. 15 are written as zeros.  The copies are
// 16 bytes, two cells (2p, 2p + 1) of one row: with z0 a multiple of 8 the
// pair starts at an even z and never straddles the periodic wrap, so both
// ends are 16-byte aligned.  Thread t copies bin t >> 4, pairs
// p = (t & 15) + 16 i of the 72 in the 12 x 12 plane; the (row, pair
// column) of the next one is a fixed step (16 pairs = two rows of 6 and 4).
__device__ __forceinline__ void ct_stage_a3_bm(const float2* __restrict__ src3, long long bstride, int nb3,
                                               float2* buf, int xa, int y0, int z0, int L, int Lm) {
  static_assert(ct::kThreads == 16 * kBinStride && ct::HY * ct::HZ == 144 && ct::HZ == 12 && ct::TZ % 8 == 0,
                "a3 staging map");
  constexpr int kPairs = ct::HY * ct::HZ / 2;  // 72
  const int bb = threadIdx.x >> 4, j = threadIdx.x & 15;
  float2* dst = buf + bb * tcc::kA3P + 2 * j;
  const int n = j < kPairs - 64 ? 5 : 4;
  if (bb < nb3) {
    const float2* src = src3 + bb * bstride + (long long)(xa & Lm) * L * L;
    int hy = j / 6;
    int hz = 2 * (j - 6 * hy);
#pragma unroll 1
    for (int i = 0; i < n; ++i) {
      cp_async16(dst + 32 * i, src + ((y0 - 2 + hy) & Lm) * L + ((z0 - 2 + hz) & Lm));
      hz += 8;
      hy += 2;
      if (hz >= ct::HZ) {
        hz -= ct::HZ;
        hy += 1;
      }
    }
  } else {
#pragma unroll 1
    for (int i = 0; i < n; ++i) *reinterpret_cast<float4*>(dst + 32 * i) = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

// kBM: fields in the bin-major layout [bin][cell] that cuFFT writes (a2 by a
// 4-D TMA map over (z, y, x, bin), a3 staged per bin); otherwise the
// bin-interleaved [cell][16] layout or a single [cell] field.
template <bool kBM>
__global__ void __launch_bounds__(ct::kThreads, 2)
mp_contract_tc_kernel(ContractArgs A, const __grid_constant__ CUtensorMap a2map) {
  namespace tc = hermes::tc;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char* base = smem_raw + ((1024u - (tc::smem_u32(smem_raw) & 1023u)) & 1023u);
  unsigned char* abf = base;                                       // A operand (a2 split)
  unsigned char* gbf = abf + tcc::kOpBytes;                        // B operand (G split)
  float* araw = reinterpret_cast<float*>(gbf + tcc::kOpBytes);    // [2][64 cells][32] TMA a2 planes
  float2* abuf = reinterpret_cast<float2*>(reinterpret_cast<unsigned char*>(araw) + 2 * tcc::kRawBytes);
  double* dacc = reinterpret_cast<double*>(abuf + 2 * tcc::kA3Buf);  // [16][16][2]
  float* hring = reinterpret_cast<float*>(dacc + 2 * kMaxBins * kMaxBins);  // [3][kHPlane]
  float* epsb = hring + 3 * hf::kHPlane;
  uint64_t* bars = reinterpret_cast<uint64_t*>(epsb + 2 * ct::kEpsPlane);  // tma[2], mma
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 3);
  float* gsm = reinterpret_cast<float*>(tmem_slot + 1);                  // 15 h-pass weights
  int* s_abort = reinterpret_cast<int*>(gsm + 16);
  float* stage = reinterpret_cast<float*>(abuf);                          // [96][33] at item end

  const int J = A.J, L = 1 << J, Lm = L - 1, CX = A.CX;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int b = tid & 15;
  // 2x2 column block of this half-warp: the two half-warps of a warp take
  // blocks 4 cells apart in z, so their rows of the swizzled G operand fall
  // in complementary halves of the 128-byte rows (no bank conflict)
  const int hw = (tid >> 4) & 1, wq = tid >> 5;
  const int cy = 2 * (wq >> 1), cz = 4 * hw + 2 * (wq & 1);
  const int nty = L / ct::TY, ntz = L / ct::TZ;
  const int n_items = (L / CX) * nty * ntz;
  const int nsteps = CX + 4;
  const bool tma_a2 = kBM || A.s2 == kBinStride;

  if (tid == 0) {
#pragma unroll
    for (int a = 0; a < 5; ++a)
#pragma unroll
      for (int l1 = 0; l1 < 3; ++l1) {
        const int l2 = l1 - a + 2;
        gsm[a * 3 + l1] = (l2 >= 0 && l2 <= 2) ? A.gm.g[l1 * 3 + (l2 < 0 ? 0 : (l2 > 2 ? 2 : l2))] : 0.f;
      }
    tc::mbar_init(&bars[0], 1);
    tc::mbar_init(&bars[1], 1);
    tc::mbar_init(&bars[2], 1);
    tc::mbar_fence_init();
    *s_abort = 0;
    if (tma_a2) tc::tma_prefetch_desc(&a2map);
  }
  if (warp == 0) tc::tmem_alloc(tmem_slot, tcc::kTmemCols);
  for (int i = tid; i < 2 * kMaxBins * kMaxBins; i += ct::kThreads) dacc[i] = 0.0;
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem_d = *tmem_slot;
  const uint32_t sa = tc::smem_u32(abf), sg = tc::smem_u32(gbf);
  uint32_t tma_ph0 = 0, tma_ph1 = 0, mma_ph = 0;
  bool mma_pending = false;

  for (int item = blockIdx.x; item < n_items; item += gridDim.x) {
    const int tz = item % ntz, ty = (item / ntz) % nty, xc = item / (ntz * nty);
    const int x0 = xc * CX, y0 = ty * ct::TY, z0 = tz * ct::TZ;
    // prologue: h(x0-2), h(x0-1), h(x0) into ring slots 0, 1, 2; a3 plane x0-2
    ct_stage_eps(A.eps1, epsb, x0 - 2, y0, z0, L, Lm);
    ct_stage_eps(A.eps1, epsb + ct::kEpsPlane, x0 - 1, y0, z0, L, Lm);
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
    ct_compute_h(gsm, epsb, hring);
    ct_compute_h(gsm, epsb + ct::kEpsPlane, hring + hf::kHPlane);
    __syncthreads();
    if (kBM)
      ct_stage_a3_bm(A.src3, A.bstride, A.nb3s, abuf, x0 - 2, y0, z0, L, Lm);
    else
      ct_stage_a3(A.src3, A.s3, abuf, x0 - 2, y0, z0, L, Lm);
    ct_stage_eps(A.eps1, epsb, x0, y0, z0, L, Lm);
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
    ct_compute_h(gsm, epsb, hring + 2 * hf::kHPlane);

    float2 G[5][4];
#pragma unroll
    for (int q = 0; q < 5; ++q)
#pragma unroll
      for (int c = 0; c < 4; ++c) G[q][c] = make_float2(0.f, 0.f);
    bool first_mma = true;

    // Two block barriers per step: the first makes the h plane computed at
    // the end of the previous step visible; the second the staged a3 / eps
    // planes (each thread waited for its own copies) and the MMA operands.
    for (int st = 0; st < nsteps; ++st) {
      const int xa = x0 - 2 + st;
      if (st + 1 < nsteps) {
        // a3 plane xa+1 and eps plane xa+3: their buffers' last readers (the
        // stencil one step back, the h pass two steps back) are done
        if (kBM)
          ct_stage_a3_bm(A.src3, A.bstride, A.nb3s, abuf + ((st + 1) & 1) * tcc::kA3Buf, xa + 1, y0, z0, L, Lm);
        else
          ct_stage_a3(A.src3, A.s3, abuf + ((st + 1) & 1) * tcc::kA3Buf, xa + 1, y0, z0, L, Lm);
        ct_stage_eps(A.eps1, epsb + ((st + 1) & 1) * ct::kEpsPlane, xa + 3, y0, z0, L, Lm);
        // a2 plane of the next step's product (its buffer's last reader, the
        // split two steps back, finished before the last block barrier)
        if (tma_a2 && tid == 0 && st + 1 >= 4) {
          uint64_t* bar = &bars[(st + 1) & 1];
          tc::fence_proxy_async_smem();
          tc::mbar_arrive_expect_tx(bar, tcc::kRawBytes);
          if (kBM)
            tc::tma_load_4d(araw + ((st + 1) & 1) * (tcc::kRawBytes / 4), &a2map, bar, 2 * z0, y0, (xa - 1) & Lm, 0);
          else
            tc::tma_load_4d(araw + ((st + 1) & 1) * (tcc::kRawBytes / 4), &a2map, bar, 0, z0, y0, (xa - 1) & Lm);
        }
      }
      cp_async_commit();
      __syncthreads();
      {
        const float2* ap = abuf + (st & 1) * tcc::kA3Buf;
        const float* hp0 = hring + (st % 3) * hf::kHPlane;
        const float* hp1 = hring + ((st + 1) % 3) * hf::kHPlane;
        const float* hp2 = hring + ((st + 2) % 3) * hf::kHPlane;
        float2 T[3][4];
#pragma unroll
        for (int d = 0; d < 3; ++d)
#pragma unroll
          for (int c = 0; c < 4; ++c) T[d][c] = make_float2(0.f, 0.f);
#pragma unroll
        for (int r = 0; r < 6; ++r) {
          float2 av[6];
          if (kBM) {  // two cells per 16-byte load (cz even, kA3P even)
            const float4* row4 = reinterpret_cast<const float4*>(ap + b * tcc::kA3P + (cy + r) * ct::HZ + cz);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
              const float4 p = row4[k];
              av[2 * k] = make_float2(p.x, p.y);
              av[2 * k + 1] = make_float2(p.z, p.w);
            }
          } else {
#pragma unroll
            for (int k = 0; k < 6; ++k) av[k] = ap[((cy + r) * ct::HZ + cz + k) * kBinStride + b];
          }
          // Rz_{l1z}(row, cz + dz) = sum_{l2z} Gamma[l1z][l2z] a3(row, cz + dz + l1z - l2z)
          float2 rz[2][3];
#pragma unroll
          for (int dz = 0; dz < 2; ++dz)
#pragma unroll
            for (int l1z = 0; l1z < 3; ++l1z) {
              const float g0 = A.gm.g[l1z * 3], g1 = A.gm.g[l1z * 3 + 1], g2 = A.gm.g[l1z * 3 + 2];
              float2 t = __fmul2_rn(make_float2(g2, g2), av[dz + l1z]);
              t = __ffma2_rn(make_float2(g1, g1), av[dz + l1z + 1], t);
              rz[dz][l1z] = __ffma2_rn(make_float2(g0, g0), av[dz + l1z + 2], t);
            }
#pragma unroll
          for (int dy = 0; dy < 2; ++dy) {
            const int uy = r - 2 - dy;
            if (uy < -2 || uy > 2) continue;
#pragma unroll
            for (int dz = 0; dz < 2; ++dz) {
              const int hoff = ((cy + dy) * ct::TZ + cz + dz) * hf::kHCol + (uy + 2) * 4;
#pragma unroll
              for (int d = 0; d < 3; ++d) {
                const float4 h4 = *reinterpret_cast<const float4*>((d == 0 ? hp0 : (d == 1 ? hp1 : hp2)) + hoff);
                float2 t = T[d][dy * 2 + dz];
                t = __ffma2_rn(make_float2(h4.x, h4.x), rz[dz][0], t);
                t = __ffma2_rn(make_float2(h4.y, h4.y), rz[dz][1], t);
                t = __ffma2_rn(make_float2(h4.z, h4.z), rz[dz][2], t);
                T[d][dy * 2 + dz] = t;
              }
            }
          }
        }
#pragma unroll
        for (int d = 0; d < 3; ++d)
#pragma unroll
          for (int l1x = 0; l1x < 3; ++l1x) {
            const float gx = A.gm.g[l1x * 3 + d];
#pragma unroll
            for (int c = 0; c < 4; ++c) G[d - l1x + 2][c] = __ffma2_rn(make_float2(gx, gx), T[d][c], G[d - l1x + 2][c]);
          }
      }
      // G(xa - 2) and the a2 plane xa - 2 become the operands of this plane's MMA
      const bool full = st >= 4;
      if (full) {
        if (mma_pending) {
          if (!tc::mbar_wait(&bars[2], mma_ph)) *s_abort = 2;
          mma_ph ^= 1u;
          mma_pending = false;
        }
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          float2 g = G[0][c];
          if (A.conj_src) g = make_float2(A.sign * g.x, -A.sign * g.y);
          tc_put_pair(gbf, (cy + (c >> 1)) * ct::TZ + cz + (c & 1), b, g.x, g.y);
        }
        // this thread's operand row (cell) and bins 4q .. 4q+3; with bin-major
        // planes ([bin][cell] in shared memory) a warp takes 32 cells of one q
        const int cell = kBM ? (tid & 63) : (tid >> 2), q = kBM ? (tid >> 6) : (tid & 3);
        float v[8];
        if (kBM) {
          const uint32_t par = (st & 1) ? tma_ph1 : tma_ph0;
          if (!tc::mbar_wait(&bars[st & 1], par)) *s_abort = 1;  // a2 plane (TMA)
          const float* src = araw + (st & 1) * (tcc::kRawBytes / 4) + cell * 2;
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const float2 p = *reinterpret_cast<const float2*>(src + (4 * q + i) * 128);
            v[2 * i] = p.x;
            v[2 * i + 1] = p.y;
          }
        } else if (tma_a2) {
          const uint32_t par = (st & 1) ? tma_ph1 : tma_ph0;
          if (!tc::mbar_wait(&bars[st & 1], par)) *s_abort = 1;  // a2 plane (TMA)
          const float4* src = reinterpret_cast<const float4*>(araw + (st & 1) * (tcc::kRawBytes / 4) + cell * 32 + 8 * q);
          const float4 p0 = src[0], p1 = src[1];
          v[0] = p0.x; v[1] = p0.y; v[2] = p0.z; v[3] = p0.w;
          v[4] = p1.x; v[5] = p1.y; v[6] = p1.z; v[7] = p1.w;
        } else {  // single bin: slot 0 holds the value
#pragma unroll
          for (int i = 0; i < 8; ++i) v[i] = 0.f;
          if (q == 0) {
            const int ccy = cell / ct::TZ, ccz = cell - ccy * ct::TZ;
            const float2 s = A.f2[((long long)((xa - 2) & Lm) * L + y0 + ccy) * L + z0 + ccz];
            v[0] = s.x;
            v[1] = s.y;
          }
        }
        if (st & 1) tma_ph1 ^= (tma_a2 ? 1u : 0u); else tma_ph0 ^= (tma_a2 ? 1u : 0u);
        uint32_t hv[4], mv[4], lv[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) split3(v[2 * i], v[2 * i + 1], hv[i], mv[i], lv[i]);
        unsigned char* atom = abf + (cell >> 3) * 1024;
        // elements 8q .. 8q+7 of the row: chunk q (hi), 4 + q (mid), q of column 1 (lo)
        *reinterpret_cast<uint4*>(atom + tc::sw128_offset(cell & 7, q)) = make_uint4(hv[0], hv[1], hv[2], hv[3]);
        *reinterpret_cast<uint4*>(atom + tc::sw128_offset(cell & 7, 4 + q)) = make_uint4(mv[0], mv[1], mv[2], mv[3]);
        *reinterpret_cast<uint4*>(atom + tcc::kAtomCol + tc::sw128_offset(cell & 7, q)) =
            make_uint4(lv[0], lv[1], lv[2], lv[3]);
        tc::fence_proxy_async_smem();
      }
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int c = 0; c < 4; ++c) G[q][c] = G[q + 1][c];
#pragma unroll
      for (int c = 0; c < 4; ++c) G[4][c] = make_float2(0.f, 0.f);
      cp_async_wait<0>();
      __syncthreads();
      if (*s_abort) break;
      // h(xa + 3) for the next step, into the ring slot this step's T_0 used
      if (st + 1 < nsteps) ct_compute_h(gsm, epsb + ((st + 1) & 1) * ct::kEpsPlane, hring + (st % 3) * hf::kHPlane);
      if (full) {
        if (tid == 0) {
          tc::tc_fence_after();
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            // K = 16 cells = two 1 KB atoms; the two atom columns 8 KB apart
            const uint64_t ad = tc::smem_desc(sa + k * 2048, tcc::kAtomCol, 1024, tc::kLayoutSw128);
            const uint64_t bd = tc::smem_desc(sg + k * 2048, tcc::kAtomCol, 1024, tc::kLayoutSw128);
            tc::mma_bf16(tmem_d, ad, bd, tcc::kIdesc, !(first_mma && k == 0));
          }
          tc::mma_commit(&bars[2]);
        }
        first_mma = false;
        mma_pending = true;
      }
    }
    cp_async_wait<0>();
    if (mma_pending) {
      if (!tc::mbar_wait(&bars[2], mma_ph)) *s_abort = 3;
      mma_ph ^= 1u;
      mma_pending = false;
    }
    __syncthreads();
    if (*s_abort) break;
    // accumulator rows 0..95 (lanes of warps 0..2): the three G parts s' are
    // summed per row (FP32, hi first), then stage[row][j], j = 2*b3 + part
    tc::tc_fence_after();
    if (warp < 3) {
      const int row = warp * 32 + (tid & 31);
      float acc[32];
      tc::tmem_ld_32x32b_x32(tmem_d + ((uint32_t)(warp * 32) << 16), acc);
#pragma unroll
      for (int part = 1; part < 3; ++part) {
        float d[32];
        tc::tmem_ld_32x32b_x32(tmem_d + ((uint32_t)(warp * 32) << 16) + part * 32, d);
#pragma unroll
        for (int i = 0; i < 32; ++i) acc[i] += d[i];
      }
#pragma unroll
      for (int i = 0; i < 32; ++i) stage[row * 33 + i] = acc[i];
    }
    tc::tc_fence_before();
    __syncthreads();
    {
      const int b2 = tid >> 4, b3 = tid & 15;
      double sr = 0.0, si = 0.0;
#pragma unroll
      for (int sp = 0; sp < 3; ++sp) {
        const float* rr = stage + (sp * 32 + 2 * b2) * 33 + 2 * b3;
        const float* ri = rr + 33;  // row of the imaginary part of a2
        if (A.packed) {  // the two real products, each its own sum
          sr += (double)rr[0];
          si += (double)ri[1];
        } else {
          sr += (double)rr[0] - (double)ri[1];
          si += (double)rr[1] + (double)ri[0];
        }
      }
      dacc[(b2 * kMaxBins + b3) * 2] += sr;
      dacc[(b2 * kMaxBins + b3) * 2 + 1] += si;
    }
    __syncthreads();  // stage (a3 buffer) idle before the next item's prologue
  }
  const int why = *s_abort;
  for (int i = tid; i < 2 * kMaxBins * kMaxBins; i += ct::kThreads)
    A.partial[(long long)blockIdx.x * 2 * kMaxBins * kMaxBins + i] = why ? __longlong_as_double(0x7ff8000000000000LL) : dacc[i];
  if (why && tid == 0 && A.status) atomicCAS(A.status, 0, why);
  __syncthreads();
  if (warp == 0) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem_d, tcc::kTmemCols);
  }
}

// out[o] = sum over blocks of partial[blk * nout + o]
__global__ void mp_reduce_kernel(const double* __restrict__ partial, int nblocks, int nout, double* __restrict__ out,
                                 double scale = 1.0) {
  const int o = blockIdx.x;
  double s = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) s += partial[(long long)b * nout + o];
  __shared__ double sh[256];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[o] = sh[0] * scale;
}

// ---- plain reference-form contraction of one (a2, a3) pair -----------------
// Per cell: eps1(x) * sum_l1 a2(x - l1) sum_l2x G sum_l2y G sum_l2z G a3(x - l2),
// the loop order of corr3pcf_multipoles.py:33-58, float32 complex.
__global__ void __launch_bounds__(256)
mp_plain_kernel(const float* __restrict__ eps1, const float2* __restrict__ a2, const float2* __restrict__ a3,
                int J, GammaC gm, double* __restrict__ partial) {
  const int L = 1 << J, Lm = L - 1;
  const long long N = 1LL << (3 * J);
  double accr = 0.0, acci = 0.0;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < N;
       idx += (long long)gridDim.x * blockDim.x) {
    const int lz = (int)(idx & Lm), ly = (int)((idx >> J) & Lm), lx = (int)(idx >> (2 * J));
    float s1r = 0.f, s1i = 0.f;
    for (int l1x = 0; l1x < 3; ++l1x) {
      const int i1x = (lx - l1x) & Lm;
      for (int l1y = 0; l1y < 3; ++l1y) {
        const int i1y = (ly - l1y) & Lm;
        for (int l1z = 0; l1z < 3; ++l1z) {
          const int i1z = (lz - l1z) & Lm;
          float s2r = 0.f, s2i = 0.f;
          for (int l2x = 0; l2x < 3; ++l2x) {
            const int i2x = (lx - l2x) & Lm;
            float ryr = 0.f, ryi = 0.f;
            for (int l2y = 0; l2y < 3; ++l2y) {
              const int i2y = (ly - l2y) & Lm;
              float rzr = 0.f, rzi = 0.f;
#pragma unroll
              for (int l2z = 0; l2z < 3; ++l2z) {
                const int i2z = (lz - l2z) & Lm;
                const float2 v = __ldg(&a3[((long long)i2x * L + i2y) * L + i2z]);
                const float g = gm.g[l1z * 3 + l2z];
                rzr = fmaf(g, v.x, rzr);
                rzi = fmaf(g, v.y, rzi);
              }
              const float g = gm.g[l1y * 3 + l2y];
              ryr = fmaf(g, rzr, ryr);
              ryi = fmaf(g, rzi, ryi);
            }
            const float g = gm.g[l1x * 3 + l2x];
            s2r = fmaf(g, ryr, s2r);
            s2i = fmaf(g, ryi, s2i);
          }
          const float2 u = __ldg(&a2[((long long)i1x * L + i1y) * L + i1z]);
          s1r += u.x * s2r - u.y * s2i;
          s1i += u.x * s2i + u.y * s2r;
        }
      }
    }
    const float d = eps1[idx];
    accr += (double)(d * s1r);
    acci += (double)(d * s1i);
  }
  __shared__ double sr[256], si[256];
  sr[threadIdx.x] = accr;
  si[threadIdx.x] = acci;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      sr[threadIdx.x] += sr[threadIdx.x + w];
      si[threadIdx.x] += si[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partial[2 * blockIdx.x] = sr[0];
    partial[2 * blockIdx.x + 1] = si[0];
  }
}

int sm_count() {
  int dev = 0, nsm = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  return nsm;
}

GammaC make_gamma(const double* g) {
  GammaC c;
  for (int i = 0; i < 9; ++i) c.g[i] = (float)g[i];
  return c;
}

YlmConst make_ylm(int l, int m) {
  YlmConst Y;
  const int mp = m < 0 ? -m : m;
  Y.l = l;
  Y.m = mp;
  double f1 = 1.0, f2 = 1.0;
  for (int i = 2; i <= l - mp; ++i) f1 *= i;
  for (int i = 2; i <= l + mp; ++i) f2 *= i;
  Y.norm = (float)sqrt((2.0 * l + 1.0) / (4.0 * 3.141592653589793) * f1 / f2);
  double pmm = 1.0, fact = 1.0;
  for (int i = 0; i < mp; ++i) {
    pmm *= -fact;
    fact += 2.0;
  }
  Y.pmm = (float)pmm;
  Y.neg_m = m < 0 ? 1 : 0;
  Y.neg_sign = (mp % 2 == 1) ? -1.f : 1.f;
  Y.norm_lo = 0.f;
  for (int e = 0; e <= kMaxEll; ++e) {
    Y.ca[e] = Y.cb[e] = 0.f;
    if (e >= mp + 2 && e <= l) {
      Y.ca[e] = (float)((2.0 * e - 1.0) / (double)(e - mp));
      Y.cb[e] = (float)((double)(e + mp - 1) / (double)(e - mp));
    }
  }
  return Y;
}

// the pair (l - 1, 0), (l, 0) for odd l: Y of (l, 0) plus the norm of l - 1
YlmConst make_ylm_pair(int l) {
  YlmConst Y = make_ylm(l, 0);
  Y.norm_lo = make_ylm(l - 1, 0).norm;
  return Y;
}

size_t table_floats(int J) {
  const long long L = 1LL << J;
  return (size_t)(3 * L * L + 1) * kBinStride;
}

}  // namespace

// Workspace: j_l table, partial sums and, for nb > 1, the bin-major fields
// (nb * L^3 complex64) that cuFFT transforms before they are interleaved.
namespace {
// The one workspace layout of the fields and contraction calls.
struct MpWs {
  float* T;          // radial table [n2][16]
  float* T2;         // second radial table (pairs of degrees)
  float* Pf;         // phi power, float
  double* partial;   // per-block partial sums [1024][16][16][2]
  double* dout;      // reduced S [16][16][2]
  int* status;       // bounded-wait status of the tensor-core contraction
  float2* binmajor;  // nb > 1: bin-major fields [nb][L^3]
  size_t used;
};
MpWs carve_ws(void* ws, size_t cap, int J, int nb) {
  hermes::Carver c(ws, cap);
  MpWs w;
  c.take<float>(2 * kMaxBins);  // rho double-float (kept for layout stability)
  w.T = c.take<float>(table_floats(J));
  w.T2 = c.take<float>(table_floats(J));
  w.Pf = c.take<float>((1 << J) + 1);
  w.partial = c.take<double>((size_t)1024 * kMaxBins * kMaxBins * 2);
  w.dout = c.take<double>((size_t)kMaxBins * kMaxBins * 2);
  w.status = c.take<int>(16);
  w.binmajor = nb > 1 ? c.take<float2>((size_t)nb << (3 * J)) : nullptr;
  w.used = c.used;
  return w;
}
}  // namespace

extern "C" int hermes_multipole_workspace_size(int J, int nb, size_t* bytes) {
  if (!bytes) return fail(HERMES_ERR_INVALID, "bytes is NULL");
  if (J < 4 || J > 10) return fail(HERMES_ERR_INVALID, "multipole: J=%d outside [4,10]", J);
  if (nb < 1 || nb > kMaxBins) return fail(HERMES_ERR_INVALID, "multipole: nb=%d outside [1,%d]", nb, kMaxBins);
  *bytes = carve_ws(nullptr, 0, J, nb).used;
  return HERMES_OK;
}

__global__ void mp_power_to_f32(const double* __restrict__ p, int n, float* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)p[i];
}

namespace {
// Shared tail of the fields entry points: validation, workspace carving and,
// after the caller has filled the radial table T, the Y_lm prepass, the
// batched inverse FFT and the interleave.
struct FieldsCtx {
  float* T;
  float* T2;
  float* Pf;
  float2* binmajor;
  float2* out;
  int L, nsm;
  long long N;
  cudaStream_t s;
  bool bin_major;
};

// bin_major: the caller's fields_out holds the batch as cuFFT leaves it,
// [nb][L^3] (no interleave, and the workspace needs no bin-major copy).
int fields_setup(const void* half_spec, int J, int l, int m, int nb, const double* phi_power, void* fields_out,
                 void* workspace, size_t workspace_bytes, void* stream, FieldsCtx* ctx, bool bin_major = false) {
  if (!half_spec || !phi_power || !fields_out) return fail(HERMES_ERR_INVALID, "multipole_fields: NULL argument");
  if (l < 0 || l > kMaxEll || m < -l || m > l) return fail(HERMES_ERR_INVALID, "multipole_fields: bad (l=%d, m=%d)", l, m);
  if (nb < 1 || nb > kMaxBins) return fail(HERMES_ERR_INVALID, "multipole_fields: nb=%d outside [1,%d]", nb, kMaxBins);
  size_t need = 0;
  int rc = hermes_multipole_workspace_size(J, bin_major ? 1 : nb, &need);
  if (rc) return rc;
  if (!workspace || workspace_bytes < need) return fail(HERMES_ERR_WORKSPACE, "multipole_fields: workspace %zu < %zu", workspace_bytes, need);
  ctx->L = 1 << J;
  ctx->N = 1LL << (3 * J);
  ctx->s = hermes::as_stream(stream);
  ctx->nsm = sm_count();
  ctx->bin_major = bin_major;
  const MpWs w = carve_ws(workspace, workspace_bytes, J, bin_major ? 1 : nb);
  ctx->T = w.T;
  ctx->T2 = w.T2;
  ctx->Pf = w.Pf;
  ctx->out = static_cast<float2*>(fields_out);
  ctx->binmajor = (nb > 1 && !bin_major) ? w.binmajor : ctx->out;
  mp_power_to_f32<<<(ctx->L + 1 + 255) / 256, 256, 0, ctx->s>>>(phi_power, ctx->L + 1, ctx->Pf);
  HERMES_LAUNCH_CHECK("mp_power_to_f32");
  return HERMES_OK;
}

// Inverse 3-D FFT of the fields: 0 = cuFFT's 3-D plan; 1 (default) = at
// J = 9, cuFFT's 1-D z lines (contiguous, near HBM speed) then
// fft512_strided_inverse over y and x in place of cuFFT's strided passes
// (15 fields: 19.95 ms per fields call against 25.7 ms).
std::atomic<int> g_fft_mode{1};

// pair: the window K_{l,0} + K_{l+1,0} for even l, with the radial tables
// of l in ctx.T and of l + 1 in ctx.T2 (m is 0).
int fields_run(const FieldsCtx& ctx, const void* half_spec, int J, int l, int m, int nb, bool pair = false) {
  cudaStream_t s = ctx.s;
  const YlmConst Y = pair ? make_ylm_pair(l + 1) : make_ylm(l, m);
  const float inv_n = (float)(1.0 / (double)ctx.N);
  const int grid = ctx.nsm * 8;
  const float2* half = static_cast<const float2*>(half_spec);
  const float4* T4 = reinterpret_cast<const float4*>(ctx.T);
  const float4* T4b = reinterpret_cast<const float4*>(ctx.T2);
  const long long we = (long long)(4 * ctx.L - 4) * (ctx.L / 2 + 1);
  const int grid_e = (int)std::min<long long>(grid, (we + 255) / 256);
#define HERMES_PREPASS(NB4, PAIR)                                                                               \
  do {                                                                                                          \
    mp_prepass_quad_kernel<NB4, PAIR><<<grid, 256, 0, s>>>(half, J, ctx.Pf, T4, T4b, Y, nb, ctx.binmajor, inv_n); \
    mp_prepass_edge_kernel<NB4, PAIR><<<grid_e, 256, 0, s>>>(half, J, ctx.Pf, T4, T4b, Y, nb, ctx.binmajor,      \
                                                            inv_n);                                            \
  } while (0)
  if (pair) {
    if (nb <= 4) HERMES_PREPASS(1, true);
    else if (nb <= 8) HERMES_PREPASS(2, true);
    else HERMES_PREPASS(4, true);
  } else {
    if (nb <= 4) HERMES_PREPASS(1, false);
    else if (nb <= 8) HERMES_PREPASS(2, false);
    else HERMES_PREPASS(4, false);
  }
#undef HERMES_PREPASS
  HERMES_LAUNCH_CHECK("mp_prepass_kernel");
  const int fft_mode = g_fft_mode.load();
  const bool own = J == 9 && fft_mode != 0;
  cufftHandle h;
  int rc = own ? hermes::get_plan_c2c_lines(J, nb, &h) : hermes::get_plan_c2c_batch(J, nb, &h);
  if (rc) return rc;
  cufftResult r = cufftSetStream(h, s);
  if (r != CUFFT_SUCCESS) return fail(HERMES_ERR_CUFFT, "cufftSetStream failed: %d", (int)r);
  r = cufftExecC2C(h, reinterpret_cast<cufftComplex*>(ctx.binmajor), reinterpret_cast<cufftComplex*>(ctx.binmajor),
                   CUFFT_INVERSE);
  if (r != CUFFT_SUCCESS) return fail(HERMES_ERR_CUFFT, "cufftExecC2C failed: %d", (int)r);
  if (own) {  // z lines by cuFFT above, then the y and x passes
    rc = hermes::fft512_strided_inverse(ctx.binmajor, nb, 1, s);
    if (rc) return rc;
    rc = hermes::fft512_strided_inverse(ctx.binmajor, nb, 0, s);
    if (rc) return rc;
  }
  if (nb > 1 && !ctx.bin_major) {
    long long nblk = ctx.N / kIlCells;
    if (nblk > (long long)ctx.nsm * 16) nblk = (long long)ctx.nsm * 16;
    mp_interleave_kernel<<<(int)nblk, 256, 0, s>>>(ctx.binmajor, nb, ctx.N, ctx.out);
    HERMES_LAUNCH_CHECK("mp_interleave_kernel");
  }
  return HERMES_OK;
}
}  // namespace

static int fields_radii(const void* half_spec, int J, int l, int m, const double* radii, int nb,
                        const double* phi_power, void* fields_out, void* workspace, size_t workspace_bytes,
                        void* stream, bool bin_major, bool pair = false) {
  if (!radii) return fail(HERMES_ERR_INVALID, "multipole_fields: NULL argument");
  FieldsCtx ctx;
  int rc = fields_setup(half_spec, J, l, m, nb, phi_power, fields_out, workspace, workspace_bytes, stream, &ctx,
                        bin_major);
  if (rc) return rc;
  RhoArgs hrho;
  for (int b = 0; b < kMaxBins; ++b) hrho.v[2 * b] = hrho.v[2 * b + 1] = 0.f;
  for (int b = 0; b < nb; ++b) {
    if (!(radii[b] >= 0.0)) return fail(HERMES_ERR_INVALID, "multipole_fields: radius %d must be >= 0", b);
    const double v = radii[b] / (double)ctx.L;
    hrho.v[2 * b] = (float)v;
    hrho.v[2 * b + 1] = (float)(v - (double)hrho.v[2 * b]);
  }
  mp_jl_table_kernel<<<ctx.nsm * 8, 256, 0, ctx.s>>>(ctx.T, 3 * ctx.L * ctx.L, hrho, nb, l);
  HERMES_LAUNCH_CHECK("mp_jl_table_kernel");
  if (pair) {
    mp_jl_table_kernel<<<ctx.nsm * 8, 256, 0, ctx.s>>>(ctx.T2, 3 * ctx.L * ctx.L, hrho, nb, l + 1);
    HERMES_LAUNCH_CHECK("mp_jl_table_kernel");
  }
  return fields_run(ctx, half_spec, J, l, m, nb, pair);
}

extern "C" int hermes_multipole_fields(const void* half_spec, int J, int l, int m, const double* radii,
                                       int nb, const double* phi_power, void* fields_out, void* workspace,
                                       size_t workspace_bytes, void* stream) {
  return fields_radii(half_spec, J, l, m, radii, nb, phi_power, fields_out, workspace, workspace_bytes, stream,
                      false);
}

extern "C" int hermes_multipole_fields_bm(const void* half_spec, int J, int l, int m, const double* radii,
                                          int nb, const double* phi_power, void* fields_out, void* workspace,
                                          size_t workspace_bytes, void* stream) {
  return fields_radii(half_spec, J, l, m, radii, nb, phi_power, fields_out, workspace, workspace_bytes, stream,
                      true);
}

extern "C" int hermes_multipole_set_fft(int mode) {
  if (mode < 0 || mode > 1) return fail(HERMES_ERR_INVALID, "multipole_set_fft: mode=%d outside [0, 1]", mode);
  return g_fft_mode.exchange(mode);
}

extern "C" int hermes_multipole_fields_pair_bm(const void* half_spec, int J, int l, const double* radii, int nb,
                                               const double* phi_power, void* fields_out, void* workspace,
                                               size_t workspace_bytes, void* stream) {
  if (l < 0 || l + 1 > kMaxEll || (l & 1))
    return fail(HERMES_ERR_INVALID, "multipole_fields_pair: l=%d must be even and below %d", l, kMaxEll);
  return fields_radii(half_spec, J, l, 0, radii, nb, phi_power, fields_out, workspace, workspace_bytes, stream,
                      true, true);
}

static int fields_window(const void* half_spec, int J, int l, int m, const hermes_window_t* bins, int nb,
                         const double* phi_power, void* fields_out, void* workspace, size_t workspace_bytes,
                         void* stream, bool bin_major) {
  if (!bins) return fail(HERMES_ERR_INVALID, "multipole_fields_window: NULL argument");
  if (nb < 1 || nb > kMaxBins) return fail(HERMES_ERR_INVALID, "multipole_fields_window: nb=%d", nb);
  FieldsCtx ctx;
  int rc = fields_setup(half_spec, J, l, m, nb, phi_power, fields_out, workspace, workspace_bytes, stream, &ctx,
                        bin_major);
  if (rc) return rc;
  IsoWins wins;
  memset(&wins, 0, sizeof(wins));
  for (int b = 0; b < nb; ++b) {
    const int t = bins[b].type;
    if (t != HERMES_WIN_SPHERE && t != HERMES_WIN_GAUSSIAN && t != HERMES_WIN_SHELL && t != HERMES_WIN_THICK_SHELL &&
        t != HERMES_WIN_GAUSSIAN_SHELL)
      return fail(HERMES_ERR_UNSUPPORTED, "multipole_fields_window: bin %d type %d is not an isotropic profile", b, t);
    rc = hermes::prepare_window(bins[b], ctx.L, &wins.w[b]);
    if (rc) return rc;
  }
  mp_iso_table_kernel<<<ctx.nsm * 8, 256, 0, ctx.s>>>(ctx.T, 3 * ctx.L * ctx.L, wins, nb);
  HERMES_LAUNCH_CHECK("mp_iso_table_kernel");
  return fields_run(ctx, half_spec, J, l, m, nb);
}

extern "C" int hermes_multipole_fields_window(const void* half_spec, int J, int l, int m,
                                              const hermes_window_t* bins, int nb, const double* phi_power,
                                              void* fields_out, void* workspace, size_t workspace_bytes,
                                              void* stream) {
  return fields_window(half_spec, J, l, m, bins, nb, phi_power, fields_out, workspace, workspace_bytes, stream,
                       false);
}

extern "C" int hermes_multipole_fields_window_bm(const void* half_spec, int J, int l, int m,
                                                 const hermes_window_t* bins, int nb, const double* phi_power,
                                                 void* fields_out, void* workspace, size_t workspace_bytes,
                                                 void* stream) {
  return fields_window(half_spec, J, l, m, bins, nb, phi_power, fields_out, workspace, workspace_bytes, stream,
                       true);
}

static int fields_table(const void* half_spec, int J, int l, int m, const double* tables, const int64_t* offsets,
                        const int32_t* sizes, const double* k_max, double grid_to_physical, int nb,
                        const double* phi_power, void* fields_out, void* workspace, size_t workspace_bytes,
                        void* stream, bool bin_major) {
  if (!tables || !offsets || !sizes || !k_max) return fail(HERMES_ERR_INVALID, "multipole_fields_table: NULL argument");
  if (nb < 1 || nb > kMaxBins) return fail(HERMES_ERR_INVALID, "multipole_fields_table: nb=%d", nb);
  if (!(grid_to_physical > 0.0)) return fail(HERMES_ERR_INVALID, "multipole_fields_table: grid_to_physical must be > 0");
  FieldsCtx ctx;
  int rc = fields_setup(half_spec, J, l, m, nb, phi_power, fields_out, workspace, workspace_bytes, stream, &ctx,
                        bin_major);
  if (rc) return rc;
  TabArgs ta;
  memset(&ta, 0, sizeof(ta));
  for (int b = 0; b < nb; ++b) {
    if (sizes[b] < 4 || offsets[b] < 0 || !(k_max[b] > 0.0))
      return fail(HERMES_ERR_INVALID, "multipole_fields_table: bin %d needs >= 4 points, offset >= 0, k_max > 0", b);
    ta.off[b] = offsets[b];
    ta.n[b] = sizes[b];
    ta.kmax[b] = k_max[b];
  }
  ta.k_scale = grid_to_physical / (double)ctx.L;
  mp_tab_table_kernel<<<ctx.nsm * 8, 256, 0, ctx.s>>>(ctx.T, 3 * ctx.L * ctx.L, tables, ta, nb);
  HERMES_LAUNCH_CHECK("mp_tab_table_kernel");
  return fields_run(ctx, half_spec, J, l, m, nb);
}

extern "C" int hermes_multipole_fields_table(const void* half_spec, int J, int l, int m, const double* tables,
                                             const int64_t* offsets, const int32_t* sizes, const double* k_max,
                                             double grid_to_physical, int nb, const double* phi_power,
                                             void* fields_out, void* workspace, size_t workspace_bytes,
                                             void* stream) {
  return fields_table(half_spec, J, l, m, tables, offsets, sizes, k_max, grid_to_physical, nb, phi_power,
                      fields_out, workspace, workspace_bytes, stream, false);
}

extern "C" int hermes_multipole_fields_table_bm(const void* half_spec, int J, int l, int m, const double* tables,
                                                const int64_t* offsets, const int32_t* sizes, const double* k_max,
                                                double grid_to_physical, int nb, const double* phi_power,
                                                void* fields_out, void* workspace, size_t workspace_bytes,
                                                void* stream) {
  return fields_table(half_spec, J, l, m, tables, offsets, sizes, k_max, grid_to_physical, nb, phi_power,
                      fields_out, workspace, workspace_bytes, stream, true);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// dependency on libcuda).
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// 4-D tensor map over bin-interleaved fields [x][y][z][16 complex] (float32
// view, innermost 32 floats), box 32 x 8 (z) x 8 (y) x 1 (x): one contraction
// tile's a2 plane, 64 rows of 128 bytes.
static int make_a2_map(const void* fields, int L, CUtensorMap* map) {
  auto enc = tensor_map_encoder();
  if (!enc) return fail(HERMES_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
  const cuuint64_t dims[4] = {2 * kBinStride, (cuuint64_t)L, (cuuint64_t)L, (cuuint64_t)L};
  const cuuint64_t row = sizeof(float) * 2 * kBinStride;
  const cuuint64_t strides[3] = {row, row * L, row * L * L};
  const cuuint32_t box[4] = {2 * kBinStride, ct::TZ, ct::TY, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<void*>(fields), dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(HERMES_ERR_CUDA, "cuTensorMapEncodeTiled failed: %d", (int)r);
  return HERMES_OK;
}

// 4-D tensor map over bin-major fields [bin][x][y][z] (float32 view: z as 2L
// floats), box 16 floats (8 z) x 8 (y) x 1 (x) x 16 (bins; bins >= nb read
// as zeros): one contraction tile's a2 plane as [bin][8 y][8 z] complex.
static int make_a2_map_bm(const void* fields, int L, int nb, CUtensorMap* map) {
  auto enc = tensor_map_encoder();
  if (!enc) return fail(HERMES_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
  const cuuint64_t dims[4] = {2 * (cuuint64_t)L, (cuuint64_t)L, (cuuint64_t)L, (cuuint64_t)nb};
  const cuuint64_t row = sizeof(float) * 2 * (cuuint64_t)L;
  const cuuint64_t strides[3] = {row, row * L, row * L * L};
  const cuuint32_t box[4] = {2 * ct::TZ, ct::TY, 1, kBinStride};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<void*>(fields), dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(HERMES_ERR_CUDA, "cuTensorMapEncodeTiled failed: %d", (int)r);
  return HERMES_OK;
}

enum { kEngineTensor = 0, kEngineSimt = 1, kEngineTensorBinMajor = 2 };

// Launches the contraction and the float64 reduction into dout [16][16][2]
// (already multiplied by `scale`), with no host synchronisation.  engine:
// tensor-core bin product (mp_contract_tc_kernel) or FP32 CUDA cores
// (mp_contract_kernel) on the fields layout of hermes_multipole_fields, or
// the tensor-core kernel on the bin-major layout of
// hermes_multipole_fields_bm.
static int mp_contract_launch(const float* eps1, const void* fields2, int nb2, const void* fields3, int nb3,
                              int conj_sign, const double* gamma, int J, int chunk_x, int ctas_per_sm, double scale,
                              double* dout, void* workspace, size_t workspace_bytes, cudaStream_t s, int engine,
                              int packed = 0) {
  if (!eps1 || !fields2 || !gamma || !dout) return fail(HERMES_ERR_INVALID, "multipole_contract: NULL argument");
  if (nb2 < 1 || nb2 > kMaxBins) return fail(HERMES_ERR_INVALID, "multipole_contract: nb2=%d", nb2);
  const int conj_src = fields3 == nullptr;
  if (conj_src) {
    nb3 = nb2;
    if (conj_sign != 1 && conj_sign != -1) return fail(HERMES_ERR_INVALID, "multipole_contract: conj_sign must be +-1");
  }
  if (nb3 < 1 || nb3 > kMaxBins) return fail(HERMES_ERR_INVALID, "multipole_contract: nb3=%d", nb3);
  if (J < 4 || J > 10) return fail(HERMES_ERR_INVALID, "multipole_contract: J=%d outside [4,10]", J);
  const int L = 1 << J;
  // default x-chunk: 128 planes from L = 256 up (what the tile autotuner picks
  // there: the 4-plane halo costs 3% and work items still outnumber the CTAs),
  // else min(64, L)
  if (chunk_x == 0) chunk_x = L >= 256 ? 128 : (L < ct::kMaxCX ? L : ct::kMaxCX);
  if (chunk_x < 1 || chunk_x > L || (chunk_x & (chunk_x - 1)) != 0)
    return fail(HERMES_ERR_INVALID, "multipole_contract: chunk_x=%d must be a power of two in [1, L=%d]", chunk_x, L);
  if (ctas_per_sm == 0) ctas_per_sm = 2;
  if (ctas_per_sm < 1 || ctas_per_sm > 2) return fail(HERMES_ERR_INVALID, "multipole_contract: ctas_per_sm=%d", ctas_per_sm);
  size_t need = 0;
  int rc = hermes_multipole_workspace_size(J, 1, &need);
  if (rc) return rc;
  if (!workspace || workspace_bytes < need)
    return fail(HERMES_ERR_WORKSPACE, "multipole_contract: workspace %zu < %zu", workspace_bytes, need);
  const MpWs w = carve_ws(workspace, workspace_bytes, J, 1);
  static bool smem_set[3][64] = {{false}};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64 || !smem_set[engine][dev]) {  // once per device, before any stream capture
    if (engine == kEngineTensor)
      HERMES_CUDA_TRY(cudaFuncSetAttribute(mp_contract_tc_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)tcc::kSmem));
    else if (engine == kEngineTensorBinMajor)
      HERMES_CUDA_TRY(cudaFuncSetAttribute(mp_contract_tc_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)tcc::kSmem));
    else
      HERMES_CUDA_TRY(cudaFuncSetAttribute(mp_contract_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)ct::kSmem));
    if (dev >= 0 && dev < 64) smem_set[engine][dev] = true;
  }
  // field layout follows hermes_multipole_fields: [cell][16] for nb > 1, [cell] for nb == 1
  ContractArgs A;
  A.eps1 = eps1;
  A.f2 = static_cast<const float2*>(fields2);
  A.src3 = static_cast<const float2*>(conj_src ? fields2 : fields3);
  A.s2 = nb2 == 1 ? 1 : kBinStride;
  A.s3 = conj_src ? A.s2 : (nb3 == 1 ? 1 : kBinStride);
  A.bstride = 1LL << (3 * J);
  A.nb3s = nb3;
  A.conj_src = conj_src;
  A.sign = (float)conj_sign;
  A.packed = packed;
  A.J = J;
  A.CX = chunk_x;
  A.gm = make_gamma(gamma);
  A.partial = w.partial;
  A.status = w.status;
  const int n_items = (L / A.CX) * (L / ct::TY) * (L / ct::TZ);
  int nblk = ctas_per_sm * sm_count();
  if (nblk > n_items) nblk = n_items;
  if (nblk > 1024) nblk = 1024;
  if (engine == kEngineTensor || engine == kEngineTensorBinMajor) {
    CUtensorMap map;
    memset(&map, 0, sizeof(map));
    if (engine == kEngineTensorBinMajor) {
      rc = make_a2_map_bm(fields2, L, nb2, &map);
      if (rc) return rc;
    } else if (A.s2 == kBinStride) {
      rc = make_a2_map(fields2, L, &map);
      if (rc) return rc;
    }
    HERMES_CUDA_TRY(cudaMemsetAsync(w.status, 0, sizeof(int), s));
    if (engine == kEngineTensorBinMajor)
      mp_contract_tc_kernel<true><<<nblk, ct::kThreads, tcc::kSmem, s>>>(A, map);
    else
      mp_contract_tc_kernel<false><<<nblk, ct::kThreads, tcc::kSmem, s>>>(A, map);
    HERMES_LAUNCH_CHECK("mp_contract_tc_kernel");
  } else {
    mp_contract_kernel<<<nblk, ct::kThreads, ct::kSmem, s>>>(A);
    HERMES_LAUNCH_CHECK("mp_contract_kernel");
  }
  mp_reduce_kernel<<<kMaxBins * kMaxBins * 2, 256, 0, s>>>(w.partial, nblk, kMaxBins * kMaxBins * 2, dout, scale);
  HERMES_LAUNCH_CHECK("mp_reduce_kernel");
  return HERMES_OK;
}

extern "C" int hermes_multipole_contract(const float* eps1, const void* fields2, int nb2, const void* fields3,
                                         int nb3, int conj_sign, const double* gamma, int J, double* out,
                                         void* workspace, size_t workspace_bytes, void* stream) {
  if (!out) return fail(HERMES_ERR_INVALID, "multipole_contract: NULL argument");
  if (J < 4 || J > 10) return fail(HERMES_ERR_INVALID, "multipole_contract: J=%d outside [4,10]", J);
  size_t need = 0;
  int rc = hermes_multipole_workspace_size(J, 1, &need);
  if (rc) return rc;
  if (!workspace || workspace_bytes < need)
    return fail(HERMES_ERR_WORKSPACE, "multipole_contract: workspace %zu < %zu", workspace_bytes, need);
  const MpWs w = carve_ws(workspace, workspace_bytes, J, 1);
  cudaStream_t s = hermes::as_stream(stream);
  const double scale = 4.0 * 3.141592653589793 / (double)(1LL << (3 * J));
  rc = mp_contract_launch(eps1, fields2, nb2, fields3, nb3, conj_sign, gamma, J, 0, 0, scale, w.dout, workspace,
                          workspace_bytes, s, kEngineTensor);
  if (rc) return rc;
  if (fields3 == nullptr) nb3 = nb2;
  std::vector<double> h((size_t)kMaxBins * kMaxBins * 2);
  int status = 0;
  HERMES_CUDA_TRY(cudaMemcpyAsync(h.data(), w.dout, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, s));
  HERMES_CUDA_TRY(cudaMemcpyAsync(&status, w.status, sizeof(int), cudaMemcpyDeviceToHost, s));
  HERMES_CUDA_TRY(cudaStreamSynchronize(s));
  if (status != 0)
    return fail(HERMES_ERR_CUDA, "multipole_contract: bounded wait %d in the tensor-core kernel gave up", status);
  for (int a = 0; a < nb2; ++a)
    for (int b = 0; b < nb3; ++b) {
      out[(a * nb3 + b) * 2] = h[(a * kMaxBins + b) * 2];
      out[(a * nb3 + b) * 2 + 1] = h[(a * kMaxBins + b) * 2 + 1];
    }
  return HERMES_OK;
}

static int contract_async(const float* eps1, const void* fields2, int nb2, const void* fields3, int nb3,
                          int conj_sign, const double* gamma, int J, int chunk_x, int ctas_per_sm, double* dev_out,
                          void* workspace, size_t workspace_bytes, void* stream, int engine, int packed = 0) {
  const double scale = 4.0 * 3.141592653589793 / (double)(1LL << (3 * (J < 0 ? 0 : (J > 10 ? 10 : J))));
  return mp_contract_launch(eps1, fields2, nb2, fields3, nb3, conj_sign, gamma, J, chunk_x, ctas_per_sm, scale,
                            dev_out, workspace, workspace_bytes, hermes::as_stream(stream), engine, packed);
}

extern "C" int hermes_multipole_contract_async(const float* eps1, const void* fields2, int nb2, const void* fields3,
                                               int nb3, int conj_sign, const double* gamma, int J, int chunk_x,
                                               int ctas_per_sm, double* dev_out, void* workspace,
                                               size_t workspace_bytes, void* stream) {
  return contract_async(eps1, fields2, nb2, fields3, nb3, conj_sign, gamma, J, chunk_x, ctas_per_sm, dev_out,
                        workspace, workspace_bytes, stream, kEngineTensor);
}

extern "C" int hermes_multipole_contract_simt_async(const float* eps1, const void* fields2, int nb2,
                                                    const void* fields3, int nb3, int conj_sign, const double* gamma,
                                                    int J, int chunk_x, int ctas_per_sm, double* dev_out,
                                                    void* workspace, size_t workspace_bytes, void* stream) {
  return contract_async(eps1, fields2, nb2, fields3, nb3, conj_sign, gamma, J, chunk_x, ctas_per_sm, dev_out,
                        workspace, workspace_bytes, stream, kEngineSimt);
}

extern "C" int hermes_multipole_contract_bm_async(const float* eps1, const void* fields2, int nb2,
                                                  const void* fields3, int nb3, int conj_sign, const double* gamma,
                                                  int J, int chunk_x, int ctas_per_sm, double* dev_out,
                                                  void* workspace, size_t workspace_bytes, void* stream) {
  return contract_async(eps1, fields2, nb2, fields3, nb3, conj_sign, gamma, J, chunk_x, ctas_per_sm, dev_out,
                        workspace, workspace_bytes, stream, kEngineTensorBinMajor);
}

// fields = a_{l,0} + a_{l+1,0} from hermes_multipole_fields_pair_bm: with
// a3 = conj(fields), the real part of a2 G is sum a_{l,0} G(a_{l,0}) =
// S_{l,0} and the product of the imaginary parts is
// sum (a_{l+1,0}/i) G(-a_{l+1,0}/i) = sum a_{l+1,0} G(a_{l+1,0}) = S_{l+1,0},
// read as separate blocks of the tensor-core accumulator.
extern "C" int hermes_multipole_contract_pair_bm_async(const float* eps1, const void* fields, int nb,
                                                       const double* gamma, int J, int chunk_x, int ctas_per_sm,
                                                       double* dev_out, void* workspace, size_t workspace_bytes,
                                                       void* stream) {
  return contract_async(eps1, fields, nb, nullptr, nb, 1, gamma, J, chunk_x, ctas_per_sm, dev_out, workspace,
                        workspace_bytes, stream, kEngineTensorBinMajor, 1);
}

extern "C" int hermes_multipole_contract_status(const void* workspace, size_t workspace_bytes, int J, int* status,
                                                void* stream) {
  if (!workspace || !status) return fail(HERMES_ERR_INVALID, "multipole_contract_status: NULL argument");
  if (J < 4 || J > 10) return fail(HERMES_ERR_INVALID, "multipole_contract_status: J=%d outside [4,10]", J);
  const MpWs w = carve_ws(const_cast<void*>(workspace), workspace_bytes, J, 1);
  cudaStream_t s = hermes::as_stream(stream);
  HERMES_CUDA_TRY(cudaMemcpyAsync(status, w.status, sizeof(int), cudaMemcpyDeviceToHost, s));
  HERMES_CUDA_TRY(cudaStreamSynchronize(s));
  return HERMES_OK;
}

extern "C" int hermes_multipole_contract_plain(const float* eps1, const void* a2, const void* a3,
                                               const double* gamma, int J, double* out, void* workspace,
                                               size_t workspace_bytes, void* stream) {
  if (!eps1 || !a2 || !a3 || !gamma || !out) return fail(HERMES_ERR_INVALID, "contract_plain: NULL argument");
  if (J < 4 || J > 10) return fail(HERMES_ERR_INVALID, "contract_plain: J=%d outside [4,10]", J);
  const int nblk = sm_count() * 8;
  if (!workspace || workspace_bytes < sizeof(double) * (2 * (size_t)nblk + 2))
    return fail(HERMES_ERR_WORKSPACE, "contract_plain: workspace too small");
  cudaStream_t s = hermes::as_stream(stream);
  double* partial = static_cast<double*>(workspace);
  double* dout = partial + 2 * nblk;
  mp_plain_kernel<<<nblk, 256, 0, s>>>(eps1, static_cast<const float2*>(a2), static_cast<const float2*>(a3), J,
                                       make_gamma(gamma), partial);
  HERMES_LAUNCH_CHECK("mp_plain_kernel");
  mp_reduce_kernel<<<2, 256, 0, s>>>(partial, nblk, 2, dout);
  HERMES_LAUNCH_CHECK("mp_reduce_kernel");
  double h[2];
  HERMES_CUDA_TRY(cudaMemcpyAsync(h, dout, sizeof(h), cudaMemcpyDeviceToHost, s));
  HERMES_CUDA_TRY(cudaStreamSynchronize(s));
  const double scale = 4.0 * 3.141592653589793 / (double)(1LL << (3 * J));
  out[0] = h[0] * scale;
  out[1] = h[1] * scale;
  return HERMES_OK;
}
