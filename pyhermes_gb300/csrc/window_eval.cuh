// Device evaluation of the built-in Fourier-space window kernels and of the
// scaling-function-weighted image sum that turns them into FFT kernels.
//
// Window transfer functions restate pyhermes/utils/window_functions.py:29-438
// (same formulas, same special cases); the image sums restate
// pyhermes/utils/convolution.py:14-38 + 263-281 (octant kernel folded to the
// rFFT grid) and :73-252 (full real / complex rFFT kernels).
//
// Precision: float32 arithmetic, except the Fourier phase.  A kernel such as
// sin(2*pi*k*R) at |k|*R ~ 100 cycles would lose ~1e-5 in float32 when the
// product k*R is formed directly, so every phase x = sqrt(n2) * (R/L) is
// carried as a double-float (hi + lo) pair, reduced modulo 1 exactly, and
// fed to sinpif/cospif.  Small-argument branches use Taylor series where the
// closed form cancels (sphere, cosine-wavelet).
#pragma once

#include <math.h>
#include <stdint.h>

#include "../../include/hermes_gb300.h"

namespace hermes {

constexpr float kTwoPi = 6.28318530717958647692f;

// Window descriptor prepared on the host (see prepare_window in spectral.cu).
struct WinDev {
  int type;
  int mode;        // HERMES_KMODE_*
  int zero_k0;     // force K(0,0,0) = 0
  int los_axis;    // 0/1/2 when the line of sight is a coordinate axis, else -1
  float len[4];    // lengths in grid units
  float rho_hi[4]; // double-float len/L (phase per unit integer frequency)
  float rho_lo[4];
  float los[3];    // unit line of sight
  float los_hi[3], los_lo[3];  // double-float los/L ... times H/L folded below
  float c0, c1;    // per-type constants (normalisations, thick-shell weights)
  float scale;     // overall multiplier
};

// Double-float square root of a non-negative integer n2 (< 2^24 exactly).
__device__ __forceinline__ void df_sqrt_int(int n2, float& hi, float& lo) {
  float fn = (float)n2;
  hi = sqrtf(fn);
  if (hi > 0.f) {
    float r = fmaf(-hi, hi, fn);  // exact residual
    lo = r / (2.f * hi);
  } else {
    lo = 0.f;
  }
}

// Product of two double-float numbers (a_hi+a_lo)*(b_hi+b_lo) as hi + lo.
__device__ __forceinline__ void df_mul(float ah, float al, float bh, float bl, float& ph, float& pl) {
  ph = ah * bh;
  pl = fmaf(ah, bh, -ph);
  pl = fmaf(ah, bl, pl);
  pl = fmaf(al, bh, pl);
}

// Fractional part in [-0.5, 0.5] of a double-float value (exact reduction).
__device__ __forceinline__ float df_frac(float hi, float lo) {
  float r = rintf(hi);
  return (hi - r) + lo;
}

// sin(2*pi*x), cos(2*pi*x) for a double-float x.
__device__ __forceinline__ void sincos_2pi_df(float hi, float lo, float& s, float& c) {
  float f = df_frac(hi, lo);
  sincospif(2.f * f, &s, &c);
}

// sphere: 3 (sin q - q cos q) / q^3, q = 2 pi x, with W(0) = 1.
__device__ __forceinline__ float w_sphere_df(float xh, float xl) {
  float q = kTwoPi * (xh + xl);
  if (q == 0.f) return 1.f;
  if (q < 0.2f) {
    float q2 = q * q;
    return 1.f + q2 * (-0.1f + q2 * (1.f / 280.f + q2 * (-1.f / 15120.f + q2 * (1.f / 1330560.f))));
  }
  float s, c;
  sincos_2pi_df(xh, xl, s, c);
  return 3.f * (s - q * c) / (q * q * q);
}

__device__ __forceinline__ float w_sinc_df(float xh, float xl) {
  float q = kTwoPi * (xh + xl);
  if (q == 0.f) return 1.f;
  float s, c;
  sincos_2pi_df(xh, xl, s, c);
  return s / q;
}

// Cylindrical Bessel J0 / J1 by the rational approximations of
// pyhermes/utils/special_functions.py:131-215; the large-argument branch
// takes the phase as a double-float x with q = 2 pi x.
__device__ __forceinline__ float bessel_j0_df(float xh, float xl) {
  float ax = kTwoPi * (xh + xl);
  if (ax < 8.f) {
    float y = ax * ax;
    float a1 = 57568490574.0f + y * (-13362590354.0f + y * (651619640.7f + y * (-11214424.18f + y * (77392.33017f + y * -184.9052456f))));
    float a2 = 57568490411.0f + y * (1029532985.0f + y * (9494680.718f + y * (59272.64853f + y * (267.8532712f + y))));
    return a1 / a2;
  }
  float z = 8.f / ax, y = z * z;
  float a1 = 1.f + y * (-0.1098628627e-2f + y * (0.2734510407e-4f + y * (-0.2073370639e-5f + y * 0.2093887211e-6f)));
  float a2 = -0.1562499995e-1f + y * (0.1430488765e-3f + y * (-0.6911147651e-5f + y * (0.7621095161e-6f - y * 0.934945152e-7f)));
  // xx = ax - 0.785398164 ; cos(xx) = cospi(2x - 1/4)
  float s, c;
  sincospif(2.f * df_frac(xh, xl) - 0.25f, &s, &c);
  return sqrtf(0.636619772f / ax) * (c * a1 - z * s * a2);
}

__device__ __forceinline__ float bessel_j1_df(float xh, float xl) {
  float ax = kTwoPi * (xh + xl);
  if (ax < 8.f) {
    float y = ax * ax;
    float a1 = ax * (72362614232.0f + y * (-7895059235.0f + y * (242396853.1f + y * (-2972611.439f + y * (15704.48260f + y * -30.16036606f)))));
    float a2 = 144725228442.0f + y * (2300535178.0f + y * (18583304.74f + y * (99447.43394f + y * (376.9991397f + y))));
    return a1 / a2;
  }
  float z = 8.f / ax, y = z * z;
  float a1 = 1.f + y * (0.183105e-2f + y * (-0.3516396496e-4f + y * (0.2457520174e-5f + y * -0.240337019e-6f)));
  float a2 = 0.04687499995f + y * (-0.2002690873e-3f + y * (0.8449199096e-5f + y * (-0.88228987e-6f + y * 0.105787412e-6f)));
  float s, c;
  sincospif(2.f * df_frac(xh, xl) - 0.75f, &s, &c);
  return sqrtf(0.636619772f / ax) * (c * a1 - z * s * a2);
}

// G(q) = q (q cosh q - sinh q) exp(-q^2/2) with the reference's cut-offs
// (window_functions.py:324-332); a series below q = 1 avoids cancellation.
__device__ __forceinline__ float cosine_wavelet_g(float q) {
  q = fabsf(q);
  if (q == 0.f) return 0.f;
  if (q < 1.0e-4f) return q * q * q * q / 3.f;
  if (q > 50.f) return 0.f;
  float q2 = q * q;
  float inner;  // q cosh q - sinh q
  if (q < 1.f) {
    inner = q * q2 * (1.f / 3.f + q2 * (1.f / 30.f + q2 * (1.f / 840.f + q2 * (1.f / 45360.f + q2 * (1.f / 3991680.f)))));
    return q * inner * expf(-0.5f * q2);
  }
  // q*(q cosh q - sinh q) e^{-q^2/2} = q/2 [ (q-1) e^{q - q^2/2} + (q+1) e^{-q - q^2/2} ]
  return 0.5f * q * ((q - 1.f) * expf(q - 0.5f * q2) + (q + 1.f) * expf(-q - 0.5f * q2));
}

// Isotropic windows (sphere, gaussian, shell, thick_shell, gaussian_shell)
// as functions of the integer squared frequency n2 = |k L|^2 alone.  Sets
// *ok = false for the other types.
__device__ __forceinline__ float2 window_iso_n2(const WinDev& w, int n2, bool* ok) {
  float nh, nl;
  *ok = true;
  switch (w.type) {
    case HERMES_WIN_SPHERE: {
      df_sqrt_int(n2, nh, nl);
      float xh, xl;
      df_mul(nh, nl, w.rho_hi[0], w.rho_lo[0], xh, xl);
      return make_float2(w_sphere_df(xh, xl), 0.f);
    }
    case HERMES_WIN_GAUSSIAN: {
      df_sqrt_int(n2, nh, nl);
      float q = kTwoPi * (nh + nl) * (w.rho_hi[0] + w.rho_lo[0]);
      return make_float2(expf(-0.5f * q * q), 0.f);
    }
    case HERMES_WIN_SHELL: {
      df_sqrt_int(n2, nh, nl);
      float xh, xl;
      df_mul(nh, nl, w.rho_hi[0], w.rho_lo[0], xh, xl);
      return make_float2(w_sinc_df(xh, xl), 0.f);
    }
    case HERMES_WIN_THICK_SHELL: {
      // c0 = r_out^3/den, c1 = r_in^3/den; rho[0] = r_out/L, rho[1] = r_in/L
      if (w.c0 == 0.f && w.c1 == 0.f) return make_float2(1.f, 0.f);
      df_sqrt_int(n2, nh, nl);
      float xh, xl, yh, yl;
      df_mul(nh, nl, w.rho_hi[0], w.rho_lo[0], xh, xl);
      df_mul(nh, nl, w.rho_hi[1], w.rho_lo[1], yh, yl);
      return make_float2(w.c0 * w_sphere_df(xh, xl) - w.c1 * w_sphere_df(yh, yl), 0.f);
    }
    case HERMES_WIN_GAUSSIAN_SHELL: {
      if (n2 == 0) return make_float2(1.f, 0.f);
      // c0 = R_smooth^2/den, c1 = R_shell^2/den (den = 0 -> W = 1: c0=c1=-1 marker)
      if (w.c0 < 0.f) return make_float2(1.f, 0.f);
      df_sqrt_int(n2, nh, nl);
      float xh, xl;
      df_mul(nh, nl, w.rho_hi[0], w.rho_lo[0], xh, xl);
      float s, c;
      sincos_2pi_df(xh, xl, s, c);
      float qsh = kTwoPi * (xh + xl);
      float sinc = qsh == 0.f ? 1.f : s / qsh;
      float qsm = kTwoPi * (nh + nl) * (w.rho_hi[1] + w.rho_lo[1]);
      return make_float2((w.c0 * c + w.c1 * sinc) * expf(-0.5f * qsm * qsm), 0.f);
    }
    default:
      *ok = false;
      return make_float2(0.f, 0.f);
  }
}

// One window at integer frequency indices (a, b, c) = k * L (signed), for
// the given magnitude n2 = a^2+b^2+c^2.  Returns (re, im).
__device__ __forceinline__ float2 window_at(const WinDev& w, int a, int b, int c) {
  const int n2 = a * a + b * b + c * c;
  {
    bool ok;
    const float2 v = window_iso_n2(w, n2, &ok);
    if (ok) return v;
  }
  float nh, nl;
  switch (w.type) {
    case HERMES_WIN_CUBIC: {
      // sin(pi k_i L_i)/(pi k_i L_i) per axis; rho[i] = L_i / L (double-float)
      float r = 1.f;
      const int idx[3] = {a, b, c};
#pragma unroll
      for (int ax = 0; ax < 3; ++ax) {
        float yh, yl;  // y = idx * L_i / L ; q = pi * y
        df_mul((float)idx[ax], 0.f, w.rho_hi[ax], w.rho_lo[ax], yh, yl);
        float q = 3.14159265358979323846f * (yh + yl);
        if (q != 0.f) {
          // sin(pi y) with y reduced modulo 2
          float hr = rintf(yh * 0.5f) * 2.f;
          float red = (yh - hr) + yl;
          r *= sinpif(red) / q;
        }
      }
      return make_float2(r, 0.f);
    }
    case HERMES_WIN_RING:
    case HERMES_WIN_DISK:
    case HERMES_WIN_CYLSHELL:
    case HERMES_WIN_CYLINDER: {
      // k_par = k . n ; k_perp = sqrt(max(k^2 - k_par^2, 0)); lengths R (perp), H (par)
      float perp_h, perp_l, par;  // in integer-frequency units (times 1/L later via rho)
      if (w.los_axis >= 0) {
        int cpar = w.los_axis == 0 ? a : (w.los_axis == 1 ? b : c);
        float sgn = w.los[w.los_axis];
        df_sqrt_int(n2 - cpar * cpar, perp_h, perp_l);
        par = sgn * (float)cpar;
      } else {
        par = (float)a * w.los[0] + (float)b * w.los[1] + (float)c * w.los[2];
        float kp2 = (float)n2 - par * par;
        if (kp2 < 0.f) kp2 = 0.f;
        perp_h = sqrtf(kp2);
        perp_l = 0.f;
      }
      float xh, xl, zh, zl;
      df_mul(perp_h, perp_l, w.rho_hi[0], w.rho_lo[0], xh, xl);  // k_perp R
      df_mul(par, 0.f, w.rho_hi[1], w.rho_lo[1], zh, zl);        // k_par H
      float qperp = kTwoPi * (xh + xl);
      float qpar = kTwoPi * (zh + zl);
      float perp, parf;
      if (w.type == HERMES_WIN_RING || w.type == HERMES_WIN_CYLSHELL) {
        perp = bessel_j0_df(fabsf(xh), xh < 0.f ? -xl : xl);
      } else {
        perp = qperp == 0.f ? 1.f : 2.f * bessel_j1_df(fabsf(xh), xh < 0.f ? -xl : xl) / fabsf(qperp);
      }
      float s, c2;
      sincos_2pi_df(zh, zl, s, c2);
      if (w.type == HERMES_WIN_RING || w.type == HERMES_WIN_DISK) {
        parf = c2;
      } else {
        parf = qpar == 0.f ? 1.f : s / qpar;
      }
      return make_float2(perp * parf, 0.f);
    }
    case HERMES_WIN_CW:
    case HERMES_WIN_CWS: {
      df_sqrt_int(n2, nh, nl);
      float q = kTwoPi * (nh + nl) * (w.rho_hi[0] + w.rho_lo[0]);
      return make_float2(w.c0 * cosine_wavelet_g(q), 0.f);
    }
    case HERMES_WIN_GDW: {
      df_sqrt_int(n2, nh, nl);
      float q = kTwoPi * (nh + nl) * (w.rho_hi[0] + w.rho_lo[0]);
      return make_float2(w.c0 * q * q * expf(-0.5f * q * q), 0.f);
    }
    case HERMES_WIN_DIRECTIONAL_DERIVATIVE: {
      // 2 pi i k_par ; c0 = 1/L folded into the caller's units: k = idx / L
      float kpar = ((float)a * w.los[0] + (float)b * w.los[1] + (float)c * w.los[2]) * w.c0;
      return make_float2(0.f, kTwoPi * kpar);
    }
    case HERMES_WIN_LAPLACIAN: {
      float k2 = (float)n2 * w.c0;  // c0 = 1/L^2
      return make_float2(-(kTwoPi * kTwoPi) * k2, 0.f);
    }
    case HERMES_WIN_INVERSE_LAPLACIAN: {
      if (n2 == 0) return make_float2(0.f, 0.f);
      float k2 = (float)n2 * w.c0;
      return make_float2(-1.f / ((kTwoPi * kTwoPi) * k2), 0.f);
    }
    default:
      return make_float2(__int_as_float(0x7fc00000), 0.f);
  }
}

// Cylindrical windows (ring, disk, cylshell, cylinder) with the line of sight
// on a grid axis factor into a perpendicular part f(k_perp R) and a parallel
// part g(k_par H), the same expressions as window_at.  (p, q) are the two
// integer frequency components across the line of sight, c the one along it.
__device__ __forceinline__ bool cyl_separable(const WinDev& w) {
  return w.los_axis >= 0 && (w.type == HERMES_WIN_RING || w.type == HERMES_WIN_DISK ||
                             w.type == HERMES_WIN_CYLSHELL || w.type == HERMES_WIN_CYLINDER);
}
__device__ __forceinline__ float cyl_perp(const WinDev& w, int p, int q) {
  float perp_h, perp_l, xh, xl;
  df_sqrt_int(p * p + q * q, perp_h, perp_l);
  df_mul(perp_h, perp_l, w.rho_hi[0], w.rho_lo[0], xh, xl);
  if (w.type == HERMES_WIN_RING || w.type == HERMES_WIN_CYLSHELL) return bessel_j0_df(fabsf(xh), xh < 0.f ? -xl : xl);
  const float qperp = kTwoPi * (xh + xl);
  return qperp == 0.f ? 1.f : 2.f * bessel_j1_df(fabsf(xh), xh < 0.f ? -xl : xl) / fabsf(qperp);
}
__device__ __forceinline__ float cyl_par(const WinDev& w, int c) {
  float zh, zl, s, c2;
  const float sg = w.los_axis == 0 ? w.los[0] : (w.los_axis == 1 ? w.los[1] : w.los[2]);
  df_mul(sg * (float)c, 0.f, w.rho_hi[1], w.rho_lo[1], zh, zl);
  sincos_2pi_df(zh, zl, s, c2);
  if (w.type == HERMES_WIN_RING || w.type == HERMES_WIN_DISK) return c2;
  const float qpar = kTwoPi * (zh + zl);
  return qpar == 0.f ? 1.f : s / qpar;
}

// Separable image sum for cyl_separable windows: with images u (per axis,
// weights P), K = [sum_{u_p, u_q} P P f(u_p, u_q)] [sum_{u_c} P g(u_c)], the
// 8 (bw^3 x 8) window evaluations of the plain sum become 4 (bw^2 x 4) f and
// 2 (bw x 2) g evaluations.  `sgn` = -1 selects signed images.
__device__ __forceinline__ float cyl_image_sum(const WinDev& w, int x, int y, int z, int L,
                                               const float* __restrict__ P, int bw, int sgn) {
  const int ax = w.los_axis;  // selects, not a run-time indexed array (keeps it in registers)
  const int ic = ax == 0 ? x : (ax == 1 ? y : z);
  const int ip = ax == 0 ? y : (ax == 1 ? z : x);
  const int iq = ax == 0 ? z : (ax == 1 ? x : y);
  float par = 0.f;
  for (int kk = 0; kk < bw; ++kk) {
    const int cp = kk * L + ic, cn = kk * L + (L - ic);
    par = fmaf(P[cp], cyl_par(w, cp), par);
    par = fmaf(P[cn], cyl_par(w, sgn * cn), par);
  }
  float perp = 0.f;
  for (int ii = 0; ii < bw; ++ii) {
    const int pp = ii * L + ip, pn = ii * L + (L - ip);
    for (int jj = 0; jj < bw; ++jj) {
      const int qp = jj * L + iq, qn = jj * L + (L - iq);
      perp = fmaf(P[pp] * P[qp], cyl_perp(w, pp, qp), perp);
      perp = fmaf(P[pp] * P[qn], cyl_perp(w, pp, sgn * qn), perp);
      perp = fmaf(P[pn] * P[qp], cyl_perp(w, sgn * pn, qp), perp);
      perp = fmaf(P[pn] * P[qn], cyl_perp(w, sgn * pn, sgn * qn), perp);
    }
  }
  return perp * par;
}

// FFT kernel value at rFFT/FFT grid index (x, y, z), 0 <= x,y,z < L: the
// phi-power-weighted sum over images (convolution.py:14-38 folded by
// :263-281 for octant mode; :73-252 for full/complex rFFT modes).
// P has L*bw + 1 entries (P[n] = |phi_hat(n/L)|^2).
__device__ __forceinline__ float2 kernel_value(const WinDev& w, int x, int y, int z, int L,
                                               const float* __restrict__ P, int bw) {
  float re = 0.f, im = 0.f;
  if (cyl_separable(w)) {
    re = cyl_image_sum(w, x, y, z, L, P, bw, w.mode == HERMES_KMODE_OCTANT ? 1 : -1);
  } else if (w.mode == HERMES_KMODE_OCTANT) {
    // images a in {x, L-x} per axis, all arguments positive, bandwidth shifts
    const int ax[2] = {x, L - x}, ay[2] = {y, L - y}, az[2] = {z, L - z};
    for (int ii = 0; ii < bw; ++ii)
      for (int jj = 0; jj < bw; ++jj)
        for (int kk = 0; kk < bw; ++kk) {
#pragma unroll
          for (int i = 0; i < 2; ++i) {
            const int a = ii * L + ax[i];
            const float pa = P[a];
#pragma unroll
            for (int j = 0; j < 2; ++j) {
              const int b = jj * L + ay[j];
              const float pab = pa * P[b];
#pragma unroll
              for (int k = 0; k < 2; ++k) {
                const int c = kk * L + az[k];
                const float2 v = window_at(w, a, b, c);
                const float pw = pab * P[c];
                re = fmaf(pw, v.x, re);
                im = fmaf(pw, v.y, im);
              }
            }
          }
        }
  } else {
    // signed images: +(ii*L + x) and -(ii*L + L - x)
    for (int ii = 0; ii < bw; ++ii)
      for (int jj = 0; jj < bw; ++jj)
        for (int kk = 0; kk < bw; ++kk) {
          const int ap = ii * L + x, an = ii * L + (L - x);
          const int bp = jj * L + y, bn = jj * L + (L - y);
          const int cp = kk * L + z, cn = kk * L + (L - z);
          const int A[2] = {ap, -an}, B[2] = {bp, -bn}, C[2] = {cp, -cn};
          const float PA[2] = {P[ap], P[an]}, PB[2] = {P[bp], P[bn]}, PC[2] = {P[cp], P[cn]};
#pragma unroll
          for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 2; ++j)
#pragma unroll
              for (int k = 0; k < 2; ++k) {
                const float2 v = window_at(w, A[i], B[j], C[k]);
                const float pw = PA[i] * PB[j] * PC[k];
                re = fmaf(pw, v.x, re);
                im = fmaf(pw, v.y, im);
              }
        }
  }
  if (w.zero_k0 && x == 0 && y == 0 && z == 0) {
    re = 0.f;
    im = 0.f;
  }
  return make_float2(re * w.scale, im * w.scale);
}

}  // namespace hermes
