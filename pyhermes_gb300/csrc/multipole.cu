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
//   mp_prepass_kernel    eps_hat(k) K_lm^b(k) / L^3 for every bin b, Y_lm
//                        shared by the bins, written as a batch of spectra
//   cuFFT (batched C2C)  -> a_lm^b(x) for every bin
//   mp_gfield_kernel     G^b(y) = sum_{l1,l2} Gamma3 eps1(y+l1) a3^b(y+l1-l2)
//                        (separable shared-memory passes)
//   mp_gemm_kernel       S[b1,b2] = sum_y a2^{b1}(y) G^{b2}(y): the bin x bin
//                        product over cells, float32 tiles, float64 partials
//   mp_reduce_kernel     float64 cross-block reduction
// The identity S = sum_y a2(y) G3(y) is the reference sum with y = x - l1.
// mp_plain_kernel is the reference-form contraction of one (a2, a3) pair
// (the per-sample path the batched engine is measured against).
#include <cufft.h>

#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "hermes_common.cuh"
#include "window_eval.cuh"

namespace hermes {
int get_plan_c2c_batch(int J, int batch, cufftHandle* out);
}

namespace {

using hermes::df_frac;
using hermes::df_mul;
using hermes::df_sqrt_int;
using hermes::fail;

constexpr int kMaxBins = 16;
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

// T[n2 * nb + b] = j_l(2 pi sqrt(n2) R_b / L), n2 = 0 .. n2max.
__global__ void mp_jl_table_kernel(float* __restrict__ T, int n2max, const float* __restrict__ rho,
                                   int nb, int l) {
  const long long total = (long long)(n2max + 1) * nb;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int n2 = (int)(i / nb), b = (int)(i % nb);
    float nh, nl, xh, xl;
    df_sqrt_int(n2, nh, nl);
    df_mul(nh, nl, rho[2 * b], rho[2 * b + 1], xh, xl);
    T[i] = sph_jl_f32(l, xh, xl);
  }
}

struct YlmConst {
  int l, m;          // m >= 0 here; negative m handled by the caller's flag
  float norm;        // sqrt((2l+1)/(4pi) (l-m)!/(l+m)!)
  float pmm;         // (-1)^m (2m-1)!!
  int neg_m;         // requested m < 0
  float neg_sign;    // (-1)^|m|
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
        pl = ((2.f * e - 1.f) * ct * p1 - (e + Y.m - 1.f) * p2) / (float)(e - Y.m);
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

// out[b][k] = eps_hat(k) * K_lm^b(k) / L^3 on the full FFT grid; eps_hat
// comes from the half spectrum of a real field (Hermitian expansion).
template <int NB>
__global__ void __launch_bounds__(256)
mp_prepass_kernel(const float2* __restrict__ half, int J, const float* __restrict__ P,
                  const float* __restrict__ T, YlmConst Y, int nb, float2* __restrict__ out, float inv_n) {
  const int L = 1 << J, H = L / 2 + 1, Lm = L - 1;
  const long long N = 1LL << (3 * J);
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < N;
       idx += (long long)gridDim.x * blockDim.x) {
    const int z = (int)(idx & Lm), y = (int)((idx >> J) & Lm), x = (int)(idx >> (2 * J));
    float2 e;
    if (z <= L / 2) {
      e = half[((long long)x * L + y) * H + z];
    } else {
      const float2 t = half[((long long)((L - x) & Lm) * L + ((L - y) & Lm)) * H + (L - z)];
      e = make_float2(t.x, -t.y);
    }
    float accr[NB], acci[NB];
#pragma unroll
    for (int b = 0; b < NB; ++b) accr[b] = acci[b] = 0.f;
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
          const float2 yv = ylm_at(Y, ia[i], ib[j], ic[k], n2);
          const float yr = pw * yv.x, yi = pw * yv.y;
          const float* tr = T + (long long)n2 * nb;
#pragma unroll
          for (int b = 0; b < NB; ++b) {
            if (b < nb) {
              const float jl = __ldg(tr + b);
              accr[b] = fmaf(jl, yr, accr[b]);
              acci[b] = fmaf(jl, yi, acci[b]);
            }
          }
        }
    const float er = e.x * inv_n, ei = e.y * inv_n;
#pragma unroll
    for (int b = 0; b < NB; ++b)
      if (b < nb) out[(long long)b * N + idx] = make_float2(er * accr[b] - ei * acci[b], er * acci[b] + ei * accr[b]);
  }
}

// ---- G fields ------------------------------------------------------------
// Output tile TXxTYxTZ cells; a3 halo [-2, +2]; eps1 halo [0, +2].
constexpr int GX = 4, GY = 8, GZ = 16;
constexpr int GThreads = 512;
constexpr int AX_ = GX + 4, AY_ = GY + 4, AZ_ = GZ + 4;    // a3 halo 8x12x20
constexpr int ZY_ = GY + 4, ZZ_ = GZ + 2;                    // z-pass region 8x12x18
constexpr int YY_ = GY + 2;                                  // y-pass region 8x10x18
constexpr int EX_ = GX + 2, EY_ = GY + 2, EZ_ = GZ + 2;      // eps halo 6x10x18
constexpr int kA3 = AX_ * AY_ * AZ_;
constexpr int kAz = AX_ * ZY_ * ZZ_;
constexpr int kAyz = AX_ * YY_ * ZZ_;
constexpr int kEps = EX_ * EY_ * EZ_;

struct GammaC {
  float g[9];  // Gamma[l1][l2], row-major
};

// a3 source: fields3 (nb3 fields) or sign * conj(fields2)
__global__ void __launch_bounds__(GThreads)
mp_gfield_kernel(const float* __restrict__ eps1, const float2* __restrict__ src, int conj_src, float sign,
                 int nb, int J, GammaC gm, float2* __restrict__ gout) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* a3 = reinterpret_cast<float2*>(smem_raw);          // kA3 (aliased by ayz)
  float2* ayz = a3;                                            // 9 * kAyz
  float2* az = ayz + 9 * kAyz;                                 // 3 * kAz
  float* eh = reinterpret_cast<float*>(az + 3 * kAz);         // kEps
  const int L = 1 << J, Lm = L - 1;
  const long long N = 1LL << (3 * J);
  const int ntz = L / GZ, nty = L / GY;
  const int tile = blockIdx.x;
  const int x0 = (tile / (ntz * nty)) * GX, y0 = ((tile / ntz) % nty) * GY, z0 = (tile % ntz) * GZ;
  const int tid = threadIdx.x;

  for (int i = tid; i < kEps; i += blockDim.x) {
    const int z = i % EZ_, y = (i / EZ_) % EY_, x = i / (EZ_ * EY_);
    eh[i] = eps1[(((long long)((x0 + x) & Lm)) * L + ((y0 + y) & Lm)) * L + ((z0 + z) & Lm)];
  }
  for (int b = 0; b < nb; ++b) {
    const float2* f = src + (long long)b * N;
    __syncthreads();  // previous bin's readers of ayz are done
    for (int i = tid; i < kA3; i += blockDim.x) {
      const int z = i % AZ_, y = (i / AZ_) % AY_, x = i / (AZ_ * AY_);
      float2 v = f[(((long long)((x0 - 2 + x) & Lm)) * L + ((y0 - 2 + y) & Lm)) * L + ((z0 - 2 + z) & Lm)];
      if (conj_src) v = make_float2(sign * v.x, -sign * v.y);
      a3[i] = v;
    }
    __syncthreads();
    // z-pass: az[l1z][x][y][z'] = sum_l2z G[l1z][l2z] a3[x][y][z' + 2 - l2z], z' in [0, GZ+2)
    for (int i = tid; i < AX_ * ZY_ * ZZ_; i += blockDim.x) {
      const int z = i % ZZ_, y = (i / ZZ_) % ZY_, x = i / (ZZ_ * ZY_);
      const float2* col = a3 + (x * AY_ + y) * AZ_ + z + 2;
      const float2 v0 = col[0], v1 = col[-1], v2 = col[-2];
#pragma unroll
      for (int l1 = 0; l1 < 3; ++l1) {
        const float g0 = gm.g[l1 * 3 + 0], g1 = gm.g[l1 * 3 + 1], g2 = gm.g[l1 * 3 + 2];
        az[l1 * kAz + i] = make_float2(g0 * v0.x + g1 * v1.x + g2 * v2.x, g0 * v0.y + g1 * v1.y + g2 * v2.y);
      }
    }
    __syncthreads();
    // y-pass: ayz[l1y][l1z][x][y'][z'] = sum_l2y G[l1y][l2y] az[l1z][x][y' + 2 - l2y][z'], y' in [0, GY+2)
    for (int i = tid; i < AX_ * YY_ * ZZ_; i += blockDim.x) {
      const int z = i % ZZ_, y = (i / ZZ_) % YY_, x = i / (ZZ_ * YY_);
      const int base = (x * ZY_ + y + 2) * ZZ_ + z;
#pragma unroll
      for (int l1z = 0; l1z < 3; ++l1z) {
        const float2 v0 = az[l1z * kAz + base], v1 = az[l1z * kAz + base - ZZ_], v2 = az[l1z * kAz + base - 2 * ZZ_];
#pragma unroll
        for (int l1y = 0; l1y < 3; ++l1y) {
          const float g0 = gm.g[l1y * 3 + 0], g1 = gm.g[l1y * 3 + 1], g2 = gm.g[l1y * 3 + 2];
          ayz[(l1y * 3 + l1z) * kAyz + i] =
              make_float2(g0 * v0.x + g1 * v1.x + g2 * v2.x, g0 * v0.y + g1 * v1.y + g2 * v2.y);
        }
      }
    }
    __syncthreads();
    // x-pass + gather: G(y) = sum_l1 e(y+l1) sum_l2x G[l1x][l2x] ayz[l1y][l1z][x + 2 + l1x - l2x][y + l1y][z + l1z]
    for (int i = tid; i < GX * GY * GZ; i += blockDim.x) {
      const int z = i % GZ, y = (i / GZ) % GY, x = i / (GZ * GY);
      float gr = 0.f, gi = 0.f;
#pragma unroll
      for (int l1y = 0; l1y < 3; ++l1y)
#pragma unroll
        for (int l1z = 0; l1z < 3; ++l1z) {
          const float2* row = ayz + (l1y * 3 + l1z) * kAyz + (y + l1y) * ZZ_ + (z + l1z);
          float2 v[5];
#pragma unroll
          for (int d = 0; d < 5; ++d) v[d] = row[(x + d) * (YY_ * ZZ_)];  // x offset d - 2
#pragma unroll
          for (int l1x = 0; l1x < 3; ++l1x) {
            const float ev = eh[((x + l1x) * EY_ + (y + l1y)) * EZ_ + (z + l1z)];
            // ayz x index: x + 2 + l1x - l2x  -> v[2 + l1x - l2x]
            const float g0 = gm.g[l1x * 3 + 0], g1 = gm.g[l1x * 3 + 1], g2 = gm.g[l1x * 3 + 2];
            const float ur = g0 * v[2 + l1x].x + g1 * v[1 + l1x].x + g2 * v[l1x].x;
            const float ui = g0 * v[2 + l1x].y + g1 * v[1 + l1x].y + g2 * v[l1x].y;
            gr = fmaf(ev, ur, gr);
            gi = fmaf(ev, ui, gi);
          }
        }
      gout[(long long)b * N + (((long long)(x0 + x)) * L + (y0 + y)) * L + (z0 + z)] = make_float2(gr, gi);
    }
  }
}

// ---- bin x bin product over cells ----------------------------------------
// S[b1][b2] = sum_y A[b1][y] * B[b2][y] (complex, no conjugation).
constexpr int kGemmThreads = 256;
constexpr int kGemmChunk = 64;

__global__ void __launch_bounds__(kGemmThreads)
mp_gemm_kernel(const float2* __restrict__ A, int na, const float2* __restrict__ B, int nbb, long long N,
               double* __restrict__ partial) {
  __shared__ float2 sa[kMaxBins][kGemmChunk + 1];
  __shared__ float2 sb[kMaxBins][kGemmChunk + 1];
  // thread -> (b1 pair, b2 pair): 8 x 8 = 64 blocks of 2x2, 4 threads per block split the chunk
  const int blk = threadIdx.x >> 2, part = threadIdx.x & 3;
  const int r0 = (blk >> 3) * 2, c0 = (blk & 7) * 2;
  double acc[2][2][2];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;
  for (long long base = (long long)blockIdx.x * kGemmChunk; base < N; base += (long long)gridDim.x * kGemmChunk) {
    __syncthreads();
    for (int i = threadIdx.x; i < kMaxBins * kGemmChunk; i += blockDim.x) {
      const int b = i / kGemmChunk, k = i % kGemmChunk;
      const long long y = base + k;
      sa[b][k] = (b < na && y < N) ? A[(long long)b * N + y] : make_float2(0.f, 0.f);
      sb[b][k] = (b < nbb && y < N) ? B[(long long)b * N + y] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    float f[2][2][2] = {};
    for (int k = part; k < kGemmChunk; k += 4) {
      const float2 a0 = sa[r0][k], a1 = sa[r0 + 1][k], b0 = sb[c0][k], b1 = sb[c0 + 1][k];
      f[0][0][0] += a0.x * b0.x - a0.y * b0.y; f[0][0][1] += a0.x * b0.y + a0.y * b0.x;
      f[0][1][0] += a0.x * b1.x - a0.y * b1.y; f[0][1][1] += a0.x * b1.y + a0.y * b1.x;
      f[1][0][0] += a1.x * b0.x - a1.y * b0.y; f[1][0][1] += a1.x * b0.y + a1.y * b0.x;
      f[1][1][0] += a1.x * b1.x - a1.y * b1.y; f[1][1][1] += a1.x * b1.y + a1.y * b1.x;
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        acc[i][j][0] += (double)f[i][j][0];
        acc[i][j][1] += (double)f[i][j][1];
      }
  }
  // combine the 4 parts of each block (adjacent lanes)
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        double v = acc[i][j][c];
        v += __shfl_xor_sync(0xffffffffu, v, 1);
        v += __shfl_xor_sync(0xffffffffu, v, 2);
        acc[i][j][c] = v;
      }
  if (part == 0) {
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int b1 = r0 + i, b2 = c0 + j;
        double* o = partial + ((long long)blockIdx.x * kMaxBins * kMaxBins + b1 * kMaxBins + b2) * 2;
        o[0] = acc[i][j][0];
        o[1] = acc[i][j][1];
      }
  }
}

// out[o] = sum over blocks of partial[blk * nout + o]
__global__ void mp_reduce_kernel(const double* __restrict__ partial, int nblocks, int nout, double* __restrict__ out) {
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
  if (threadIdx.x == 0) out[o] = sh[0];
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
  return Y;
}

size_t table_floats(int J, int nb) {
  const long long L = 1LL << J;
  return (size_t)(3 * L * L + 1) * nb;
}

}  // namespace

extern "C" int hermes_multipole_workspace_size(int J, int nb, size_t* bytes) {
  if (!bytes) return fail(HERMES_ERR_INVALID, "bytes is NULL");
  if (J < 3 || J > 10) return fail(HERMES_ERR_INVALID, "multipole: J=%d outside [3,10]", J);
  if (nb < 1 || nb > kMaxBins) return fail(HERMES_ERR_INVALID, "multipole: nb=%d outside [1,%d]", nb, kMaxBins);
  const size_t N = (size_t)1 << (3 * J);
  hermes::Carver c(nullptr, 0);
  c.take<float>(2 * kMaxBins);         // rho double-float
  c.take<float>(table_floats(J, nb));  // j_l table
  c.take<float>((1 << J) + 1);         // phi power float
  c.take<float2>((size_t)nb * N);      // G fields
  c.take<double>((size_t)4096 * kMaxBins * kMaxBins * 2);  // partials
  c.take<double>((size_t)kMaxBins * kMaxBins * 2);
  *bytes = c.used;
  return HERMES_OK;
}

__global__ void mp_power_to_f32(const double* __restrict__ p, int n, float* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)p[i];
}

extern "C" int hermes_multipole_fields(const void* half_spec, int J, int l, int m, const double* radii,
                                       int nb, const double* phi_power, void* fields_out, void* workspace,
                                       size_t workspace_bytes, void* stream) {
  if (!half_spec || !radii || !phi_power || !fields_out) return fail(HERMES_ERR_INVALID, "multipole_fields: NULL argument");
  if (l < 0 || l > 40 || m < -l || m > l) return fail(HERMES_ERR_INVALID, "multipole_fields: bad (l=%d, m=%d)", l, m);
  size_t need = 0;
  int rc = hermes_multipole_workspace_size(J, nb, &need);
  if (rc) return rc;
  if (!workspace || workspace_bytes < need) return fail(HERMES_ERR_WORKSPACE, "multipole_fields: workspace %zu < %zu", workspace_bytes, need);
  const int L = 1 << J;
  const long long N = 1LL << (3 * J);
  cudaStream_t s = hermes::as_stream(stream);
  hermes::Carver c(workspace, workspace_bytes);
  float* rho = c.take<float>(2 * kMaxBins);
  float* T = c.take<float>(table_floats(J, nb));
  float* Pf = c.take<float>(L + 1);
  float hrho[2 * kMaxBins];
  for (int b = 0; b < nb; ++b) {
    if (!(radii[b] >= 0.0)) return fail(HERMES_ERR_INVALID, "multipole_fields: radius %d must be >= 0", b);
    const double v = radii[b] / (double)L;
    hrho[2 * b] = (float)v;
    hrho[2 * b + 1] = (float)(v - (double)hrho[2 * b]);
  }
  HERMES_CUDA_TRY(cudaMemcpyAsync(rho, hrho, sizeof(float) * 2 * nb, cudaMemcpyHostToDevice, s));
  mp_power_to_f32<<<(L + 1 + 255) / 256, 256, 0, s>>>(phi_power, L + 1, Pf);
  HERMES_LAUNCH_CHECK("mp_power_to_f32");
  const int n2max = 3 * L * L;
  const int nsm = sm_count();
  mp_jl_table_kernel<<<nsm * 8, 256, 0, s>>>(T, n2max, rho, nb, l);
  HERMES_LAUNCH_CHECK("mp_jl_table_kernel");
  const YlmConst Y = make_ylm(l, m);
  const float inv_n = (float)(1.0 / (double)N);
  float2* out = static_cast<float2*>(fields_out);
  const int grid = nsm * 8;
  const float2* half = static_cast<const float2*>(half_spec);
  if (nb <= 4) mp_prepass_kernel<4><<<grid, 256, 0, s>>>(half, J, Pf, T, Y, nb, out, inv_n);
  else if (nb <= 8) mp_prepass_kernel<8><<<grid, 256, 0, s>>>(half, J, Pf, T, Y, nb, out, inv_n);
  else mp_prepass_kernel<16><<<grid, 256, 0, s>>>(half, J, Pf, T, Y, nb, out, inv_n);
  HERMES_LAUNCH_CHECK("mp_prepass_kernel");
  cufftHandle h;
  rc = hermes::get_plan_c2c_batch(J, nb, &h);
  if (rc) return rc;
  cufftResult r = cufftSetStream(h, s);
  if (r != CUFFT_SUCCESS) return fail(HERMES_ERR_CUFFT, "cufftSetStream failed: %d", (int)r);
  r = cufftExecC2C(h, reinterpret_cast<cufftComplex*>(out), reinterpret_cast<cufftComplex*>(out), CUFFT_INVERSE);
  if (r != CUFFT_SUCCESS) return fail(HERMES_ERR_CUFFT, "cufftExecC2C failed: %d", (int)r);
  return HERMES_OK;
}

extern "C" int hermes_multipole_contract(const float* eps1, const void* fields2, int nb2, const void* fields3,
                                         int nb3, int conj_sign, const double* gamma, int J, double* out,
                                         void* workspace, size_t workspace_bytes, void* stream) {
  if (!eps1 || !fields2 || !gamma || !out) return fail(HERMES_ERR_INVALID, "multipole_contract: NULL argument");
  if (nb2 < 1 || nb2 > kMaxBins) return fail(HERMES_ERR_INVALID, "multipole_contract: nb2=%d", nb2);
  const int conj_src = fields3 == nullptr;
  if (conj_src) {
    nb3 = nb2;
    if (conj_sign != 1 && conj_sign != -1) return fail(HERMES_ERR_INVALID, "multipole_contract: conj_sign must be +-1");
  }
  if (nb3 < 1 || nb3 > kMaxBins) return fail(HERMES_ERR_INVALID, "multipole_contract: nb3=%d", nb3);
  size_t need = 0;
  int rc = hermes_multipole_workspace_size(J, nb2 > nb3 ? nb2 : nb3, &need);
  if (rc) return rc;
  if (!workspace || workspace_bytes < need) return fail(HERMES_ERR_WORKSPACE, "multipole_contract: workspace %zu < %zu", workspace_bytes, need);
  const int L = 1 << J;
  const long long N = 1LL << (3 * J);
  cudaStream_t s = hermes::as_stream(stream);
  hermes::Carver c(workspace, workspace_bytes);
  c.take<float>(2 * kMaxBins);
  c.take<float>(table_floats(J, nb2 > nb3 ? nb2 : nb3));
  c.take<float>(L + 1);
  float2* G = c.take<float2>((size_t)(nb2 > nb3 ? nb2 : nb3) * N);
  double* partial = c.take<double>((size_t)4096 * kMaxBins * kMaxBins * 2);
  double* dout = c.take<double>((size_t)kMaxBins * kMaxBins * 2);
  const GammaC gm = make_gamma(gamma);
  const int ntiles = (L / GX) * (L / GY) * (L / GZ);
  const size_t smem = sizeof(float2) * (9 * kAyz + 3 * kAz) + sizeof(float) * kEps;
  static_assert(9 * kAyz >= kA3, "a3 halo must fit in the aliased y-pass buffer");
  HERMES_CUDA_TRY(cudaFuncSetAttribute(mp_gfield_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const float2* src = static_cast<const float2*>(conj_src ? fields2 : fields3);
  mp_gfield_kernel<<<ntiles, GThreads, smem, s>>>(eps1, src, conj_src, (float)conj_sign, nb3, J, gm, G);
  HERMES_LAUNCH_CHECK("mp_gfield_kernel");
  int nblk = sm_count() * 8;
  if (nblk > 4096) nblk = 4096;
  mp_gemm_kernel<<<nblk, kGemmThreads, 0, s>>>(static_cast<const float2*>(fields2), nb2, G, nb3, N, partial);
  HERMES_LAUNCH_CHECK("mp_gemm_kernel");
  mp_reduce_kernel<<<kMaxBins * kMaxBins * 2, 256, 0, s>>>(partial, nblk, kMaxBins * kMaxBins * 2, dout);
  HERMES_LAUNCH_CHECK("mp_reduce_kernel");
  std::vector<double> h((size_t)kMaxBins * kMaxBins * 2);
  HERMES_CUDA_TRY(cudaMemcpyAsync(h.data(), dout, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, s));
  HERMES_CUDA_TRY(cudaStreamSynchronize(s));
  const double scale = 4.0 * 3.141592653589793 / (double)N;
  for (int a = 0; a < nb2; ++a)
    for (int b = 0; b < nb3; ++b) {
      out[(a * nb3 + b) * 2] = h[(a * kMaxBins + b) * 2] * scale;
      out[(a * nb3 + b) * 2 + 1] = h[(a * kMaxBins + b) * 2 + 1] * scale;
    }
  return HERMES_OK;
}

extern "C" int hermes_multipole_contract_plain(const float* eps1, const void* a2, const void* a3,
                                               const double* gamma, int J, double* out, void* workspace,
                                               size_t workspace_bytes, void* stream) {
  if (!eps1 || !a2 || !a3 || !gamma || !out) return fail(HERMES_ERR_INVALID, "contract_plain: NULL argument");
  if (J < 3 || J > 10) return fail(HERMES_ERR_INVALID, "contract_plain: J=%d outside [3,10]", J);
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
