// Spectral window passes around cuFFT: `field @ window`, kernel
// materialisation, and multi-bin pair products by Parseval.
//
// Reference path (pyhermes/utils/convolution.py, io/window.py,
// theory/corr2pcf.py:366-372): materialise a float64 kernel array of
// L^2 (L/2+1) values per window (8 images x W(k) per mode), then
// irfftn(rfftn(eps) * K), then mean(conv * eps2) -- two FFTs and a kernel
// build per bin.  Here the kernel is evaluated on the fly in the pass that
// touches the spectrum, and the 2PCF products of every bin are one pass over
// the half spectra:  sum_x (f1 * K)(x) f2(x) / L^3 = sum_k F1 K conj(F2) / L^6.
#include <cufft.h>

#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "hermes_common.cuh"
#include "window_eval.cuh"
#include "pair_products.cuh"

namespace hermes {

// ---- cuFFT plan cache ----------------------------------------------------
enum PlanKind { kR2C = 0, kC2R = 1, kC2C = 2, kC2CLines = 3 };

static std::mutex g_plan_mu;
static std::map<std::tuple<int, int, int, int>, cufftHandle> g_plans;

int get_plan(int J, PlanKind kind, int batch, cufftHandle* out) {
  int dev = 0;
  HERMES_CUDA_TRY(cudaGetDevice(&dev));
  auto key = std::make_tuple(dev, J, (int)kind, batch);
  std::lock_guard<std::mutex> lk(g_plan_mu);
  auto it = g_plans.find(key);
  if (it != g_plans.end()) {
    *out = it->second;
    return HERMES_OK;
  }
  cufftHandle h;
  const int L = 1 << J;
  if (kind == kC2CLines) {  // 1-D transforms of the batch * L^2 contiguous z lines
    int n1[1] = {L};
    cufftResult r = cufftPlanMany(&h, 1, n1, nullptr, 1, L, nullptr, 1, L, CUFFT_C2C, batch * L * L);
    if (r != CUFFT_SUCCESS) return fail(HERMES_ERR_CUFFT, "cufftPlanMany(lines, J=%d, batch=%d) failed: %d", J, batch, (int)r);
    g_plans[key] = h;
    *out = h;
    return HERMES_OK;
  }
  int n[3] = {L, L, L};
  cufftType t = kind == kR2C ? CUFFT_R2C : (kind == kC2R ? CUFFT_C2R : CUFFT_C2C);
  long long dist_in = kind == kC2R ? (long long)L * L * (L / 2 + 1) : (long long)L * L * L;
  long long dist_out = kind == kR2C ? (long long)L * L * (L / 2 + 1) : (long long)L * L * L;
  cufftResult r = cufftPlanMany(&h, 3, n, nullptr, 1, (int)dist_in, nullptr, 1, (int)dist_out, t, batch);
  if (r != CUFFT_SUCCESS) return fail(HERMES_ERR_CUFFT, "cufftPlanMany(J=%d, kind=%d, batch=%d) failed: %d", J, (int)kind, batch, (int)r);
  g_plans[key] = h;
  *out = h;
  return HERMES_OK;
}

// Batched contiguous complex-to-complex plan (batch fields of L^3, distance L^3).
int get_plan_c2c_batch(int J, int batch, cufftHandle* out) { return get_plan(J, kC2C, batch, out); }

// 1-D complex-to-complex plan over the z lines (length L, contiguous) of
// `fields` fields of L^3.
int get_plan_c2c_lines(int J, int fields, cufftHandle* out) { return get_plan(J, kC2CLines, fields, out); }

#define HERMES_CUFFT_TRY(expr)                                                   \
  do {                                                                           \
    cufftResult _r = (expr);                                                     \
    if (_r != CUFFT_SUCCESS) return hermes::fail(HERMES_ERR_CUFFT, "%s failed: %d", #expr, (int)_r); \
  } while (0)

// ---- host-side window preparation ---------------------------------------
static void split_df(double v, float& hi, float& lo) {
  hi = (float)v;
  lo = (float)(v - (double)hi);
}

int prepare_window(const hermes_window_t& in, int L, WinDev* out) {
  WinDev w;
  memset(&w, 0, sizeof(w));
  w.type = in.type;
  w.mode = in.kernel_mode;
  w.zero_k0 = in.zero_mode_zero ? 1 : 0;
  w.los_axis = -1;
  w.scale = (float)(in.scale == 0.0 ? 1.0 : in.scale);
  if (in.type < 0 || in.type > HERMES_WIN_INVERSE_LAPLACIAN)
    return fail(HERMES_ERR_INVALID, "window: unknown type %d", in.type);
  if (in.kernel_mode < 0 || in.kernel_mode > HERMES_KMODE_COMPLEX_RFFT)
    return fail(HERMES_ERR_INVALID, "window: unknown kernel_mode %d", in.kernel_mode);
  const double invL = 1.0 / (double)L;
  for (int i = 0; i < 4; ++i) {
    w.len[i] = (float)in.len[i];
    split_df(in.len[i] * invL, w.rho_hi[i], w.rho_lo[i]);
  }
  const double e = 2.718281828459045;
  const double pi = 3.141592653589793;
  switch (in.type) {
    case HERMES_WIN_THICK_SHELL: {
      double R = in.len[0], dR = in.len[1];
      if (!(R >= 0.0) || !(dR > 0.0)) return fail(HERMES_ERR_INVALID, "thick_shell requires R >= 0 and delta_R > 0");
      double rin = R - 0.5 * dR;
      if (rin < 0.0) rin = 0.0;
      double rout = R + 0.5 * dR;
      double den = rout * rout * rout - rin * rin * rin;
      if (den == 0.0) {
        w.c0 = 0.f;
        w.c1 = 0.f;
      } else {
        w.c0 = (float)(rout * rout * rout / den);
        w.c1 = (float)(rin * rin * rin / den);
      }
      split_df(rout * invL, w.rho_hi[0], w.rho_lo[0]);
      split_df(rin * invL, w.rho_hi[1], w.rho_lo[1]);
      break;
    }
    case HERMES_WIN_GAUSSIAN_SHELL: {
      double rs = in.len[0], rm = in.len[1];
      double den = rs * rs + rm * rm;
      if (den == 0.0) {
        w.c0 = -1.f;
        w.c1 = -1.f;
      } else {
        w.c0 = (float)(rm * rm / den);
        w.c1 = (float)(rs * rs / den);
      }
      break;
    }
    case HERMES_WIN_CW: {
      double ccw = 2.0 * sqrt(2.0) / (sqrt(1.0 + 5.0 * e) * pow(pi, 0.25));
      w.c0 = (float)(sqrt(2.0 * pi) * ccw * pow(in.len[0], 0.5));
      break;
    }
    case HERMES_WIN_CWS: {
      double ccws = 2.0 * sqrt(2.0) / (sqrt(9.0 + 55.0 * e) * pow(pi, 0.75));
      w.c0 = (float)(pow(2.0 * pi, 1.5) * ccws * pow(in.len[0], 1.5));
      break;
    }
    case HERMES_WIN_GDW:
      w.c0 = (float)(pow(2.0, 2.5) * pow(pi, 0.75) / sqrt(15.0) * pow(in.len[0], 1.5));
      break;
    case HERMES_WIN_LAPLACIAN:
    case HERMES_WIN_INVERSE_LAPLACIAN:
      w.c0 = (float)(invL * invL);
      break;
    default:
      break;
  }
  if (in.type >= HERMES_WIN_RING && in.type <= HERMES_WIN_CYLINDER ||
      in.type == HERMES_WIN_DIRECTIONAL_DERIVATIVE) {
    double nx = in.los[0], ny = in.los[1], nz = in.los[2];
    double nrm = sqrt(nx * nx + ny * ny + nz * nz);
    if (!(nrm > 0.0)) return fail(HERMES_ERR_INVALID, "window: line of sight must be non-zero");
    nx /= nrm;
    ny /= nrm;
    nz /= nrm;
    w.los[0] = (float)nx;
    w.los[1] = (float)ny;
    w.los[2] = (float)nz;
    const double v[3] = {nx, ny, nz};
    for (int a = 0; a < 3; ++a) {
      if (fabs(fabs(v[a]) - 1.0) == 0.0 && v[(a + 1) % 3] == 0.0 && v[(a + 2) % 3] == 0.0) w.los_axis = a;
    }
    if (in.type == HERMES_WIN_DIRECTIONAL_DERIVATIVE) w.c0 = (float)invL;
  }
  *out = w;
  return HERMES_OK;
}

// ---- kernels -------------------------------------------------------------
__global__ void phi_power_to_f32(const double* __restrict__ p, int n, float* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)p[i];
}

// spec[k] *= K(k) * factor on the half spectrum [L][L][L/2+1].  The gaussian
// exp(-q^2/2) factors over the axes, so its image sum is G(x) G(y) G(z) with
// G(i) = sum over the axis images u of P(|u|) exp(-(2 pi u R / L)^2 / 2),
// tabulated per block in shared memory (the other windows are evaluated per
// mode by kernel_value).
__global__ void spec_apply_window_kernel(float2* __restrict__ spec, WinDev w, int L,
                                         const double* __restrict__ pd, int np, int bw, float factor) {
  extern __shared__ float P[];
  float* G = P + np;  // [L], gaussian only
  for (int i = threadIdx.x; i < np; i += blockDim.x) P[i] = (float)pd[i];
  __syncthreads();
  const bool sep = w.type == HERMES_WIN_GAUSSIAN;
  if (sep) {
    for (int i = threadIdx.x; i < L; i += blockDim.x) {
      float g = 0.f;
      for (int kk = 0; kk < bw; ++kk) {
        const int u1 = kk * L + i, u2 = kk * L + (L - i);
        const float q1 = kTwoPi * ((float)u1 * w.rho_hi[0] + (float)u1 * w.rho_lo[0]);
        const float q2 = kTwoPi * ((float)u2 * w.rho_hi[0] + (float)u2 * w.rho_lo[0]);
        g = fmaf(P[u1], expf(-0.5f * q1 * q1), g);
        g = fmaf(P[u2], expf(-0.5f * q2 * q2), g);
      }
      G[i] = g;
    }
    __syncthreads();
  }
  const int H = L / 2 + 1;
  const long long total = (long long)L * L * H;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < total; m += stride) {
    const int z = (int)(m % H);
    const long long r = m / H;
    const int y = (int)(r % L), x = (int)(r / L);
    float2 K;
    if (sep) {
      K = make_float2(G[x] * G[y] * G[z] * w.scale, 0.f);
      if (w.zero_k0 && m == 0) K.x = 0.f;
    } else {
      K = kernel_value(w, x, y, z, L, P, bw);
    }
    const float2 s = spec[m];
    spec[m] = make_float2((s.x * K.x - s.y * K.y) * factor, (s.x * K.y + s.y * K.x) * factor);
  }
}

__global__ void materialize_kernel(WinDev w, int L, const double* __restrict__ pd, int np, int bw,
                                   float* __restrict__ kr, float2* __restrict__ kc) {
  extern __shared__ float P[];
  for (int i = threadIdx.x; i < np; i += blockDim.x) P[i] = (float)pd[i];
  __syncthreads();
  const int H = L / 2 + 1;
  const long long total = (long long)L * L * H;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < total; m += stride) {
    const int z = (int)(m % H);
    const long long r = m / H;
    const int y = (int)(r % L), x = (int)(r / L);
    const float2 K = kernel_value(w, x, y, z, L, P, bw);
    if (kr) kr[m] = K.x;
    if (kc) kc[m] = K;
  }
}

__global__ void spec_multiply_kernel(float2* __restrict__ spec, const float* __restrict__ kr,
                                     const float2* __restrict__ kc, long long total, float factor) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < total; m += stride) {
    const float2 s = spec[m];
    float2 K = kc ? kc[m] : make_float2(kr[m], 0.f);
    spec[m] = make_float2((s.x * K.x - s.y * K.y) * factor, (s.x * K.y + s.y * K.x) * factor);
  }
}

__global__ void reduce_partials_kernel(const double* __restrict__ partial, int nblocks, int nout,
                                       double scale, double* __restrict__ out) {
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

int grid_for(long long total, int threads) {
  int dev = 0, nsm = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  long long want = (total + threads - 1) / threads;
  long long cap = (long long)nsm * 16;
  return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

int check_power(int J, int bw) {
  if (J < 2 || J > 10) return fail(HERMES_ERR_INVALID, "J=%d outside [2,10]", J);
  if (bw < 1) return fail(HERMES_ERR_INVALID, "bandwidth must be >= 1");
  long long n = (long long)(1 << J) * bw;
  if (3 * n * n >= (1LL << 24)) return fail(HERMES_ERR_UNSUPPORTED, "bandwidth*L too large for exact float frequencies");
  return HERMES_OK;
}

}  // namespace hermes

using namespace hermes;

extern "C" int hermes_fft_r2c(const float* field, void* spec, int J, void* stream) {
  if (J < 2 || J > 10) return fail(HERMES_ERR_INVALID, "fft: J=%d outside [2,10]", J);
  cufftHandle h;
  int rc = get_plan(J, kR2C, 1, &h);
  if (rc) return rc;
  HERMES_CUFFT_TRY(cufftSetStream(h, as_stream(stream)));
  HERMES_CUFFT_TRY(cufftExecR2C(h, const_cast<cufftReal*>(field), reinterpret_cast<cufftComplex*>(spec)));
  return HERMES_OK;
}

extern "C" int hermes_fft_c2r(void* spec, float* field, int J, void* stream) {
  if (J < 2 || J > 10) return fail(HERMES_ERR_INVALID, "fft: J=%d outside [2,10]", J);
  cufftHandle h;
  int rc = get_plan(J, kC2R, 1, &h);
  if (rc) return rc;
  HERMES_CUFFT_TRY(cufftSetStream(h, as_stream(stream)));
  HERMES_CUFFT_TRY(cufftExecC2R(h, reinterpret_cast<cufftComplex*>(spec), field));
  return HERMES_OK;
}

extern "C" int hermes_window_workspace_size(int J, size_t* bytes) {
  if (!bytes) return fail(HERMES_ERR_INVALID, "bytes is NULL");
  if (J < 2 || J > 10) return fail(HERMES_ERR_INVALID, "J=%d outside [2,10]", J);
  const size_t L = (size_t)1 << J;
  *bytes = L * L * (L / 2 + 1) * sizeof(float2);
  return HERMES_OK;
}

extern "C" int hermes_window_apply(const float* eps, float* out, int J, const hermes_window_t* win,
                                   const double* phi_power, int bandwidth, void* workspace,
                                   size_t workspace_bytes, void* stream) {
  if (!eps || !out || !win || !phi_power) return fail(HERMES_ERR_INVALID, "window_apply: NULL argument");
  int rc = check_power(J, bandwidth);
  if (rc) return rc;
  size_t need = 0;
  hermes_window_workspace_size(J, &need);
  if (!workspace || workspace_bytes < need)
    return fail(HERMES_ERR_WORKSPACE, "window_apply: workspace %zu < %zu", workspace_bytes, need);
  const int L = 1 << J;
  WinDev w;
  rc = prepare_window(*win, L, &w);
  if (rc) return rc;
  float2* spec = static_cast<float2*>(workspace);
  rc = hermes_fft_r2c(eps, spec, J, stream);
  if (rc) return rc;
  const int np = L * bandwidth + 1;
  const long long total = (long long)L * L * (L / 2 + 1);
  const float factor = (float)(1.0 / ((double)L * L * L));
  spec_apply_window_kernel<<<grid_for(total, 256), 256, (np + L) * sizeof(float), as_stream(stream)>>>(
      spec, w, L, phi_power, np, bandwidth, factor);
  HERMES_LAUNCH_CHECK("spec_apply_window_kernel");
  return hermes_fft_c2r(spec, out, J, stream);
}

extern "C" int hermes_window_materialize(const hermes_window_t* win, const double* phi_power, int bandwidth,
                                         int J, float* k_real, void* k_cplx, void* stream) {
  if (!win || !phi_power) return fail(HERMES_ERR_INVALID, "materialize: NULL argument");
  if ((k_real == nullptr) == (k_cplx == nullptr))
    return fail(HERMES_ERR_INVALID, "materialize: give exactly one of k_real / k_cplx");
  int rc = check_power(J, bandwidth);
  if (rc) return rc;
  const int L = 1 << J;
  WinDev w;
  rc = prepare_window(*win, L, &w);
  if (rc) return rc;
  const int np = L * bandwidth + 1;
  const long long total = (long long)L * L * (L / 2 + 1);
  materialize_kernel<<<grid_for(total, 256), 256, np * sizeof(float), as_stream(stream)>>>(
      w, L, phi_power, np, bandwidth, k_real, static_cast<float2*>(k_cplx));
  HERMES_LAUNCH_CHECK("materialize_kernel");
  return HERMES_OK;
}

extern "C" int hermes_spectrum_multiply(void* spec, const float* k_real, const void* k_cplx, int J,
                                        double factor, void* stream) {
  if (!spec || ((k_real == nullptr) == (k_cplx == nullptr)))
    return fail(HERMES_ERR_INVALID, "spectrum_multiply: give spec and exactly one kernel");
  if (J < 2 || J > 10) return fail(HERMES_ERR_INVALID, "J=%d outside [2,10]", J);
  const long long L = 1LL << J;
  const long long total = L * L * (L / 2 + 1);
  spec_multiply_kernel<<<grid_for(total, 256), 256, 0, as_stream(stream)>>>(
      static_cast<float2*>(spec), k_real, static_cast<const float2*>(k_cplx), total, (float)factor);
  HERMES_LAUNCH_CHECK("spec_multiply_kernel");
  return HERMES_OK;
}

// Cylindrical bins (ring / disk / cylshell / cylinder) with the line of sight
// on z: the kernel is K(x, y, z) = scale * A(x, y) * B(z) with
//   A = sum over the (x, y) images of P P f(k_perp R),  B = sum over the z
//   images of P g(k_par H)   (cyl_image_sum).
// So sum_k T(k) K_b(k) = sum_(x,y) A_b(x, y) * [sum_z T(x, y, z) B_b(z)]: per
// column a [columns x z] by [z x bins] product, then a weighted sum.
//
// A depends on (x, y) only through the image set {x, L-x} x {y, L-y} and
// p^2 + q^2, so A(x, y) = A(min(x, L-x), min(y, L-y)) = A(y, x).
// cyl_perp_table_kernel evaluates it once per (x, y) in the triangle
// 0 <= y <= x <= L/2 and bin (1/8 of the plane), into a table that the
// column kernel reads.
//
// Column kernel: a block takes kCylBins bins (two per lane); B is tabulated
// for them in shared memory as [z][bin].  A warp takes CW consecutive
// columns (their modes are contiguous), stages the weighted products
// T = w_z Re(u conj v) in chunks of kCylZ z-planes as [z][pair][column], and
// per z reads CW columns' T (broadcast, 128-bit) and its two bins' B (64-bit)
// for 2 x CW FMAs per pair: a register tile instead of one shared-memory load
// per FMA.  The spectra are read once per bin group; the groups run side by
// side, so the second and later reads mostly hit L2.
constexpr int kCylBins = 64;
constexpr int kCylZ = 64;

template <int NP>
struct CylCols {
  static constexpr int value = NP == 1 ? 8 : 4;  // columns per warp task
};

__global__ void cyl_perp_table_kernel(const WinDev* __restrict__ wins, int n_bins, int nbp,
                                      const double* __restrict__ pd, int np, int L, int bw,
                                      float* __restrict__ atab) {
  extern __shared__ float Pt[];
  for (int i = threadIdx.x; i < np; i += blockDim.x) Pt[i] = (float)pd[i];
  __syncthreads();
  const int H = L / 2 + 1;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)H * H * nbp) return;
  const int b = (int)(i % nbp);
  const long long cell = i / nbp;
  const int x = (int)(cell / H), y = (int)(cell - (long long)x * H);
  if (y > x) return;
  float av = 0.f;
  if (b < n_bins) {
    const WinDev& w = wins[b];
    const int sgn = w.mode == HERMES_KMODE_OCTANT ? 1 : -1;
    const int n_img = 4 * bw * bw;
    for (int t = 0; t < n_img; ++t) {
      const int pair = t >> 2, sp = t & 1, sq = (t >> 1) & 1;
      const int ii = pair / bw, jj = pair - ii * bw;
      const int pu = sp ? ii * L + (L - x) : ii * L + x;
      const int qu = sq ? jj * L + (L - y) : jj * L + y;
      av = fmaf(Pt[pu] * Pt[qu], cyl_perp(w, sp ? sgn * pu : pu, sq ? sgn * qu : qu), av);
    }
  }
  atab[((size_t)x * H + y) * nbp + b] = av;
  atab[((size_t)y * H + x) * nbp + b] = av;
}

template <int NP>
__global__ void __launch_bounds__(kPPThreads, 2)
pair_products_cylz_kernel(PPArgs a, const WinDev* __restrict__ wins, const double* __restrict__ pd,
                          const float* __restrict__ atab, int nbp, double* __restrict__ partial,
                          double* __restrict__ k0) {
  constexpr int kWarps = kPPThreads / 32;
  constexpr int CW = CylCols<NP>::value;
  constexpr int TZ = CW * NP;  // floats per z-plane of a warp's staged chunk
  extern __shared__ __align__(16) unsigned char cyl_sm[];
  const int L = a.L, H = L / 2 + 1;
  float* P = reinterpret_cast<float*>(cyl_sm);
  float* B = P + ((a.np + 3) & ~3);                                  // [H][kCylBins]
  float* T = B + (size_t)H * kCylBins;                               // [kWarps][kCylZ][NP][CW]
  double* red = reinterpret_cast<double*>(T + (size_t)kWarps * kCylZ * TZ);  // [kWarps][kCylBins][NP]
  for (int i = threadIdx.x; i < a.np; i += blockDim.x) P[i] = (float)pd[i];
  const int b0 = blockIdx.y * kCylBins;
  const int nb = min(kCylBins, a.n_bins - b0);
  __syncthreads();
  if (blockIdx.x == 0 && threadIdx.x < nb) k0[b0 + threadIdx.x] = (double)kernel_value(wins[b0 + threadIdx.x], 0, 0, 0, L, P, a.bw).x;
  const int sgn = wins[b0].mode == HERMES_KMODE_OCTANT ? 1 : -1;
  for (int i = threadIdx.x; i < kCylBins * H; i += blockDim.x) {
    const int z = i / kCylBins, b = i - z * kCylBins;
    float v = 0.f;
    if (b < nb) {
      const WinDev& w = wins[b0 + b];
      for (int kk = 0; kk < a.bw; ++kk) {
        const int cp = kk * L + z, cn = kk * L + (L - z);
        v = fmaf(P[cp], cyl_par(w, cp), v);
        v = fmaf(P[cn], cyl_par(w, sgn * cn), v);
      }
      v *= w.scale;
    }
    B[i] = v;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float* Tw = T + (size_t)wid * kCylZ * TZ;
  double acc[2][NP];
  int zk[2];
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    const int b = 2 * lane + j;
    zk[j] = b < nb ? wins[b0 + b].zero_k0 : 0;
#pragma unroll
    for (int p = 0; p < NP; ++p) acc[j][p] = 0.0;
  }
  const long long ncol = (long long)L * L;  // a multiple of CW
  for (long long col0 = ((long long)blockIdx.x * kWarps + wid) * CW; col0 < ncol;
       col0 += (long long)gridDim.x * kWarps * CW) {
    // (bin 2 lane, bin 2 lane + 1) sums of each column, updated by paired FMAs
    float2 fac[CW][NP];
#pragma unroll
    for (int c = 0; c < CW; ++c)
#pragma unroll
      for (int p = 0; p < NP; ++p) fac[c][p] = make_float2(0.f, 0.f);
    float t00[NP];
    for (int zc = 0; zc < H; zc += kCylZ) {
      const int zn = min(kCylZ, H - zc);
      __syncwarp();
      // lane i stages z-plane zc + i of all CW columns: per column the lanes
      // read consecutive modes (coalesced), the CW loads are in flight
      // together, and the plane's products are written as 128-bit rows
#pragma unroll
      for (int ii = 0; ii < kCylZ / 32; ++ii) {
        const int i = lane + 32 * ii;
        if (i < zn) {
          const int z = zc + i;
          const float wgt = (z == 0 || z == L / 2) ? 1.f : 2.f;
          float tv[NP][CW];
#pragma unroll
          for (int c = 0; c < CW; ++c) {
            const long long m = (col0 + c) * H + z;
#pragma unroll
            for (int p = 0; p < NP; ++p) {
              const float2 u = a.si[p][m], v = a.sj[p][m];
              tv[p][c] = (a.exclude_k0 && m == 0) ? 0.f : wgt * (u.x * v.x + u.y * v.y);
            }
          }
#pragma unroll
          for (int p = 0; p < NP; ++p)
#pragma unroll
            for (int c4 = 0; c4 < CW; c4 += 4)
              *reinterpret_cast<float4*>(Tw + (i * NP + p) * CW + c4) =
                  make_float4(tv[p][c4], tv[p][c4 + 1], tv[p][c4 + 2], tv[p][c4 + 3]);
        }
      }
      __syncwarp();
      if (zc == 0) {
#pragma unroll
        for (int p = 0; p < NP; ++p) t00[p] = Tw[p * CW];  // column col0 at z = 0
      }
      const float* Bz = B + (size_t)zc * kCylBins + 2 * lane;
#pragma unroll 4
      for (int z = 0; z < zn; ++z) {
        const float2 bz = *reinterpret_cast<const float2*>(Bz + (size_t)z * kCylBins);
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          float tv[CW];
#pragma unroll
          for (int c4 = 0; c4 < CW; c4 += 4) {
            const float4 t4 = *reinterpret_cast<const float4*>(Tw + (z * NP + p) * CW + c4);
            tv[c4] = t4.x;
            tv[c4 + 1] = t4.y;
            tv[c4 + 2] = t4.z;
            tv[c4 + 3] = t4.w;
          }
#pragma unroll
          for (int c = 0; c < CW; ++c) fac[c][p] = __ffma2_rn(make_float2(tv[c], tv[c]), bz, fac[c][p]);
        }
      }
    }
    // the task's CW columns are summed in float32 and added to the float64
    // total once per task (float64 throughput is low on this part)
    float task[2][NP];
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int p = 0; p < NP; ++p) task[j][p] = 0.f;
#pragma unroll
    for (int c = 0; c < CW; ++c) {
      const long long col = col0 + c;
      const int x = (int)(col / L), y = (int)(col - (long long)x * L);
      const int xq = min(x, L - x), yq = min(y, L - y);
      const float2 av = *reinterpret_cast<const float2*>(atab + ((size_t)xq * H + yq) * nbp + b0 + 2 * lane);
      const float aj[2] = {av.x, av.y};
#pragma unroll
      for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          float f = j == 0 ? fac[c][p].x : fac[c][p].y;
          if (col == 0 && zk[j]) f -= t00[p] * B[2 * lane + j];  // K(0,0,0) forced to 0
          task[j][p] = fmaf(aj[j], f, task[j][p]);
        }
    }
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int p = 0; p < NP; ++p) acc[j][p] += (double)task[j][p];
  }
  // block reduction over warps (fixed order -> deterministic)
#pragma unroll
  for (int j = 0; j < 2; ++j)
#pragma unroll
    for (int p = 0; p < NP; ++p) red[((size_t)wid * kCylBins + 2 * lane + j) * NP + p] = acc[j][p];
  __syncthreads();
  for (int i = threadIdx.x; i < nb * NP; i += blockDim.x) {
    double v = 0.0;
    for (int w2 = 0; w2 < kWarps; ++w2) v += red[(size_t)w2 * kCylBins * NP + i];
    const int b = i / NP, p = i - b * NP;
    partial[((long long)blockIdx.x * a.n_bins + b0 + b) * a.n_pairs + p] = v;
  }
}

static size_t cylz_smem(int np, int L, int n_pairs) {
  const int H = L / 2 + 1;
  const int cw = n_pairs == 1 ? 8 : 4;
  return sizeof(float) * ((((size_t)np + 3) & ~(size_t)3) + (size_t)H * kCylBins +
                          (size_t)(kPPThreads / 32) * kCylZ * cw * n_pairs) +
         sizeof(double) * (size_t)(kPPThreads / 32) * kCylBins * n_pairs;
}

// Bins padded to whole groups of kCylBins (the A table's row stride).
static int cylz_nbp(int n_bins) { return (n_bins + kCylBins - 1) / kCylBins * kCylBins; }

// True when every bin is a cylindrical window with the line of sight on z
// and all bins use the same image mode (the column kernel's precondition).
static bool all_cyl_z(const std::vector<WinDev>& hw) {
  for (const WinDev& w : hw) {
    const bool cyl = w.type == HERMES_WIN_RING || w.type == HERMES_WIN_DISK || w.type == HERMES_WIN_CYLSHELL ||
                     w.type == HERMES_WIN_CYLINDER;
    if (!cyl || w.los_axis != 2 || w.mode != hw[0].mode) return false;
  }
  return !hw.empty();
}

static long long pp_mode_blocks(int J) {
  const long long L = 1LL << J;
  const long long total = L * L * (L / 2 + 1);
  const long long per = (long long)kPPThreads * kPPModesPerThread;
  return (total + per - 1) / per;
}

extern "C" int hermes_pair_products_workspace_size(int J, int n_bins, int n_pairs, size_t* bytes) {
  if (!bytes) return fail(HERMES_ERR_INVALID, "bytes is NULL");
  if (J < 2 || J > 10) return fail(HERMES_ERR_INVALID, "J=%d outside [2,10]", J);
  if (n_bins < 1 || n_pairs < 1 || n_pairs > kMaxPairs)
    return fail(HERMES_ERR_INVALID, "pair_products: n_bins >= 1 and 1 <= n_pairs <= %d", kMaxPairs);
  const size_t H = ((size_t)1 << J) / 2 + 1;
  Carver c(nullptr, 0);
  c.take<WinDev>(n_bins);
  c.take<double>((size_t)pp_mode_blocks(J) * n_bins * n_pairs);
  c.take<double>((size_t)n_bins * n_pairs);
  c.take<double>((size_t)n_bins);
  c.take<float>(H * H * (size_t)cylz_nbp(n_bins));  // A table of cylindrical bins
  *bytes = c.used;
  return HERMES_OK;
}

extern "C" int hermes_pair_products(const void* const* spectra, int n_spec, const int32_t* pairs, int n_pairs,
                                    const hermes_window_t* bins, int n_bins, const double* phi_power,
                                    int bandwidth, int J, int exclude_k0, double* out, double* k0_out,
                                    void* workspace, size_t workspace_bytes, void* stream) {
  if (!spectra || !pairs || !bins || !phi_power || !out) return fail(HERMES_ERR_INVALID, "pair_products: NULL argument");
  size_t need = 0;
  int rc = hermes_pair_products_workspace_size(J, n_bins, n_pairs, &need);
  if (rc) return rc;
  rc = check_power(J, bandwidth);
  if (rc) return rc;
  if (!workspace || workspace_bytes < need)
    return fail(HERMES_ERR_WORKSPACE, "pair_products: workspace %zu < %zu", workspace_bytes, need);
  const int L = 1 << J;
  PPArgs a;
  memset(&a, 0, sizeof(a));
  if (n_spec < 1 || n_spec > 2 * kMaxPairs) return fail(HERMES_ERR_INVALID, "pair_products: n_spec=%d", n_spec);
  for (int i = 0; i < n_spec; ++i)
    if (!spectra[i]) return fail(HERMES_ERR_INVALID, "pair_products: spectra[%d] is NULL", i);
  for (int p = 0; p < n_pairs; ++p) {
    if (pairs[2 * p] < 0 || pairs[2 * p] >= n_spec || pairs[2 * p + 1] < 0 || pairs[2 * p + 1] >= n_spec)
      return fail(HERMES_ERR_INVALID, "pair_products: pair %d indexes outside [0,%d)", p, n_spec);
    a.si[p] = static_cast<const float2*>(spectra[pairs[2 * p]]);
    a.sj[p] = static_cast<const float2*>(spectra[pairs[2 * p + 1]]);
  }
  a.n_pairs = n_pairs;
  a.L = L;
  a.bw = bandwidth;
  a.np = L * bandwidth + 1;
  a.n_bins = n_bins;
  a.exclude_k0 = exclude_k0 ? 1 : 0;
  std::vector<WinDev> hw(n_bins);
  for (int b = 0; b < n_bins; ++b) {
    rc = prepare_window(bins[b], L, &hw[b]);
    if (rc) return rc;
  }
  Carver c(workspace, workspace_bytes);
  WinDev* dwin = c.take<WinDev>(n_bins);
  const long long nblk = pp_mode_blocks(J);
  double* partial = c.take<double>((size_t)nblk * n_bins * n_pairs);
  double* dout = c.take<double>((size_t)n_bins * n_pairs);
  double* dk0 = c.take<double>((size_t)n_bins);
  const int H = L / 2 + 1;
  const int nbp = cylz_nbp(n_bins);
  float* atab = c.take<float>((size_t)H * H * nbp);
  cudaStream_t s = as_stream(stream);
  HERMES_CUDA_TRY(cudaMemcpyAsync(dwin, hw.data(), sizeof(WinDev) * n_bins, cudaMemcpyHostToDevice, s));
  if (all_cyl_z(hw) && n_pairs <= 4 && cylz_smem(a.np, L, n_pairs) <= 200 * 1024) {
    const long long tab_threads = (long long)H * H * nbp;
    cyl_perp_table_kernel<<<(unsigned)((tab_threads + 255) / 256), 256, a.np * sizeof(float), s>>>(
        dwin, n_bins, nbp, phi_power, a.np, L, bandwidth, atab);
    HERMES_LAUNCH_CHECK("cyl_perp_table_kernel");
    const size_t csm = cylz_smem(a.np, L, n_pairs);
    const void* fn = n_pairs == 1 ? (const void*)pair_products_cylz_kernel<1>
                   : n_pairs == 2 ? (const void*)pair_products_cylz_kernel<2>
                   : n_pairs == 3 ? (const void*)pair_products_cylz_kernel<3>
                                  : (const void*)pair_products_cylz_kernel<4>;
    HERMES_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)csm));
    // every block resident at once over all bin groups (whole waves), so
    // each block's table of B(z) is reused over many columns and the groups
    // read the same columns at about the same time
    int dev = 0, nsm = 148, per_sm = 1;
    HERMES_CUDA_TRY(cudaGetDevice(&dev));
    HERMES_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    HERMES_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kPPThreads, csm));
    if (per_sm < 1) per_sm = 1;
    const int groups = nbp / kCylBins;
    long long cblk = (long long)per_sm * nsm / groups;
    const long long max_tasks = (long long)L * L / ((kPPThreads / 32) * (n_pairs == 1 ? 8 : 4));
    if (cblk > max_tasks) cblk = max_tasks;
    if (cblk > nblk) cblk = nblk;  // partial sums sized for nblk blocks
    if (cblk < 1) cblk = 1;
    dim3 cgrid((unsigned)cblk, (unsigned)groups);
    switch (n_pairs) {
      case 1: pair_products_cylz_kernel<1><<<cgrid, kPPThreads, csm, s>>>(a, dwin, phi_power, atab, nbp, partial, dk0); break;
      case 2: pair_products_cylz_kernel<2><<<cgrid, kPPThreads, csm, s>>>(a, dwin, phi_power, atab, nbp, partial, dk0); break;
      case 3: pair_products_cylz_kernel<3><<<cgrid, kPPThreads, csm, s>>>(a, dwin, phi_power, atab, nbp, partial, dk0); break;
      default: pair_products_cylz_kernel<4><<<cgrid, kPPThreads, csm, s>>>(a, dwin, phi_power, atab, nbp, partial, dk0); break;
    }
    HERMES_LAUNCH_CHECK("pair_products_cylz_kernel");
    const double cscale = 1.0 / ((double)L * L * L * (double)L * L * L);
    reduce_partials_kernel<<<n_bins * n_pairs, 256, 0, s>>>(partial, (int)cblk, n_bins * n_pairs, cscale, dout);
    HERMES_LAUNCH_CHECK("reduce_partials_kernel");
    HERMES_CUDA_TRY(cudaMemcpyAsync(out, dout, sizeof(double) * n_bins * n_pairs, cudaMemcpyDeviceToHost, s));
    if (k0_out) HERMES_CUDA_TRY(cudaMemcpyAsync(k0_out, dk0, sizeof(double) * n_bins, cudaMemcpyDeviceToHost, s));
    HERMES_CUDA_TRY(cudaStreamSynchronize(s));
    return HERMES_OK;
  }
  dim3 grid((unsigned)nblk, (unsigned)((n_bins + kBinsPerGroup - 1) / kBinsPerGroup));
  const size_t sm = a.np * sizeof(float);
  cudaError_t le = cudaSuccess;
  switch (n_pairs) {
    case 1: le = launch_pair_products_1(grid, sm, s, a, dwin, phi_power, partial, dk0); break;
    case 2: le = launch_pair_products_2(grid, sm, s, a, dwin, phi_power, partial, dk0); break;
    case 3: le = launch_pair_products_3(grid, sm, s, a, dwin, phi_power, partial, dk0); break;
    case 4: le = launch_pair_products_4(grid, sm, s, a, dwin, phi_power, partial, dk0); break;
    default: return fail(HERMES_ERR_UNSUPPORTED, "pair_products: n_pairs=%d > 4", n_pairs);
  }
  if (le != cudaSuccess) return cuda_fail(le, "pair_products_kernel launch");
  const double scale = 1.0 / ((double)L * L * L * (double)L * L * L);
  reduce_partials_kernel<<<n_bins * n_pairs, 256, 0, s>>>(partial, (int)nblk, n_bins * n_pairs, scale, dout);
  HERMES_LAUNCH_CHECK("reduce_partials_kernel");
  HERMES_CUDA_TRY(cudaMemcpyAsync(out, dout, sizeof(double) * n_bins * n_pairs, cudaMemcpyDeviceToHost, s));
  if (k0_out) HERMES_CUDA_TRY(cudaMemcpyAsync(k0_out, dk0, sizeof(double) * n_bins, cudaMemcpyDeviceToHost, s));
  HERMES_CUDA_TRY(cudaStreamSynchronize(s));
  return HERMES_OK;
}
