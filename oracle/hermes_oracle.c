/*
 * hermes_oracle.c — float64 CPU restatement of the PyHermes field-pipeline
 * kernels.  TEST INFRASTRUCTURE ONLY: used by tests/, the smoke check and the
 * CPU-baseline legs of bench.py as the checker; never by the product path.
 *
 * Each function names the reference lines (SYSUSPA-Projects/PyHermes) whose
 * arithmetic it restates.  Loop order and operation order follow the
 * reference so float64 results agree to rounding (bit-exact for the integer
 * cell / fraction indices).  Build with -ffp-contract=off: the reference
 * (numba/LLVM, NumPy) does not fuse multiply-add.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

static inline int64_t pmod(int64_t a, int64_t L) {
  int64_t r = a % L;
  return r < 0 ? r + L : r;
}

/* utils/wavelet_grid.py:17-55 (_project_scaling_grid_impl, full grid,
 * base_x = x_padding = 0).  Sequential over particles like the reference;
 * negative indices wrap like NumPy/numba.  grid: L^3 float64 (zeroed here). */
int oracle_deposit(const double* pos, const double* w, int64_t n, const double* phi,
                   int n_phi, int res, int J, double box, double* grid) {
  const int64_t L = (int64_t)1 << J;
  const int S = n_phi / res;
  const double scale = (double)L / box;
  memset(grid, 0, sizeof(double) * (size_t)(L * L * L));
  for (int64_t p = 0; p < n; ++p) {
    int64_t c[3];
    int f[3];
    for (int a = 0; a < 3; ++a) {
      double s = pos[3 * p + a] * scale;
      double fl = floor(s);
      c[a] = (int64_t)(int32_t)fl;
      f[a] = (int32_t)((s - (double)(int32_t)fl) * (double)res);
    }
    const double wt = w[p];
    for (int sx = 0; sx < S; ++sx) {
      const double phx = wt * phi[f[0] + res * sx];
      const int64_t gx = pmod(c[0] - sx, L);
      for (int sy = 0; sy < S; ++sy) {
        const double phxy = phx * phi[f[1] + res * sy];
        const int64_t gy = pmod(c[1] - sy, L);
        for (int sz = 0; sz < S; ++sz) {
          const int64_t gz = pmod(c[2] - sz, L);
          grid[(gx * L + gy) * L + gz] += phxy * phi[f[2] + res * sz];
        }
      }
    }
  }
  return 0;
}

/* Per-cell particle counts (the integer companion of the deposit):
 * counts[c] = number of particles whose floor(pos*L/box) cell (wrapped) is c. */
int oracle_cell_counts(const double* pos, int64_t n, int J, double box, uint32_t* counts) {
  const int64_t L = (int64_t)1 << J;
  const double scale = (double)L / box;
  memset(counts, 0, sizeof(uint32_t) * (size_t)(L * L * L));
  for (int64_t p = 0; p < n; ++p) {
    int64_t c[3];
    for (int a = 0; a < 3; ++a) c[a] = pmod((int64_t)(int32_t)floor(pos[3 * p + a] * scale), L);
    counts[(c[0] * L + c[1]) * L + c[2]] += 1;
  }
  return 0;
}

/* utils/wavelet_grid.py:143-186 (interpolate_grid_at_pos_numba):
 * out[i] = sum_s grid[(c-s)&mask] * phi_x * phi_y * phi_z at scaled
 * positions (already multiplied by L/box) plus an offset (dx,dy,dz). */
int oracle_interp(const double* scaled, int64_t n, const double* grid, int J, const double* phi,
                  int n_phi, int res, double dx, double dy, double dz, double* out) {
  const int64_t L = (int64_t)1 << J;
  const int64_t mask = L - 1;
  const int S = n_phi / res;
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < n; ++p) {
    const double sxp = scaled[3 * p] + dx, syp = scaled[3 * p + 1] + dy, szp = scaled[3 * p + 2] + dz;
    const int64_t xc = (int64_t)floor(sxp), yc = (int64_t)floor(syp), zc = (int64_t)floor(szp);
    const int64_t xf = (int64_t)((sxp - (double)xc) * res);
    const int64_t yf = (int64_t)((syp - (double)yc) * res);
    const int64_t zf = (int64_t)((szp - (double)zc) * res);
    double acc = 0.0;
    for (int a = 0; a < S; ++a) {
      const int64_t xg = (xc - a) & mask;
      const double px = phi[xf + a * res];
      for (int b = 0; b < S; ++b) {
        const int64_t yg = (yc - b) & mask;
        const double py = phi[yf + b * res];
        for (int c = 0; c < S; ++c) {
          const int64_t zg = (zc - c) & mask;
          const double pz = phi[zf + c * res];
          acc += grid[(xg * L + yg) * L + zg] * px * py * pz;
        }
      }
    }
    out[p] = acc;
  }
  return 0;
}

int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------------
 * Window transfer functions: utils/window_functions.py:29-438 and the
 * special functions they call, utils/special_functions.py:131-270.
 * ------------------------------------------------------------------------ */
enum {
  W_SPHERE = 0, W_GAUSSIAN, W_SHELL, W_THICK_SHELL, W_GAUSSIAN_SHELL, W_CUBIC, W_RING, W_DISK,
  W_CYLSHELL, W_CYLINDER, W_CW, W_CWS, W_GDW, W_DIRDERIV, W_LAPLACIAN, W_INVLAPLACIAN
};

static const double PI = 3.141592653589793;

static double j0_ref(double x) { /* special_functions.py:131-170 */
  double ax = fabs(x);
  if (ax < 8.0) {
    double y = x * x;
    double a1 = 57568490574.0 + y * (-13362590354.0 + y * (651619640.7 + y * (-11214424.18 + y * (77392.33017 + y * -184.9052456))));
    double a2 = 57568490411.0 + y * (1029532985.0 + y * (9494680.718 + y * (59272.64853 + y * (267.8532712 + y))));
    return a1 / a2;
  }
  double z = 8.0 / ax, y = z * z, xx = ax - 0.785398164;
  double a1 = 1.0 + y * (-0.1098628627e-2 + y * (0.2734510407e-4 + y * (-0.2073370639e-5 + y * 0.2093887211e-6)));
  double a2 = -0.1562499995e-1 + y * (0.1430488765e-3 + y * (-0.6911147651e-5 + y * (0.7621095161e-6 - y * 0.934945152e-7)));
  return sqrt(0.636619772 / ax) * (cos(xx) * a1 - z * sin(xx) * a2);
}

static double j1_ref(double x) { /* special_functions.py:173-215 */
  double ax = fabs(x);
  if (ax < 8.0) {
    double y = x * x;
    double a1 = x * (72362614232.0 + y * (-7895059235.0 + y * (242396853.1 + y * (-2972611.439 + y * (15704.48260 + y * -30.16036606)))));
    double a2 = 144725228442.0 + y * (2300535178.0 + y * (18583304.74 + y * (99447.43394 + y * (376.9991397 + y))));
    return a1 / a2;
  }
  double z = 8.0 / ax, y = z * z, xx = ax - 2.356194491;
  double a1 = 1.0 + y * (0.183105e-2 + y * (-0.3516396496e-4 + y * (0.2457520174e-5 + y * -0.240337019e-6)));
  double a2 = 0.04687499995 + y * (-0.2002690873e-3 + y * (0.8449199096e-5 + y * (-0.88228987e-6 + y * 0.105787412e-6)));
  double ans = sqrt(0.636619772 / ax) * (cos(xx) * a1 - z * sin(xx) * a2);
  return x < 0.0 ? -ans : ans;
}

static double jn01_ref(int n, double x) { /* jn_numba for n in {0,1}: special_functions.py:218-235 */
  double sign = 1.0;
  if (x < 0.0) {
    x = -x;
    if (n % 2 == 1) sign = -sign;
  }
  return n == 0 ? sign * j0_ref(x) : sign * j1_ref(x);
}

static double w_sphere(double ki, double kj, double kk, double R) {
  double k = sqrt(ki * ki + kj * kj + kk * kk);
  double q = 2 * PI * k * R;
  if (q == 0.0) return 1.0;
  return 3 * (sin(q) - q * cos(q)) / (q * q * q);
}

static double cw_g(double q) { /* window_functions.py:324-332 */
  double a = fabs(q);
  if (a == 0.0) return 0.0;
  if (a < 1.0e-4) return a * a * a * a / 3.0;
  if (a > 50.0) return 0.0;
  return a * (a * cosh(a) - sinh(a)) * exp(-0.5 * a * a);
}

static void los_norm(const double* los, double* n) {
  double nr = sqrt(los[0] * los[0] + los[1] * los[1] + los[2] * los[2]);
  n[0] = los[0] / nr;
  n[1] = los[1] / nr;
  n[2] = los[2] / nr;
}

/* W(k) for the built-in types; returns the real part, *im the imaginary. */
static double window_value(int type, const double* a, const double* los, double ki, double kj, double kk,
                           double* im) {
  *im = 0.0;
  switch (type) {
    case W_SPHERE: return w_sphere(ki, kj, kk, a[0]);
    case W_GAUSSIAN: {
      double k = sqrt(ki * ki + kj * kj + kk * kk), q = 2 * PI * k * a[0];
      return exp(-(q * q) / 2);
    }
    case W_SHELL: {
      double k = sqrt(ki * ki + kj * kj + kk * kk), q = 2 * PI * k * a[0];
      return q == 0.0 ? 1.0 : sin(q) / q;
    }
    case W_THICK_SHELL: {
      double rin = a[0] - 0.5 * a[1];
      if (rin < 0.0) rin = 0.0;
      double rout = a[0] + 0.5 * a[1];
      double den = rout * rout * rout - rin * rin * rin;
      if (den == 0.0) return 1.0;
      return (rout * rout * rout * w_sphere(ki, kj, kk, rout) - rin * rin * rin * w_sphere(ki, kj, kk, rin)) / den;
    }
    case W_GAUSSIAN_SHELL: {
      double k = sqrt(ki * ki + kj * kj + kk * kk);
      if (k == 0) return 1.0;
      double qs = 2 * PI * k * a[0], qm = 2 * PI * k * a[1];
      double den = a[0] * a[0] + a[1] * a[1];
      if (den == 0.0) return 1.0;
      double sinc = qs == 0.0 ? 1.0 : sin(qs) / qs;
      return (a[1] * a[1] * cos(qs) + a[0] * a[0] * sinc) / den * exp(-(qm * qm) / 2);
    }
    case W_CUBIC: {
      double q[3] = {PI * ki * a[0], PI * kj * a[1], PI * kk * a[2]}, r = 1.0;
      for (int i = 0; i < 3; ++i) r *= q[i] == 0.0 ? 1.0 : sin(q[i]) / q[i];
      return r;
    }
    case W_RING: case W_DISK: case W_CYLSHELL: case W_CYLINDER: {
      double n[3];
      los_norm(los, n);
      double kpar = ki * n[0] + kj * n[1] + kk * n[2];
      double k2 = ki * ki + kj * kj + kk * kk;
      double kp2 = k2 - kpar * kpar;
      if (kp2 < 0.0) kp2 = 0.0;
      double qperp = 2.0 * PI * sqrt(kp2) * a[0], qpar = 2.0 * PI * kpar * a[1];
      double perp, par;
      if (type == W_RING || type == W_CYLSHELL) perp = jn01_ref(0, qperp);
      else perp = qperp == 0.0 ? 1.0 : 2.0 * jn01_ref(1, qperp) / qperp;
      if (type == W_RING || type == W_DISK) par = cos(qpar);
      else par = qpar == 0.0 ? 1.0 : sin(qpar) / qpar;
      return perp * par;
    }
    case W_CW: {
      double k = sqrt(ki * ki + kj * kj + kk * kk), q = 2 * PI * k * a[0];
      double c = 2 * sqrt(2.0) / (sqrt(1.0 + 5.0 * 2.718281828459045) * pow(PI, 0.25));
      return sqrt(2.0 * PI) * c * pow(a[0], 0.5) * cw_g(q);
    }
    case W_CWS: {
      double k = sqrt(ki * ki + kj * kj + kk * kk), q = 2 * PI * k * a[0];
      double c = 2 * sqrt(2.0) / (sqrt(9.0 + 55.0 * 2.718281828459045) * pow(PI, 0.75));
      return pow(2.0 * PI, 1.5) * c * pow(a[0], 1.5) * cw_g(q);
    }
    case W_GDW: {
      double k = sqrt(ki * ki + kj * kj + kk * kk), q = 2 * PI * k * a[0];
      return pow(2.0, 2.5) * pow(PI, 0.75) / sqrt(15.0) * pow(a[0], 1.5) * q * q * exp(-(q * q) / 2);
    }
    case W_DIRDERIV: {
      double n[3];
      los_norm(los, n);
      *im = 2.0 * PI * (ki * n[0] + kj * n[1] + kk * n[2]);
      return 0.0;
    }
    case W_LAPLACIAN: return -((2.0 * PI) * (2.0 * PI)) * (ki * ki + kj * kj + kk * kk);
    case W_INVLAPLACIAN: {
      double k2 = ki * ki + kj * kj + kk * kk;
      return k2 == 0.0 ? 0.0 : -1.0 / (((2.0 * PI) * (2.0 * PI)) * k2);
    }
  }
  return NAN;
}

/* Octant kernel (convolution.py:14-38) folded to the rFFT grid (:263-281).
 * out: float64 [L, L, L/2+1]; P: L*bw+1 samples. */
int oracle_window_octant(int type, const double* args, const double* los, int L, int bw, const double* P,
                         double* out) {
  const int64_t M = L + 1;
  double* wa = (double*)malloc(sizeof(double) * (size_t)(M * M * M));
  if (!wa) return -1;
  const double invL = 1.0 / L;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < M; ++i)
    for (int64_t j = 0; j < M; ++j)
      for (int64_t k = 0; k < M; ++k) {
        double t = 0.0, im;
        for (int ii = 0; ii < bw; ++ii)
          for (int jj = 0; jj < bw; ++jj)
            for (int kk = 0; kk < bw; ++kk) {
              t += P[ii * L + i] * P[jj * L + j] * P[kk * L + k] *
                   window_value(type, args, los, (ii * L + i) * invL, (jj * L + j) * invL, (kk * L + k) * invL, &im);
            }
        wa[(i * M + j) * M + k] = t;
      }
  const int64_t H = L / 2 + 1;
#define WA(a, b, c) wa[((int64_t)(a) * M + (b)) * M + (c)]
#pragma omp parallel for schedule(static)
  for (int64_t x = 0; x < L; ++x)
    for (int64_t y = 0; y < L; ++y)
      for (int64_t z = 0; z < H; ++z)
        out[(x * L + y) * H + z] = WA(x, y, z) + WA(L - x, y, z) + WA(x, L - y, z) + WA(x, y, L - z) +
                                   WA(L - x, L - y, z) + WA(L - x, y, L - z) + WA(x, L - y, L - z) +
                                   WA(L - x, L - y, L - z);
#undef WA
  free(wa);
  return 0;
}

/* Full real / complex rFFT kernels (convolution.py:73-157, :168-252).
 * out: float64 [L, L, L/2+1, 2] (re, im). */
int oracle_window_rfft(int type, const double* args, const double* los, int L, int bw, const double* P,
                       double* out) {
  const int64_t H = L / 2 + 1;
  const double invL = 1.0 / L;
#pragma omp parallel for schedule(static)
  for (int64_t x = 0; x < L; ++x)
    for (int64_t y = 0; y < L; ++y)
      for (int64_t z = 0; z < H; ++z) {
        double tr = 0.0, ti = 0.0;
        for (int ii = 0; ii < bw; ++ii) {
          const int64_t xpi = ii * L + x, xni = ii * L + (L - x);
          const double xp = xpi * invL, xn = -xni * invL;
          for (int jj = 0; jj < bw; ++jj) {
            const int64_t ypi = jj * L + y, yni = jj * L + (L - y);
            const double yp = ypi * invL, yn = -yni * invL;
            for (int kk = 0; kk < bw; ++kk) {
              const int64_t zpi = kk * L + z, zni = kk * L + (L - z);
              const double zp = zpi * invL, zn = -zni * invL;
              const double px = P[xpi], nx = P[xni], py = P[ypi], ny = P[yni], pz = P[zpi], nz = P[zni];
              const double wx[8] = {px, nx, px, px, nx, nx, px, nx};
              const double wy[8] = {py, py, ny, py, ny, py, ny, ny};
              const double wz[8] = {pz, pz, pz, nz, pz, nz, nz, nz};
              const double ax[8] = {xp, xn, xp, xp, xn, xn, xp, xn};
              const double ay[8] = {yp, yp, yn, yp, yn, yp, yn, yn};
              const double az[8] = {zp, zp, zp, zn, zp, zn, zn, zn};
              for (int t = 0; t < 8; ++t) {
                double im, re = window_value(type, args, los, ax[t], ay[t], az[t], &im);
                double w = wx[t] * wy[t] * wz[t];
                tr += w * re;
                ti += w * im;
              }
            }
          }
        }
        out[2 * ((x * L + y) * H + z)] = tr;
        out[2 * ((x * L + y) * H + z) + 1] = ti;
      }
  return 0;
}

/* ------------------------------------------------------------------------
 * 3PCF multipoles: special functions (utils/special_functions.py:49-128,
 * 273-334), radial multipole windows (utils/radial_multipole_windows.py:
 * 66-183) and the triple-product contraction
 * (utils/corr3pcf_multipoles.py:134-170).
 * ------------------------------------------------------------------------ */
double oracle_spherical_jn(int l, double x) {
  if (l < 0) return NAN;
  if (x == 0.0) return l == 0 ? 1.0 : 0.0;
  double ax = fabs(x);
  if (ax <= 5.0e-2) {
    if (l == 0) {
      double x2 = x * x;
      return 1.0 - x2 / 6.0 + x2 * x2 / 120.0;
    }
    double denom = 1.0;
    for (int n = 1; n <= l; ++n) denom *= 2.0 * n + 1.0;
    double x2 = x * x;
    return (pow(x, l) / denom) * (1.0 - x2 / (2.0 * (2.0 * l + 3.0)) + x2 * x2 / (8.0 * (2.0 * l + 3.0) * (2.0 * l + 5.0)));
  }
  double sx = sin(x), cx = cos(x);
  double j0 = sx / x;
  if (l == 0) return j0;
  double j1 = sx / (x * x) - cx / x;
  if (l == 1) return j1;
  if (ax < l + 1.0) {
    int n_stop = l + 40;
    double jp1 = 0.0, jcur = 1.0, jt = 0.0, jd0 = 0.0, jd1 = 0.0;
    for (int n = n_stop; n > 0; --n) {
      double jm1 = ((2.0 * n + 1.0) / x) * jcur - jp1;
      if (n - 1 == l) jt = jm1;
      if (n - 1 == 1) jd1 = jm1;
      if (n - 1 == 0) jd0 = jm1;
      jp1 = jcur;
      jcur = jm1;
      if (fabs(jcur) > 1.0e200) {
        jp1 *= 1.0e-200; jcur *= 1.0e-200; jt *= 1.0e-200; jd0 *= 1.0e-200; jd1 *= 1.0e-200;
      } else if (fabs(jcur) < 1.0e-200 && jcur != 0.0) {
        jp1 *= 1.0e200; jcur *= 1.0e200; jt *= 1.0e200; jd0 *= 1.0e200; jd1 *= 1.0e200;
      }
    }
    if (fabs(jd0) >= fabs(jd1) || jd1 == 0.0) return jt * (j0 / jd0);
    return jt * (j1 / jd1);
  }
  double jm1 = j0, jc = j1;
  for (int e = 1; e < l; ++e) {
    double jn = ((2.0 * e + 1.0) / x) * jc - jm1;
    jm1 = jc;
    jc = jn;
  }
  return jc;
}

static double assoc_legendre(int l, int m, double x) {
  double pmm = 1.0;
  if (m > 0) {
    double somx2 = sqrt(fmax(0.0, 1.0 - x * x)), fact = 1.0;
    for (int i = 0; i < m; ++i) {
      pmm *= -fact * somx2;
      fact += 2.0;
    }
  }
  if (l == m) return pmm;
  double pmmp1 = x * (2.0 * m + 1.0) * pmm;
  if (l == m + 1) return pmmp1;
  double a = pmm, b = pmmp1, pll = 0.0;
  for (int e = m + 2; e <= l; ++e) {
    pll = ((2.0 * e - 1.0) * x * b - (e + m - 1.0) * a) / (e - m);
    a = b;
    b = pll;
  }
  return pll;
}

static double fact_small(int n) {
  double o = 1.0;
  for (int i = 2; i <= n; ++i) o *= i;
  return o;
}

/* Y_l^m(khat) (special_functions.py:307-334); returns re, *im. */
void oracle_sph_harm(int l, int m, double ki, double kj, double kk, double* re, double* im) {
  *re = 0.0;
  *im = 0.0;
  if (abs(m) > l) return;
  double k = sqrt(ki * ki + kj * kj + kk * kk);
  if (k == 0.0) {
    if (l == 0 && m == 0) *re = 1.0 / sqrt(4.0 * PI);
    return;
  }
  double mu = kk / k;
  if (mu > 1.0) mu = 1.0;
  else if (mu < -1.0) mu = -1.0;
  double theta = acos(mu), phi = atan2(kj, ki);
  int mp = m < 0 ? -m : m;
  double x = cos(theta);
  double P = assoc_legendre(l, mp, x);
  double norm = sqrt((2.0 * l + 1.0) / (4.0 * PI) * fact_small(l - mp) / fact_small(l + mp));
  double r = norm * P * cos(mp * phi), i = norm * P * sin(mp * phi);
  if (m >= 0) {
    *re = r;
    *im = i;
  } else {
    double sign = (mp % 2 == 1) ? -1.0 : 1.0;
    *re = sign * r;
    *im = -sign * i;
  }
}

static double sphere_profile(double k, double R) {
  double q = 2.0 * PI * k * R;
  if (q == 0.0) return 1.0;
  return 3.0 * (sin(q) - q * cos(q)) / (q * q * q);
}

/* _radial_profile (radial_multipole_windows.py:112-125); codes 0..4 =
 * shell, gaussian_shell, thick_shell, sphere, gaussian. */
static double radial_profile(double k, int code, const double* a, int l) {
  switch (code) {
    case 0: return oracle_spherical_jn(l, 2.0 * PI * k * a[0]);
    case 1: {
      if (k == 0.0) return 1.0;
      double qs = 2.0 * PI * k * a[0], qm = 2.0 * PI * k * a[1];
      double den = a[0] * a[0] + a[1] * a[1];
      if (den == 0.0) return 1.0;
      double sinc = qs == 0.0 ? 1.0 : sin(qs) / qs;
      return (a[1] * a[1] * cos(qs) + a[0] * a[0] * sinc) / den * exp(-0.5 * qm * qm);
    }
    case 2: {
      double rin = a[0] - 0.5 * a[1];
      if (rin < 0.0) rin = 0.0;
      double rout = a[0] + 0.5 * a[1];
      double den = rout * rout * rout - rin * rin * rin;
      if (den == 0.0) return 1.0;
      return (rout * rout * rout * sphere_profile(k, rout) - rin * rin * rin * sphere_profile(k, rin)) / den;
    }
    case 3: return sphere_profile(k, a[0]);
    case 4: {
      double q = 2.0 * PI * k * a[0];
      return exp(-0.5 * q * q);
    }
  }
  return NAN;
}

/* calculate_radial_multipole_window_array_numba (radial_multipole_windows.py:
 * 147-183): complex [L,L,L] (interleaved re, im), args in grid units. */
int oracle_radial_multipole_window_range(int L, const double* P, int code, const double* args, int l, int m,
                                         int x_begin, int x_end, double* out);
int oracle_radial_multipole_window(int L, const double* P, int code, const double* args, int l, int m,
                                   double* out) {
  return oracle_radial_multipole_window_range(L, P, code, args, l, m, 0, L, out);
}

/* The same window on the x planes [x_begin, x_end) only; out holds those
 * planes, [x_end - x_begin][L][L] interleaved complex. */
int oracle_radial_multipole_window_range(int L, const double* P, int code, const double* args, int l, int m,
                                         int x_begin, int x_end, double* out) {
  const double invL = 1.0 / L;
  if (x_begin < 0 || x_end > L || x_begin > x_end) return -1;
  out -= (int64_t)x_begin * L * L * 2;
#pragma omp parallel for schedule(static)
  for (int x = x_begin; x < x_end; ++x) {
    const double ki[2] = {(x - L) * invL, x * invL};
    const double pi_[2] = {P[L - x], P[x]};
    for (int y = 0; y < L; ++y) {
      const double kj[2] = {(y - L) * invL, y * invL};
      const double pj[2] = {P[L - y], P[y]};
      for (int z = 0; z < L; ++z) {
        const double kk[2] = {(z - L) * invL, z * invL};
        const double pk[2] = {P[L - z], P[z]};
        double sr = 0.0, si = 0.0;
        for (int a = 0; a < 2; ++a)
          for (int b = 0; b < 2; ++b)
            for (int c = 0; c < 2; ++c) {
              double yr = 0.0, yi = 0.0, rad = 0.0;
              if (l >= 0 && abs(m) <= l) {
                double kn = sqrt(ki[a] * ki[a] + kj[b] * kj[b] + kk[c] * kk[c]);
                rad = radial_profile(kn, code, args, l);
                oracle_sph_harm(l, m, ki[a], kj[b], kk[c], &yr, &yi);
              }
              double w = pi_[a] * pj[b] * pk[c];
              sr += w * (rad * yr);
              si += w * (rad * yi);
            }
        int64_t o = (((int64_t)x * L + y) * L + z) * 2;
        out[o] = sr;
        out[o + 1] = si;
      }
    }
  }
  return 0;
}

/* compute_3d_summand_cpu (corr3pcf_multipoles.py:134-170): sum over cells of
 * data(x) * sum_{l1,l2} Gamma3(l1,l2) a1(x-l1) a2(x-l2); a1/a2 interleaved
 * complex [L^3]; returns re/im. */
int oracle_contract_range(const double* data, const double* a1, const double* a2, const double* gamma, int L,
                          int S, int x_begin, int x_end, double* out_re, double* out_im);
int oracle_contract(const double* data, const double* a1, const double* a2, const double* gamma, int L, int S,
                    double* out_re, double* out_im) {
  return oracle_contract_range(data, a1, a2, gamma, L, S, 0, L, out_re, out_im);
}

/* The same sum over the cells of the x planes [x_begin, x_end) only (their
 * neighbourhoods still read the whole periodic grid). */
int oracle_contract_range(const double* data, const double* a1, const double* a2, const double* gamma, int L,
                          int S, int x_begin, int x_end, double* out_re, double* out_im) {
  const int64_t plane = (int64_t)L * L;
  if (x_begin < 0 || x_end > L || x_begin > x_end) return -1;
  const int64_t idx_begin = (int64_t)x_begin * plane, idx_end = (int64_t)x_end * plane;
  double tr = 0.0, ti = 0.0;
#pragma omp parallel for reduction(+ : tr, ti) schedule(static)
  for (int64_t idx = idx_begin; idx < idx_end; ++idx) {
    const int64_t lx = idx / plane, rem = idx - lx * plane, ly = rem / L, lz = rem - ly * L;
    double s1r = 0.0, s1i = 0.0;
    for (int l1x = 0; l1x < S; ++l1x) {
      const int64_t i1x = pmod(lx - l1x, L);
      for (int l1y = 0; l1y < S; ++l1y) {
        const int64_t i1y = pmod(ly - l1y, L);
        for (int l1z = 0; l1z < S; ++l1z) {
          const int64_t i1z = pmod(lz - l1z, L);
          double s2r = 0.0, s2i = 0.0;
          for (int l2x = 0; l2x < S; ++l2x) {
            const int64_t i2x = pmod(lx - l2x, L);
            const double gx = gamma[l1x * S + l2x];
            for (int l2y = 0; l2y < S; ++l2y) {
              const int64_t i2y = pmod(ly - l2y, L);
              const double gxy = gx * gamma[l1y * S + l2y];
              for (int l2z = 0; l2z < S; ++l2z) {
                const int64_t i2z = pmod(lz - l2z, L);
                const double w = gxy * gamma[l1z * S + l2z];
                const int64_t o = ((i2x * L + i2y) * L + i2z) * 2;
                s2r += w * a2[o];
                s2i += w * a2[o + 1];
              }
            }
          }
          const int64_t o1 = ((i1x * L + i1y) * L + i1z) * 2;
          s1r += a1[o1] * s2r - a1[o1 + 1] * s2i;
          s1i += a1[o1] * s2i + a1[o1 + 1] * s2r;
        }
      }
    }
    const double d = data[idx];
    tr += d * s1r;
    ti += d * s1i;
  }
  *out_re = tr;
  *out_im = ti;
  return 0;
}

/* S[b2][b3] = sum over cells of data(x) * sum_{l1,l2} Gamma3(l1,l2)
 * a2_b2(x-l1) a3_b3(x-l2) for every bin pair at once: per pair the
 * per-cell arithmetic of oracle_contract (compute_3d_summand_cpu,
 * corr3pcf_multipoles.py:134-170), with the inner sum over l2 formed once
 * per (cell, l1, b3) and reused by every b2.  a2: [nb2][L^3], a3: [nb3][L^3]
 * interleaved complex; out: [nb2][nb3][2].  Per-thread partial sums are added
 * in thread order. */
int oracle_contract_bins_range(const double* data, const double* a2, int nb2, const double* a3, int nb3,
                               const double* gamma, int L, int x_begin, int x_end, double* out);
int oracle_contract_bins(const double* data, const double* a2, int nb2, const double* a3, int nb3,
                         const double* gamma, int L, double* out) {
  return oracle_contract_bins_range(data, a2, nb2, a3, nb3, gamma, L, 0, L, out);
}

/* The sum restricted to the cells of x planes [x_begin, x_end) (their
 * neighbourhoods still read the whole periodic grid). */
int oracle_contract_bins_range(const double* data, const double* a2, int nb2, const double* a3, int nb3,
                               const double* gamma, int L, int x_begin, int x_end, double* out) {
  enum { S = 3, MAXB = 16 };
  if (nb2 < 1 || nb3 < 1 || nb2 > MAXB || nb3 > MAXB) return -1;
  if (x_begin < 0 || x_end > L || x_begin > x_end) return -1;
  const int64_t N = (int64_t)L * L * L, plane = (int64_t)L * L;
  const int64_t idx_begin = (int64_t)x_begin * plane, idx_end = (int64_t)x_end * plane;
  int nthr = 1;
#ifdef _OPENMP
  nthr = omp_get_max_threads();
#endif
  double* part = (double*)calloc((size_t)nthr * nb2 * nb3 * 2, sizeof(double));
  if (!part) return -2;
#pragma omp parallel
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
    double* acc = part + (size_t)t * nb2 * nb3 * 2;
    double s2r[MAXB], s2i[MAXB], s1r[MAXB * MAXB], s1i[MAXB * MAXB];
#pragma omp for schedule(static)
    for (int64_t idx = idx_begin; idx < idx_end; ++idx) {
      const int64_t lx = idx / plane, rem = idx - lx * plane, ly = rem / L, lz = rem - ly * L;
      for (int q = 0; q < nb2 * nb3; ++q) s1r[q] = s1i[q] = 0.0;
      for (int l1x = 0; l1x < S; ++l1x) {
        const int64_t i1x = pmod(lx - l1x, L);
        for (int l1y = 0; l1y < S; ++l1y) {
          const int64_t i1y = pmod(ly - l1y, L);
          for (int l1z = 0; l1z < S; ++l1z) {
            const int64_t i1z = pmod(lz - l1z, L);
            for (int b = 0; b < nb3; ++b) s2r[b] = s2i[b] = 0.0;
            for (int l2x = 0; l2x < S; ++l2x) {
              const int64_t i2x = pmod(lx - l2x, L);
              const double gx = gamma[l1x * S + l2x];
              for (int l2y = 0; l2y < S; ++l2y) {
                const int64_t i2y = pmod(ly - l2y, L);
                const double gxy = gx * gamma[l1y * S + l2y];
                for (int l2z = 0; l2z < S; ++l2z) {
                  const int64_t i2z = pmod(lz - l2z, L);
                  const double w = gxy * gamma[l1z * S + l2z];
                  const int64_t o = ((i2x * L + i2y) * L + i2z) * 2;
                  for (int b = 0; b < nb3; ++b) {
                    s2r[b] += w * a3[(size_t)b * 2 * N + o];
                    s2i[b] += w * a3[(size_t)b * 2 * N + o + 1];
                  }
                }
              }
            }
            const int64_t o1 = ((i1x * L + i1y) * L + i1z) * 2;
            for (int a = 0; a < nb2; ++a) {
              const double ar = a2[(size_t)a * 2 * N + o1], ai = a2[(size_t)a * 2 * N + o1 + 1];
              for (int b = 0; b < nb3; ++b) {
                s1r[a * nb3 + b] += ar * s2r[b] - ai * s2i[b];
                s1i[a * nb3 + b] += ar * s2i[b] + ai * s2r[b];
              }
            }
          }
        }
      }
      const double d = data[idx];
      for (int q = 0; q < nb2 * nb3; ++q) {
        acc[2 * q] += d * s1r[q];
        acc[2 * q + 1] += d * s1i[q];
      }
    }
  }
  for (int q = 0; q < nb2 * nb3 * 2; ++q) {
    double s = 0.0;
    for (int t = 0; t < nthr; ++t) s += part[(size_t)t * nb2 * nb3 * 2 + q];
    out[q] = s;
  }
  free(part);
  return 0;
}
