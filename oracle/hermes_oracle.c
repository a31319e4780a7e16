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
