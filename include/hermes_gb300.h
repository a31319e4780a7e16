/*
 * hermes_gb300.h — C ABI of the GB300-native PyHermes field pipeline.
 *
 * Every entry point:
 *   - takes plain pointers and sizes (device pointers unless named h_*),
 *   - is asynchronous on the caller's `stream` (a cudaStream_t passed as
 *     void*; NULL = legacy default stream) unless documented otherwise,
 *   - never aborts: returns HERMES_OK (0) or a negative HERMES_ERR_* code and
 *     leaves a message for hermes_last_error() (thread-local),
 *   - allocates no device memory of its own except where stated (cuFFT plans
 *     are cached per (shape, device) inside the library); scratch space is a
 *     caller-owned `workspace` sized by the matching *_workspace_size call.
 *
 * Reference interfaces replaced (paths are within SYSUSPA-Projects/PyHermes):
 *   see the comment above each declaration.
 */
#ifndef HERMES_GB300_H
#define HERMES_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define HERMES_OK 0
#define HERMES_ERR_INVALID -1     /* bad argument (shape, size, null)        */
#define HERMES_ERR_CUDA -2        /* a CUDA runtime call failed              */
#define HERMES_ERR_CUFFT -3       /* a cuFFT call failed                     */
#define HERMES_ERR_WORKSPACE -4   /* workspace too small                     */
#define HERMES_ERR_UNSUPPORTED -5 /* valid request this build does not serve */
#define HERMES_ERR_DATA -6        /* input data rejected (non-finite, range) */
#define HERMES_ERR_TIMEOUT -7     /* a bounded device wait gave up           */

/* Library version string and the message of the last failing call. */
const char* hermes_version(void);
const char* hermes_last_error(void);

/* ---- SFC deposit ---------------------------------------------------------
 * Replaces utils/wavelet_grid.py:58-70 project_scaling_grid_numba (and its
 * body _project_scaling_grid_impl :17-55) as called from
 * base/sfc_projection.py:317-324.
 *
 * eps[x,y,z] (C order, L = 2^J) = sum_p w_p * phi[fx+res*sx] * phi[fy+res*sy]
 *   * phi[fz+res*sz] over s in [0,support)^3 at cell (c - s) mod L, with
 *   c = floor(pos*L/box), f = int((pos*L/box - c)*res), computed in float64.
 * pos: n x 3 float64 (row-major), w: n float64 (the normalised projection
 * weights), phi: n_phi float64 samples with n_phi = support*res, support 3.
 * eps_out: L^3 float32 (eps_f64_out may be used instead: L^3 float64; give
 * exactly one of the two). counts_out (nullable): L^3 uint32 per-cell
 * particle counts (cell c of each particle).
 * Accumulation is fixed-point int64 per cell, so the result does not depend
 * on particle order or thread scheduling (bitwise deterministic).
 * Positions are wrapped periodically into [0, box).  Non-finite positions
 * or weights are counted in the device status word (see
 * hermes_deposit_status) and skipped.
 */
int hermes_deposit_workspace_size(int64_t n, int J, size_t* bytes);
int hermes_deposit(const double* pos, const double* w, int64_t n, int J,
                   double box, const double* phi, int n_phi, int phi_res,
                   float* eps_out, double* eps_f64_out, uint32_t* counts_out,
                   void* workspace, size_t workspace_bytes, void* stream);
/* The two phases of hermes_deposit, callable separately (same arguments and
 * workspace): the counting sort of particles into (tile, region) buckets,
 * then the per-tile accumulation that writes eps_out / counts_out. */
int hermes_deposit_sort(const double* pos, const double* w, int64_t n, int J,
                        double box, const double* phi, int n_phi, int phi_res,
                        void* workspace, size_t workspace_bytes, void* stream);
int hermes_deposit_accumulate(int64_t n, int J, double box, const double* phi,
                              int n_phi, int phi_res, float* eps_out,
                              double* eps_f64_out, uint32_t* counts_out,
                              void* workspace, size_t workspace_bytes,
                              void* stream);
/* Reads (synchronously) the count of skipped non-finite particles from the
 * workspace of the last hermes_deposit issued with it. */
int hermes_deposit_status(const void* workspace, int64_t* n_rejected,
                          void* stream);

#ifdef __cplusplus
}
#endif
#endif /* HERMES_GB300_H */
