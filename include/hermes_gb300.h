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
/* hermes_deposit without any device allocation, for callers that cannot
 * allocate device memory (code inside an allocator's callbacks, plug-ins of
 * hosts that budget all of HBM, runs that must not fail on allocation).  No
 * counterpart in the reference: it is an addition of this library.  Same
 * arguments and result as hermes_deposit minus the workspace; the scratch
 * is a 4.5 MiB array built into the library (held on every GPU that loads
 * it until exit).  Limits: n <= 131072 particles, J <= 8; larger requests
 * return HERMES_ERR_INVALID.  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress), so make that first call
 * before any stream capture; the address is kept for the life of the
 * process, so it is not valid after cudaDeviceReset or in a second CUDA
 * context on the same device.  All calls share the one array: calls whose
 * work overlaps on the GPU (other streams, other host threads) race. */
int hermes_deposit_noalloc(const double* pos, const double* w, int64_t n, int J,
                           double box, const double* phi, int n_phi, int phi_res,
                           float* eps_out, double* eps_f64_out, uint32_t* counts_out,
                           void* stream);
/* Reads (synchronously) the count of skipped non-finite particles from the
 * workspace of the last hermes_deposit issued with it. */
int hermes_deposit_status(const void* workspace, int64_t* n_rejected,
                          void* stream);
/* Tile shape (cells along x, y, z) of the deposit accumulation at grid level
 * J, for hermes_deposit, hermes_deposit_sort / _accumulate and
 * hermes_deposit_workspace_size from this call on, process-wide.  No
 * counterpart in the reference (its deposit has no tiles): it is the control
 * the deposit tile autotuner sets.  Powers of two; x and y in [4, 128], z in
 * [4, 128]; at most 16384 cells; (0, 0, 0) restores the default 8 x 16 x 32.
 * A tile larger than the grid is clipped to it.  The field is the same bit
 * for bit for every tile (integer fixed-point sums); the workspace size
 * depends on the tile, so query it after setting the tile, and do not change
 * the tile of a level while another thread deposits at it.
 * hermes_deposit_noalloc always uses the default tile. */
int hermes_deposit_set_tile(int J, int tx, int ty, int tz);
int hermes_deposit_get_tile(int J, int* tx, int* ty, int* tz);

/* The scaling function's precomputes on the device, as
 * utils/wavelet_grid.py:94-118 fourier_power_spectrum (power_out[n] =
 * |phi_hat(n / L)|^2, n = 0 .. L * bandwidth, L * bandwidth + 1 float64) and
 * utils/corr3pcf_multipoles.py:22-30 cal_gamma (gamma_out[l1 * S + l2],
 * S = n_phi / phi_res <= 5, float64).  phi: device float64 [n_phi]; either
 * output may be NULL.  The Python layer keeps its host copy of these small
 * tables (cached per phi); this is the same computation for C callers. */
int hermes_phi_prepare(const double* phi, int n_phi, int phi_res, int L, int bandwidth,
                       double* power_out, double* gamma_out, void* stream);

/* ---- spectral windows ------------------------------------------------------
 * Built-in window transfer functions (utils/window_functions.py:441-458),
 * evaluated on the fly inside the passes below instead of being materialised
 * as an L^3 kernel array.  Lengths are in grid units (the reference's
 * WindowFunc rescales len_args by L/box, io/window.py:112).
 */
#define HERMES_WIN_SPHERE 0                 /* len = {R}                 */
#define HERMES_WIN_GAUSSIAN 1               /* len = {R}                 */
#define HERMES_WIN_SHELL 2                  /* len = {R}                 */
#define HERMES_WIN_THICK_SHELL 3            /* len = {R, delta_R}        */
#define HERMES_WIN_GAUSSIAN_SHELL 4         /* len = {R_shell, R_smooth} */
#define HERMES_WIN_CUBIC 5                  /* len = {Lx, Ly, Lz}        */
#define HERMES_WIN_RING 6                   /* len = {R, H}, los         */
#define HERMES_WIN_DISK 7                   /* len = {R, H}, los         */
#define HERMES_WIN_CYLSHELL 8               /* len = {R, H}, los         */
#define HERMES_WIN_CYLINDER 9               /* len = {R, H}, los         */
#define HERMES_WIN_CW 10                    /* len = {R}                 */
#define HERMES_WIN_CWS 11                   /* len = {R}                 */
#define HERMES_WIN_GDW 12                   /* len = {R}                 */
#define HERMES_WIN_DIRECTIONAL_DERIVATIVE 13 /* los                      */
#define HERMES_WIN_LAPLACIAN 14
#define HERMES_WIN_INVERSE_LAPLACIAN 15

/* Kernel modes (io/window.py:172-195, utils/window_params.py:75-84). */
#define HERMES_KMODE_OCTANT 0        /* real, mirror-symmetric images      */
#define HERMES_KMODE_FULL_RFFT 1     /* real, signed images                */
#define HERMES_KMODE_COMPLEX_RFFT 2  /* complex, signed images             */

typedef struct hermes_window {
  int32_t type;           /* HERMES_WIN_*                                   */
  int32_t kernel_mode;    /* HERMES_KMODE_*                                 */
  int32_t zero_mode_zero; /* 1: K(0,0,0) = 0 (io/window.py:266-272)         */
  int32_t reserved;
  double len[4];          /* length arguments in grid units                 */
  double los[3];          /* line of sight / direction (any non-zero norm)  */
  double scale;           /* multiplies the kernel (composite scalar ops)   */
} hermes_window_t;

/* Forward / inverse 3D FFTs in float32 (the reference's scipy.fft rfftn,
 * irfftn, fftn, ifftn in utils/convolution.py:284-295).  Unnormalised like
 * cuFFT (the inverse passes below fold in 1/L^3).  C2R overwrites `spec`. */
int hermes_fft_r2c(const float* field, void* spec /* float2 [L,L,L/2+1] */,
                   int J, void* stream);
int hermes_fft_c2r(void* spec, float* field, int J, void* stream);

/* field @ window for a real field and an rFFT-grid window
 * (utils/convolution.py:284-288 + io/sfc_field.py:93-150): rfftn, multiply by
 * the window kernel evaluated on the fly (phi_power: L*bandwidth+1 float64
 * samples of |phi_hat|^2, wavelet_grid.py:94-100), irfftn.  `out` may alias
 * `eps`.  Workspace: hermes_window_workspace_size. */
int hermes_window_workspace_size(int J, size_t* bytes);
int hermes_window_apply(const float* eps, float* out, int J,
                        const hermes_window_t* win, const double* phi_power,
                        int bandwidth, void* workspace, size_t workspace_bytes,
                        void* stream);

/* Materialise a window kernel on the rFFT grid (io/window.py:274-343):
 * k_real float [L,L,L/2+1] for real modes, or k_cplx float2 for
 * HERMES_KMODE_COMPLEX_RFFT (give the one that matches). */
int hermes_window_materialize(const hermes_window_t* win, const double* phi_power,
                              int bandwidth, int J, float* k_real, void* k_cplx,
                              void* stream);
/* spec *= K (materialised kernel, real or complex) -- for composite windows. */
int hermes_spectrum_multiply(void* spec, const float* k_real, const void* k_cplx,
                             int J, double factor, void* stream);

/* Pair products for many bins in one pass over the spectra
 * (theory/corr2pcf.py:366-372 pair_product_with_window, by Parseval):
 *   out[b*n_pairs+p] = (1/L^6) sum_k F_i(k) K_b(k) conj(F_j(k))
 * over the full k grid (half spectrum with Hermitian weights), where
 * (i, j) = pairs[2p], pairs[2p+1] index into `spectra`, an array of
 * n_spec device pointers to float2 [L,L,L/2+1] half spectra (host array).
 * If exclude_k0 != 0 the k = 0 term is left out (added by the caller in
 * float64 for mean-subtracted fields).  bins: host array of n_bins windows.
 * out: host float64 [n_bins * n_pairs]; k0_out (nullable): host float64
 * [n_bins] kernel values K_b(0); the call synchronises `stream`. */
int hermes_pair_products_workspace_size(int J, int n_bins, int n_pairs, size_t* bytes);
int hermes_pair_products(const void* const* spectra, int n_spec, const int32_t* pairs,
                         int n_pairs, const hermes_window_t* bins, int n_bins,
                         const double* phi_power, int bandwidth, int J, int exclude_k0,
                         double* out, double* k0_out, void* workspace,
                         size_t workspace_bytes, void* stream);

/* ---- 3PCF multipoles ---------------------------------------------------------
 * Replaces, per (l, m), the per-sample loop of
 * utils/corr3pcf_multipoles.py:505-555 (_stream_convolution_fields +
 * compute_multipole_m_summand) for all radial bins at once.
 *
 * hermes_multipole_fields: for a real field with half spectrum `half_spec`
 * (float2 [L,L,L/2+1], from hermes_fft_r2c) and thin-shell radii `radii`
 * (host, grid units, nb <= 16), writes
 *   a_lm^b = ifftn(fftn(eps) * K_lm^b)
 * into fields_out, complex64 and bin-interleaved: [L^3][16] (cell c, bin b at
 * c*16 + b; slots b >= nb are unspecified) when nb > 1, plain [L^3] when
 * nb == 1,
 * with K_lm^b the radial-multipole window of radial_multipole_windows.py:
 * 128-183 (shell profile: j_l(2 pi |k| R_b) Y_lm(khat), 8 phi-weighted
 * images; phi_power: L+1 float64 samples).
 *
 * hermes_multipole_contract: S[b2][b3] (host float64 complex, [nb2][nb3][2])
 *   = 4 pi / L^3 sum_x eps1(x) sum_{l1,l2} Gamma3(l1,l2) a2^{b2}(x-l1) a3^{b3}(x-l2)
 * for every bin pair (corr3pcf_multipoles.py:33-58 + :451), with
 * a2 = fields2 and a3 = fields3 (each in the layout hermes_multipole_fields
 * writes for its nb), or a3 = conj_sign * conj(fields2) when
 * fields3 is NULL (the a_{l,-m} = (-1)^{l+m} conj(a_{lm}) identity for a
 * shared field and shared bins).  gamma: host float64 [3][3] triple overlaps
 * (corr3pcf_multipoles.py:22-30).  Synchronises `stream`.
 *
 * hermes_multipole_contract_plain: the same sum for one (a2, a3) pair in the
 * reference's per-cell loop form (workspace >= 16*(#SM*8+1) bytes).
 *
 * hermes_multipole_workspace_size(J, nb): bytes of device workspace for
 * fields/contract calls with up to nb bins: two radial tables of
 * (3 L^2 + 1) x 16 floats (the second for degree pairs), the contraction's
 * partial sums and, for nb > 1, the nb * L^3 complex64 bin-major fields
 * that the inverse FFT transforms before the interleave.
 */
int hermes_multipole_workspace_size(int J, int nb, size_t* bytes);
int hermes_multipole_fields(const void* half_spec, int J, int l, int m,
                            const double* radii, int nb, const double* phi_power,
                            void* fields_out, void* workspace, size_t workspace_bytes,
                            void* stream);
int hermes_multipole_contract(const float* eps1, const void* fields2, int nb2,
                              const void* fields3, int nb3, int conj_sign,
                              const double* gamma, int J, double* out,
                              void* workspace, size_t workspace_bytes, void* stream);
/* hermes_multipole_fields_window / _table: the same fields for radial
 * profiles other than the thin shell (radial_multipole_windows.py:186-313),
 * the Y_lm, image sum, FFT and output layout unchanged.  _window: isotropic
 * analytic transfers of `bins` (host, nb; types SPHERE, GAUSSIAN, SHELL,
 * THICK_SHELL, GAUSSIAN_SHELL, lengths in grid units) -- the l = 0 monopole
 * path of the reference.  _table: U_l(k) from uniform tables over
 * [0, k_max[b]] (tables: device float64, bin b at offsets[b], sizes[b] >= 4
 * points; offsets, sizes, k_max on the host), evaluated at physical
 * k = |k_grid| * grid_to_physical (grid_to_physical = L / box) with the
 * reference's local cubic (utils/radial_multipole_windows.py:186-210); the
 * tables come from the host restatement of build_radial_multipole_table
 * (utils/radial_profiles.py:651-709). */
int hermes_multipole_fields_window(const void* half_spec, int J, int l, int m,
                                   const hermes_window_t* bins, int nb, const double* phi_power,
                                   void* fields_out, void* workspace, size_t workspace_bytes,
                                   void* stream);
int hermes_multipole_fields_table(const void* half_spec, int J, int l, int m, const double* tables,
                                  const int64_t* offsets, const int32_t* sizes, const double* k_max,
                                  double grid_to_physical, int nb, const double* phi_power,
                                  void* fields_out, void* workspace, size_t workspace_bytes,
                                  void* stream);

/* hermes_multipole_contract_async: the same S[b2][b3] (times 4 pi / L^3) into
 * the DEVICE array dev_out [16][16][2] float64 (slots b >= nb are zero or
 * unspecified), with no host synchronisation and no host-device copy, so a
 * sequence of fields/contract calls can be captured into a CUDA graph once
 * cuFFT plans and kernel attributes exist (make one uncaptured call per J
 * first).  chunk_x: x planes per work item (power of two <= L; 0 = min(64, L));
 * ctas_per_sm: 1 or 2 (0 = 2) -- the tile choices an autotuner varies.  Same
 * reference sum as hermes_multipole_contract (corr3pcf_multipoles.py:33-58). */
int hermes_multipole_contract_async(const float* eps1, const void* fields2, int nb2,
                                    const void* fields3, int nb3, int conj_sign,
                                    const double* gamma, int J, int chunk_x, int ctas_per_sm,
                                    double* dev_out, void* workspace, size_t workspace_bytes,
                                    void* stream);
/* Contraction engines.  hermes_multipole_contract and _async run the stencil
 * G^{b3}(y) = sum Gamma3 eps1 a3 on the CUDA cores (FP32) and the bin x bin
 * product S += a2^{b2} G^{b3} of every plane on the tcgen05 tensor cores:
 * BF16x3 operands (each FP32 value split into three BF16 parts, ~24
 * significant bits, all nine partial products summed), FP32 accumulation
 * in tensor memory over a work item, float64 across items
 * (corr3pcf_multipoles.py:33-58 + :99-131).
 * hermes_multipole_contract_simt_async: the same sum with the product on the
 * CUDA cores in FP32 (the all-FP32 comparison path); same arguments.
 * hermes_multipole_contract_status: after a tensor-core contraction on the
 * same workspace, *status = 0, or the first bounded wait that gave up (1: an
 * a2 plane's TMA load, 2 or 3: an MMA completion); its results are then NaN.
 * Synchronises `stream`. */
int hermes_multipole_contract_simt_async(const float* eps1, const void* fields2, int nb2,
                                         const void* fields3, int nb3, int conj_sign,
                                         const double* gamma, int J, int chunk_x, int ctas_per_sm,
                                         double* dev_out, void* workspace, size_t workspace_bytes,
                                         void* stream);
int hermes_multipole_contract_status(const void* workspace, size_t workspace_bytes, int J, int* status,
                                     void* stream);

/* Bin-major layout (same reference functions as the calls above).
 * hermes_multipole_fields_bm / _window_bm / _table_bm: the fields of
 * hermes_multipole_fields / _window / _table written as complex64
 * [nb][L^3], bin b at fields_out + b * L^3, the layout the batched inverse
 * FFT produces: no interleave pass, and the workspace is
 * hermes_multipole_workspace_size(J, 1) (no bin-major staging copy).
 * hermes_multipole_contract_bm_async: hermes_multipole_contract_async on
 * fields in that layout (tensor-core engine; a2 planes by a 4-D TMA map
 * over (z, y, x, bin), a3 planes staged per bin); workspace as above.
 * The sums are the same operations on the same values as the interleaved
 * path, so S is bit-identical to it. */
int hermes_multipole_fields_bm(const void* half_spec, int J, int l, int m, const double* radii, int nb,
                               const double* phi_power, void* fields_out, void* workspace,
                               size_t workspace_bytes, void* stream);
int hermes_multipole_fields_window_bm(const void* half_spec, int J, int l, int m, const hermes_window_t* bins,
                                      int nb, const double* phi_power, void* fields_out, void* workspace,
                                      size_t workspace_bytes, void* stream);
int hermes_multipole_fields_table_bm(const void* half_spec, int J, int l, int m, const double* tables,
                                     const int64_t* offsets, const int32_t* sizes, const double* k_max,
                                     double grid_to_physical, int nb, const double* phi_power, void* fields_out,
                                     void* workspace, size_t workspace_bytes, void* stream);
int hermes_multipole_contract_bm_async(const float* eps1, const void* fields2, int nb2,
                                       const void* fields3, int nb3, int conj_sign,
                                       const double* gamma, int J, int chunk_x, int ctas_per_sm,
                                       double* dev_out, void* workspace, size_t workspace_bytes,
                                       void* stream);
/* Degree pairs (no reference counterpart; together they replace the m = 0
 * terms of degrees l and l + 1 in the loop of calc_DDD_multipole,
 * utils/corr3pcf_multipoles.py:512-555, for thin shells on the bin-major
 * layout).  For m = 0 the field a_{l,0} is real for even l and imaginary
 * for odd l, so one complex field carries both degrees of a pair.
 * hermes_multipole_fields_pair_bm: l even (l + 1 <= 40); fields_out =
 * a_{l,0} + a_{l+1,0} for the nb radii, complex64 [nb][L^3], one prepass
 * and one batched inverse FFT (workspace: hermes_multipole_workspace_size(J,
 * 1)).  HERMES_ERR_INVALID for odd or out-of-range l.
 * hermes_multipole_contract_pair_bm_async: on those fields, dev_out[b2][b3]
 * = (S_{l,0}[b2][b3], S_{l+1,0}[b2][b3]), each the m = 0 summand that
 * hermes_multipole_contract_bm_async gives for its degree alone (real; the
 * imaginary parts there are rounding), scaled the same way. */
int hermes_multipole_fields_pair_bm(const void* half_spec, int J, int l, const double* radii, int nb,
                                    const double* phi_power, void* fields_out, void* workspace,
                                    size_t workspace_bytes, void* stream);
int hermes_multipole_contract_pair_bm_async(const float* eps1, const void* fields, int nb,
                                            const double* gamma, int J, int chunk_x, int ctas_per_sm,
                                            double* dev_out, void* workspace, size_t workspace_bytes,
                                            void* stream);
/* The inverse 3-D FFT of the multipole fields (replaces the ifftn of
 * _stream_convolution_fields, utils/corr3pcf_multipoles.py:267-321).
 * hermes_multipole_set_fft: 0 = cuFFT's batched 3-D plan; 1 (default) = at
 * J = 9, cuFFT's 1-D z lines followed by hermes_fft512_strided_inverse over
 * y and x (other J keep the 3-D plan).  Returns the previous mode,
 * HERMES_ERR_INVALID outside [0, 1].  Process-wide.
 * hermes_fft512_strided_inverse: in-place unnormalised inverse 512-point
 * FFTs (e^{+2 pi i n k / 512}, as CUFFT_INVERSE) along axis 0 (x, element
 * stride 512^2) or 1 (y, stride 512) of nfields (1..64) complex64 fields
 * [512][512][512]. */
int hermes_multipole_set_fft(int mode);
int hermes_fft512_strided_inverse(void* data, int nfields, int axis, void* stream);
int hermes_multipole_contract_plain(const float* eps1, const void* a2, const void* a3,
                                    const double* gamma, int J, double* out,
                                    void* workspace, size_t workspace_bytes, void* stream);

/* hermes_mixing_solve: replaces solve_multipoles_from_ratio +
 * build_mixing_matrix (utils/special_functions.py:366-409) for n_sys samples
 * at once, float64 on the device.  A, B: [n_sys][n] (n = lmax + 1 <= 32,
 * B[s][0] != 0, checked by the caller as the reference raises ValueError);
 * gaunt: [n][n][n], gaunt[k][l][l'] = legendre_triple_coeff(l, l', k).
 * Writes zeta_out [n_sys][n] = M^{-1} A and, when non-NULL, m_out
 * [n_sys][n][n] (the mixing matrices) and cond_out [n_sys] (2-norm condition
 * numbers).  All pointers are device memory; asynchronous on `stream`. */
int hermes_mixing_solve(const double* A, const double* B, const double* gaunt, int n_sys, int n,
                        double* zeta_out, double* m_out, double* cond_out, void* stream);

/* ---- Monte Carlo 3PCF ---------------------------------------------------------
 * hermes_interp: utils/wavelet_grid.py:143-186 interpolate_grid_at_pos_numba:
 * out[i] (float64) = 27-point phi-weighted value of `grid` (float32 [L^3]) at
 * scaled position (pos * L/box) + (dx, dy, dz); phi: 3*phi_res float64.
 *
 * hermes_mc_triplets: utils/corr3pcf_kernels.py:66-140 for one mu:
 *   sum_out = sum_i w_i n1(x_i) sum_r n2(x_i + d2_r) n3(x_i + d3_r)
 * (float64), with n1 = eps1 interpolated (box-random centres) or rho1 when
 * eps1 is NULL (particle centres, w = center_w or 1).  offsets: n_rot x 6
 * float64 (scaled) triangle offsets (generate_triangle_offsets, :21-63, from
 * the reference's per-rotation seeded uniforms).  samples_out (nullable):
 * float32 [n_centers][n_rot] per-triplet products.  Synchronises `stream`.
 */
int hermes_mc_workspace_size(size_t* bytes);
int hermes_interp(const float* grid, int J, const double* scaled_pos, int64_t n,
                  const double* phi, int n_phi, int phi_res, double dx, double dy,
                  double dz, double* out, void* workspace, size_t workspace_bytes,
                  void* stream);
int hermes_mc_triplets(const float* eps1, const float* eps2, const float* eps3, int J,
                       const double* centers, const double* center_w, int64_t n_centers,
                       const double* offsets, int n_rot, const double* phi, int n_phi,
                       int phi_res, double rho1, double* sum_out, float* samples_out,
                       void* workspace, size_t workspace_bytes, void* stream);

/* hermes_mc_sample: the same triplet product with ONE rotation per sampled
 * centre, for importance sampling of single triplets (the learned proposal
 * has no reference counterpart; each value is the reference's per-triplet
 * product n1 n2 n3 of utils/corr3pcf_kernels.py:66-140).  Sample k's centre
 * is pool[i] (pool: device [M][3] float64, grid units), i = idx[k] (device
 * int64, clamped to [0, M)) or uniform in [0, M) when idx is NULL.  Offsets
 * come from `offsets` [n][6] (device float64, grid units) or, when NULL, the
 * triangle (R1, R2, mu) (grid units) rotated by three uniforms as
 * generate_triangle_offsets (corr3pcf_kernels.py:21-63).  Random draws are
 * SplitMix64 of (seed, k), so results do not depend on the launch shape.
 * f_k = weights[k] (or 1) * n1 n2 n3; sums_out (host) = {sum f, sum f^2} in
 * float64.  Workspace: hermes_mc_workspace_size.  Synchronises `stream`. */
int hermes_mc_sample(const float* eps1, const float* eps2, const float* eps3, int J,
                     const double* pool, int64_t M, const int64_t* idx, const double* weights,
                     const double* offsets, int64_t n, double R1, double R2, double mu, uint64_t seed,
                     const double* phi, int n_phi, int phi_res, double* sums_out,
                     void* workspace, size_t workspace_bytes, void* stream);

/* The Monte Carlo gathers on fields in a brick layout (no counterpart in the
 * reference, whose fields are C order): hermes_field_to_bricks copies a
 * float32 [L^3] C-order field into 2 x 2 x 2 bricks of 32 bytes (one DRAM
 * sector; bricks in C order of the brick coordinates, the 8 cells of a
 * brick in (x, y, z) bit order), so a 27-point interpolation reads exactly 8
 * sectors instead of 9 rows of 1-2 sectors.  hermes_mc_triplets_bricks and
 * hermes_mc_sample_bricks take the same arguments as hermes_mc_triplets and
 * hermes_mc_sample with eps1..eps3 in that layout and return the same values
 * bit for bit (the same float32 products in the same order). */
int hermes_field_to_bricks(const float* field, int J, float* bricks, void* stream);
int hermes_mc_triplets_bricks(const float* eps1, const float* eps2, const float* eps3, int J,
                              const double* centers, const double* center_w, int64_t n_centers,
                              const double* offsets, int n_rot, const double* phi, int n_phi,
                              int phi_res, double rho1, double* sum_out, float* samples_out,
                              void* workspace, size_t workspace_bytes, void* stream);
int hermes_mc_sample_bricks(const float* eps1, const float* eps2, const float* eps3, int J,
                            const double* pool, int64_t M, const int64_t* idx, const double* weights,
                            const double* offsets, int64_t n, double R1, double R2, double mu,
                            uint64_t seed, const double* phi, int n_phi, int phi_res,
                            double* sums_out, void* workspace, size_t workspace_bytes, void* stream);

/* ---- learned proposal network (no reference counterpart) ---------------------
 * A tanh MLP with dims[0] inputs, dims[n_layers] outputs, widths <= 128:
 * params = per layer W [in][out] then b [out] (float32).  forward writes
 * every layer's output into acts (sum_l batch*dims[l+1] floats) and reads
 * params or, for inference, a bfloat16 copy (params_bf16, from
 * hermes_to_bf16).  backward: grads (same layout) of sum(dy * y) through the
 * network; scratch: hermes_mlp_scratch_floats(batch) floats.  mse_grad:
 * dy = 2 (y - target)/n and the mean squared error (host float64; scratch:
 * one device double; synchronises).  adam_step: one Adam update (step >= 1). */
int hermes_mlp_param_count(const int32_t* dims, int n_layers, int64_t* n_params);
int hermes_mlp_scratch_floats(int64_t batch, int64_t* n);
int hermes_mlp_forward(const float* params, const void* params_bf16, const int32_t* dims,
                       int n_layers, const float* x, int64_t batch, float* acts,
                       void* stream);
int hermes_mlp_backward(const float* params, const int32_t* dims, int n_layers,
                        const float* x, int64_t batch, const float* acts, const float* dy,
                        float* grads, float* scratch, void* stream);
int hermes_mse_grad(const float* y, const float* target, int64_t n, float* dy,
                    double* loss_out, double* scratch, void* stream);
/* hermes_poisson_grad: as mse_grad for the Poisson deviance of log-mean
 * predictions y against non-negative targets: loss = mean(exp(y) - t y),
 * dy = (exp(y) - t) / n (minimised by y = log E[t | input]). */
int hermes_poisson_grad(const float* y, const float* target, int64_t n, float* dy,
                        double* loss_out, double* scratch, void* stream);
int hermes_adam_step(float* params, const float* grads, float* m, float* v, int64_t n,
                     float lr, float b1, float b2, float eps, int step, void* stream);
int hermes_to_bf16(const float* in, int64_t n, void* out, void* stream);
/* hermes_mlp_infer_tc: the network's output y [batch] for inputs x
 * [batch][dims[0]] with the 128 x 128 hidden layers on the tcgen05 tensor
 * cores (BF16 weights and activations, FP32 accumulation), for networks
 * dims = (d0 <= 16, 128, ..., 128, 1) with 1..4 hidden 128 x 128 layers
 * (HERMES_ERR_UNSUPPORTED otherwise).  params: the float32 layout above.
 * status: one device int, 0 on return of the kernel or 1 when a bounded
 * wait gave up (y is then incomplete).  Asynchronous on `stream`. */
int hermes_mlp_infer_tc(const float* params, const int32_t* dims, int n_layers, const float* x,
                        int64_t batch, float* y, int* status, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* HERMES_GB300_H */
