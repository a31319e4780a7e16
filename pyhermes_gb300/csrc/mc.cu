// Monte Carlo 3PCF on the GPU: field interpolation at points and triplet
// products over (centre, rotation) pairs.
//
// Restates pyhermes/utils/wavelet_grid.py:143-186 (interpolate_grid_at_pos:
// the 27-point phi-weighted gather) and pyhermes/utils/corr3pcf_kernels.py:
// 66-140 (estimate_triplet_product_{particle,box_random}_centers).  The
// reference draws three uniforms per rotation from a re-seeded MT19937 and
// builds the two triangle offsets on the host (generate_triangle_offsets,
// :21-63); the offsets are tiny (n_rot x 6 doubles) and are passed in, so the
// GPU sums exactly the same (centre, offset) pairs.  One thread per centre
// loads the centre once, gathers n1 once and loops over the rotations;
// products are float32, sums float64 with a fixed-order block reduction.
#include "hermes_common.cuh"

namespace {

using hermes::fail;

// Cell and fraction index of a scaled coordinate exactly as the reference:
// c = floor(s), f = int((s - c) * res) in float64.
__device__ __forceinline__ void mc_axis(double s, int res, int L, int& c, int& f) {
  const double fl = floor(s);
  c = ((int)fl) & (L - 1);
  int fi = (int)__dmul_rn(__dsub_rn(s, fl), (double)res);
  f = fi < 0 ? 0 : (fi >= res ? res - 1 : fi);
}

// Index of cell (x, y, z) of an L^3 field: C order (z fastest), or the brick
// layout of hermes_field_to_bricks: 2 x 2 x 2 bricks of 32 bytes (one DRAM
// sector) in C order of the brick coordinates, the 8 cells of a brick in
// (x, y, z) bit order.  A 3 x 3 x 3 stencil then touches exactly 8 sectors,
// against 9 rows of 1-2 sectors each in C order.
template <bool kBricks>
__device__ __forceinline__ size_t mc_cell(int x, int y, int z, int J) {
  if (!kBricks) return (((size_t)x << J) + y) << J | (size_t)z;
  const int h = J - 1;
  const size_t brick = ((((size_t)(x >> 1) << h) + (y >> 1)) << h) + (z >> 1);
  return brick << 3 | (size_t)((x & 1) << 2 | (y & 1) << 1 | (z & 1));
}

// 27-point interpolation of a float32 field at scaled position (sx, sy, sz).
template <bool kBricks = false>
__device__ __forceinline__ float mc_interp(const float* __restrict__ grid, const float* __restrict__ phis, int res,
                                           int J, double sx, double sy, double sz) {
  const int L = 1 << J;
  int cx, cy, cz, fx, fy, fz;
  mc_axis(sx, res, L, cx, fx);
  mc_axis(sy, res, L, cy, fy);
  mc_axis(sz, res, L, cz, fz);
  const int m = L - 1;
  float acc = 0.f;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int xg = (cx - a) & m;
    const float px = phis[fx + a * res];
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      const int yg = (cy - b) & m;
      const float py = phis[fy + b * res];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int zg = (cz - c) & m;
        acc += __ldg(grid + mc_cell<kBricks>(xg, yg, zg, J)) * px * py * phis[fz + c * res];
      }
    }
  }
  return acc;
}

__global__ void mc_phi_kernel(const double* __restrict__ phi, int n, float* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = (float)phi[i];
}

__global__ void mc_interp_kernel(const float* __restrict__ grid, int J, const double* __restrict__ pos, int64_t n,
                                 const float* __restrict__ phis, int res, double dx, double dy, double dz,
                                 double* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (double)mc_interp(grid, phis, res, J, pos[3 * i] + dx, pos[3 * i + 1] + dy, pos[3 * i + 2] + dz);
}

// sum_i w_i n1_i sum_r n2(x_i + d2_r) n3(x_i + d3_r); n1 = eps1 interpolated
// (box-random centres) or rho1 (particle centres: eps1 == NULL).  When
// samples != NULL also writes the per-(centre, rotation) products f_ir.
// kBricks: the fields are in the brick layout (mc_cell).
template <bool kBricks>
__global__ void __launch_bounds__(256)
mc_triplet_kernel(const float* __restrict__ eps1, const float* __restrict__ eps2, const float* __restrict__ eps3,
                  int J, const double* __restrict__ centers, const double* __restrict__ cw, int64_t nc,
                  const double* __restrict__ offsets, int n_rot, const float* __restrict__ phis, int res,
                  double rho1, double* __restrict__ partial, float* __restrict__ samples) {
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += (int64_t)gridDim.x * blockDim.x) {
    const double x = centers[3 * i], y = centers[3 * i + 1], z = centers[3 * i + 2];
    const float n1 = eps1 ? mc_interp<kBricks>(eps1, phis, res, J, x, y, z) : (float)rho1;
    const float w = cw ? (float)cw[i] : 1.f;
    float s = 0.f;
    for (int r = 0; r < n_rot; ++r) {
      const double* o = offsets + 6 * r;
      const float n2 = mc_interp<kBricks>(eps2, phis, res, J, x + o[0], y + o[1], z + o[2]);
      const float n3 = mc_interp<kBricks>(eps3, phis, res, J, x + o[3], y + o[4], z + o[5]);
      const float f = w * n1 * n2 * n3;
      if (samples) samples[i * n_rot + r] = f;
      s += f;
    }
    acc += (double)s;
  }
  __shared__ double sh[256];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void mc_sum_kernel(const double* __restrict__ partial, int n, double* __restrict__ out) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += partial[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

// SplitMix64 (Steele, Lea and Flood, 2014): a counter-based generator, so a
// sample's draws depend only on (seed, sample index) and not on the launch.
__device__ __forceinline__ unsigned long long mc_splitmix(unsigned long long& s) {
  unsigned long long z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double mc_u01(unsigned long long& s) {
  return (double)(mc_splitmix(s) >> 11) * (1.0 / 9007199254740992.0);
}

// generate_triangle_offsets (corr3pcf_kernels.py:21-63) in float64 with the
// angles given as fractions of a turn: phi = 2 pi fp, alpha = 2 pi fa.
__device__ __forceinline__ void mc_triangle(double R1, double R2, double mu, double fp, double ct1, double fa,
                                            double o[6]) {
  const double st1 = sqrt(1.0 - ct1 * ct1);
  double sp, cp, sa, ca;
  sincospi(2.0 * fp, &sp, &cp);
  sincospi(2.0 * fa, &sa, &ca);
  const double dx1 = st1 * cp, dy1 = st1 * sp, dz1 = ct1;
  double ox1, oy1, oz1;
  if (fabs(dx1) > 1e-10 || fabs(dy1) > 1e-10) {
    ox1 = -dy1; oy1 = dx1; oz1 = 0.0;
  } else {
    ox1 = 0.0; oy1 = -dz1; oz1 = dy1;
  }
  const double nrm = sqrt(ox1 * ox1 + oy1 * oy1 + oz1 * oz1);
  ox1 /= nrm; oy1 /= nrm; oz1 /= nrm;
  const double ox2 = dy1 * oz1 - dz1 * oy1, oy2 = dz1 * ox1 - dx1 * oz1, oz2 = dx1 * oy1 - dy1 * ox1;
  double st2 = 1.0 - mu * mu;
  if (st2 < 0.0) st2 = 0.0;
  const double st = sqrt(st2);
  o[0] = R1 * dx1; o[1] = R1 * dy1; o[2] = R1 * dz1;
  o[3] = R2 * (mu * dx1 + st * (ca * ox1 + sa * ox2));
  o[4] = R2 * (mu * dy1 + st * (ca * oy1 + sa * oy2));
  o[5] = R2 * (mu * dz1 + st * (ca * oz1 + sa * oz2));
}

// One triplet per sample k: centre c = pool[i], i = idx[k] (clamped to
// [0, M)) or uniform in [0, M) when idx == NULL; offsets from `offsets`
// [n][6] or drawn (phi, cos theta1, alpha uniform, as the reference's three
// uniforms); value f_k = w_k n1(c) n2(c + o1) n3(c + o2) (w_k = 1 when w is
// NULL).  Block partial sums of f and f^2.
template <bool kBricks>
__global__ void __launch_bounds__(256)
mc_sample_kernel(const float* __restrict__ eps1, const float* __restrict__ eps2, const float* __restrict__ eps3,
                 int J, const double* __restrict__ pool, long long M, const long long* __restrict__ idx,
                 const double* __restrict__ w, const double* __restrict__ offsets, long long n, double R1, double R2,
                 double mu,
                 unsigned long long seed, const float* __restrict__ phis, int res, double* __restrict__ partial) {
  double acc = 0.0, acc2 = 0.0;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    unsigned long long st = seed ^ ((unsigned long long)k * 0xD1B54A32D192ED03ull);
    long long i;
    if (idx) {
      i = idx[k];
      i = i < 0 ? 0 : (i >= M ? M - 1 : i);  // indices outside the pool are clamped, never read past it
    } else {
      i = (long long)(mc_u01(st) * (double)M);
      if (i >= M) i = M - 1;
    }
    double o[6];
    if (offsets) {
#pragma unroll
      for (int q = 0; q < 6; ++q) o[q] = offsets[6 * k + q];
    } else {
      const double a = mc_u01(st), bb = mc_u01(st), c = mc_u01(st);
      mc_triangle(R1, R2, mu, a, 2.0 * bb - 1.0, c, o);
    }
    const double x = pool[3 * i], y = pool[3 * i + 1], z = pool[3 * i + 2];
    const float n1 = mc_interp<kBricks>(eps1, phis, res, J, x, y, z);
    const float n2 = mc_interp<kBricks>(eps2, phis, res, J, x + o[0], y + o[1], z + o[2]);
    const float n3 = mc_interp<kBricks>(eps3, phis, res, J, x + o[3], y + o[4], z + o[5]);
    double f = (double)(n1 * n2 * n3);
    if (w) f *= w[k];
    acc += f;
    acc2 += f * f;
  }
  __shared__ double sh[2][256];
  sh[0][threadIdx.x] = acc;
  sh[1][threadIdx.x] = acc2;
  __syncthreads();
  for (int s2 = blockDim.x / 2; s2 > 0; s2 >>= 1) {
    if (threadIdx.x < s2) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + s2];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + s2];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partial[blockIdx.x] = sh[0][0];
    partial[gridDim.x + blockIdx.x] = sh[1][0];
  }
}

// dst[mc_cell<true>(x, y, z)] = src[mc_cell<false>(x, y, z)]: one thread per
// destination element, so the writes are contiguous; a warp's 32 reads are
// 4 bricks = 8 rows of 2 cells.
__global__ void mc_to_bricks_kernel(const float* __restrict__ src, int J, float* __restrict__ dst) {
  const size_t n = (size_t)1 << (3 * J);
  const int h = J - 1;
  const size_t hm = ((size_t)1 << h) - 1;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const size_t brick = i >> 3;
    const int c = (int)(i & 7);
    const int x = (int)(((brick >> (2 * h)) & hm) << 1) | (c >> 2);
    const int y = (int)(((brick >> h) & hm) << 1) | ((c >> 1) & 1);
    const int z = (int)((brick & hm) << 1) | (c & 1);
    dst[i] = __ldg(src + mc_cell<false>(x, y, z, J));
  }
}

int mc_grid() {
  int dev = 0, nsm = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  return nsm * 8;
}

}  // namespace

extern "C" int hermes_mc_workspace_size(size_t* bytes) {
  if (!bytes) return fail(HERMES_ERR_INVALID, "bytes is NULL");
  hermes::Carver c(nullptr, 0);
  c.take<float>(4 * 1024);
  c.take<double>(2 * ((size_t)mc_grid() + 1));
  *bytes = c.used;
  return HERMES_OK;
}

static int mc_prepare(const double* phi, int n_phi, int res, void* workspace, size_t workspace_bytes, float** phis,
                      double** partial, cudaStream_t s) {
  if (!phi || res <= 0 || n_phi != 3 * res || res > 1024)
    return fail(HERMES_ERR_INVALID, "mc: phi must hold 3*res samples with res <= 1024 (n_phi=%d, res=%d)", n_phi, res);
  size_t need = 0;
  hermes_mc_workspace_size(&need);
  if (!workspace || workspace_bytes < need) return fail(HERMES_ERR_WORKSPACE, "mc: workspace %zu < %zu", workspace_bytes, need);
  hermes::Carver c(workspace, workspace_bytes);
  *phis = c.take<float>(4 * 1024);
  *partial = c.take<double>(2 * ((size_t)mc_grid() + 1));
  mc_phi_kernel<<<4, 256, 0, s>>>(phi, n_phi, *phis);
  HERMES_LAUNCH_CHECK("mc_phi_kernel");
  return HERMES_OK;
}

extern "C" int hermes_interp(const float* grid, int J, const double* scaled_pos, int64_t n, const double* phi,
                             int n_phi, int phi_res, double dx, double dy, double dz, double* out, void* workspace,
                             size_t workspace_bytes, void* stream) {
  if (!grid || (n > 0 && (!scaled_pos || !out))) return fail(HERMES_ERR_INVALID, "interp: NULL argument");
  if (J < 2 || J > 10) return fail(HERMES_ERR_INVALID, "interp: J=%d outside [2,10]", J);
  cudaStream_t s = hermes::as_stream(stream);
  float* phis;
  double* partial;
  int rc = mc_prepare(phi, n_phi, phi_res, workspace, workspace_bytes, &phis, &partial, s);
  if (rc) return rc;
  if (n == 0) return HERMES_OK;
  mc_interp_kernel<<<mc_grid(), 256, 0, s>>>(grid, J, scaled_pos, n, phis, phi_res, dx, dy, dz, out);
  HERMES_LAUNCH_CHECK("mc_interp_kernel");
  return HERMES_OK;
}

static int mc_triplets(const float* eps1, const float* eps2, const float* eps3, int J, const double* centers,
                       const double* center_w, int64_t n_centers, const double* offsets, int n_rot, const double* phi,
                       int n_phi, int phi_res, double rho1, double* sum_out, float* samples_out, void* workspace,
                       size_t workspace_bytes, void* stream, bool bricks) {
  if (!eps2 || !eps3 || !sum_out || (n_centers > 0 && !centers) || (n_rot > 0 && !offsets))
    return fail(HERMES_ERR_INVALID, "mc_triplets: NULL argument");
  if (J < 2 || J > 10) return fail(HERMES_ERR_INVALID, "mc_triplets: J=%d outside [2,10]", J);
  if (n_rot < 0 || n_centers < 0) return fail(HERMES_ERR_INVALID, "mc_triplets: negative count");
  cudaStream_t s = hermes::as_stream(stream);
  float* phis;
  double* partial;
  int rc = mc_prepare(phi, n_phi, phi_res, workspace, workspace_bytes, &phis, &partial, s);
  if (rc) return rc;
  const int g = mc_grid();
  if (bricks)
    mc_triplet_kernel<true><<<g, 256, 0, s>>>(eps1, eps2, eps3, J, centers, center_w, n_centers, offsets, n_rot, phis,
                                              phi_res, rho1, partial, samples_out);
  else
    mc_triplet_kernel<false><<<g, 256, 0, s>>>(eps1, eps2, eps3, J, centers, center_w, n_centers, offsets, n_rot,
                                               phis, phi_res, rho1, partial, samples_out);
  HERMES_LAUNCH_CHECK("mc_triplet_kernel");
  mc_sum_kernel<<<1, 256, 0, s>>>(partial, g, partial + g);
  HERMES_LAUNCH_CHECK("mc_sum_kernel");
  HERMES_CUDA_TRY(cudaMemcpyAsync(sum_out, partial + g, sizeof(double), cudaMemcpyDeviceToHost, s));
  HERMES_CUDA_TRY(cudaStreamSynchronize(s));
  return HERMES_OK;
}

static int mc_sample(const float* eps1, const float* eps2, const float* eps3, int J, const double* pool, int64_t M,
                     const int64_t* idx, const double* weights, const double* offsets, int64_t n, double R1, double R2,
                     double mu, uint64_t seed, const double* phi, int n_phi, int phi_res, double* sums_out,
                     void* workspace, size_t workspace_bytes, void* stream, bool bricks) {
  if (!eps1 || !eps2 || !eps3 || !sums_out) return fail(HERMES_ERR_INVALID, "mc_sample: NULL argument");
  if (J < 2 || J > 10) return fail(HERMES_ERR_INVALID, "mc_sample: J=%d outside [2,10]", J);
  if (n < 0 || M < 0) return fail(HERMES_ERR_INVALID, "mc_sample: negative count");
  if (n > 0 && (!pool || M == 0)) return fail(HERMES_ERR_INVALID, "mc_sample: empty centre pool");
  cudaStream_t s = hermes::as_stream(stream);
  float* phis;
  double* partial;
  int rc = mc_prepare(phi, n_phi, phi_res, workspace, workspace_bytes, &phis, &partial, s);
  if (rc) return rc;
  const int g = mc_grid();
  if (bricks)
    mc_sample_kernel<true><<<g, 256, 0, s>>>(eps1, eps2, eps3, J, pool, (long long)M,
                                             reinterpret_cast<const long long*>(idx), weights, offsets, (long long)n,
                                             R1, R2, mu, (unsigned long long)seed, phis, phi_res, partial);
  else
    mc_sample_kernel<false><<<g, 256, 0, s>>>(eps1, eps2, eps3, J, pool, (long long)M,
                                              reinterpret_cast<const long long*>(idx), weights, offsets, (long long)n,
                                              R1, R2, mu, (unsigned long long)seed, phis, phi_res, partial);
  HERMES_LAUNCH_CHECK("mc_sample_kernel");
  mc_sum_kernel<<<1, 256, 0, s>>>(partial, g, partial + 2 * g);
  HERMES_LAUNCH_CHECK("mc_sum_kernel");
  mc_sum_kernel<<<1, 256, 0, s>>>(partial + g, g, partial + 2 * g + 1);
  HERMES_LAUNCH_CHECK("mc_sum_kernel");
  HERMES_CUDA_TRY(cudaMemcpyAsync(sums_out, partial + 2 * g, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
  HERMES_CUDA_TRY(cudaStreamSynchronize(s));
  return HERMES_OK;
}

extern "C" int hermes_mc_triplets(const float* eps1, const float* eps2, const float* eps3, int J,
                                  const double* centers, const double* center_w, int64_t n_centers,
                                  const double* offsets, int n_rot, const double* phi, int n_phi, int phi_res,
                                  double rho1, double* sum_out, float* samples_out, void* workspace,
                                  size_t workspace_bytes, void* stream) {
  return mc_triplets(eps1, eps2, eps3, J, centers, center_w, n_centers, offsets, n_rot, phi, n_phi, phi_res, rho1,
                     sum_out, samples_out, workspace, workspace_bytes, stream, false);
}

extern "C" int hermes_mc_triplets_bricks(const float* eps1, const float* eps2, const float* eps3, int J,
                                         const double* centers, const double* center_w, int64_t n_centers,
                                         const double* offsets, int n_rot, const double* phi, int n_phi, int phi_res,
                                         double rho1, double* sum_out, float* samples_out, void* workspace,
                                         size_t workspace_bytes, void* stream) {
  return mc_triplets(eps1, eps2, eps3, J, centers, center_w, n_centers, offsets, n_rot, phi, n_phi, phi_res, rho1,
                     sum_out, samples_out, workspace, workspace_bytes, stream, true);
}

extern "C" int hermes_mc_sample(const float* eps1, const float* eps2, const float* eps3, int J, const double* pool,
                                int64_t M, const int64_t* idx, const double* weights, const double* offsets,
                                int64_t n, double R1, double R2, double mu, uint64_t seed, const double* phi,
                                int n_phi, int phi_res, double* sums_out, void* workspace, size_t workspace_bytes,
                                void* stream) {
  return mc_sample(eps1, eps2, eps3, J, pool, M, idx, weights, offsets, n, R1, R2, mu, seed, phi, n_phi, phi_res,
                   sums_out, workspace, workspace_bytes, stream, false);
}

extern "C" int hermes_mc_sample_bricks(const float* eps1, const float* eps2, const float* eps3, int J,
                                       const double* pool, int64_t M, const int64_t* idx, const double* weights,
                                       const double* offsets, int64_t n, double R1, double R2, double mu,
                                       uint64_t seed, const double* phi, int n_phi, int phi_res, double* sums_out,
                                       void* workspace, size_t workspace_bytes, void* stream) {
  return mc_sample(eps1, eps2, eps3, J, pool, M, idx, weights, offsets, n, R1, R2, mu, seed, phi, n_phi, phi_res,
                   sums_out, workspace, workspace_bytes, stream, true);
}

extern "C" int hermes_field_to_bricks(const float* field, int J, float* bricks, void* stream) {
  if (!field || !bricks) return fail(HERMES_ERR_INVALID, "field_to_bricks: NULL argument");
  if (J < 2 || J > 10) return fail(HERMES_ERR_INVALID, "field_to_bricks: J=%d outside [2,10]", J);
  if (field == bricks) return fail(HERMES_ERR_INVALID, "field_to_bricks: the copy cannot be in place");
  mc_to_bricks_kernel<<<mc_grid(), 256, 0, hermes::as_stream(stream)>>>(field, J, bricks);
  HERMES_LAUNCH_CHECK("mc_to_bricks_kernel");
  return HERMES_OK;
}
