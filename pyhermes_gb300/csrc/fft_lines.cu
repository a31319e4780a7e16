// Inverse 512-point FFTs along the strided axes of complex64 fields
// [nf][512][512][512] (x, y, z; z contiguous), in place, unnormalised
// (a[k] <- sum_n a[n] e^{+2 pi i n k / 512}, cuFFT's CUFFT_INVERSE).
//
// The multipole fields' inverse 3-D transform (15 fields of 512^3 at J=9)
// spends two thirds of its time in cuFFT's two strided passes, which move
// their 30 GB each at about half of HBM bandwidth.  Here a CTA owns 16
// adjacent z columns of one (field, other-axis) slab and the 512 elements
// of the transformed axis: every row it reads or writes is 128 contiguous
// bytes, each element is read and written once, and the transform runs in
// shared memory as three radix-8 stages
// (512 = 8 * 8 * 8; n = n1 + 64 n2, k = k2 + 8 k1 with the 64-point part
// split the same way), twiddles from a float64 table per CTA.
#include "hermes_common.cuh"

namespace hermes {
namespace {

constexpr int kLen = 512;
constexpr int kPitch = kLen + 1;  // float2 per column in shared memory (odd: conflict-free columns)

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// a[k] <- sum_n a[n] e^{+2 pi i n k / 8}: two 4-point transforms of the
// even and odd inputs, combined with e^{+i pi k / 4}.
__device__ __forceinline__ void idft8(float2 (&a)[8]) {
  constexpr float r = 0.70710678118654752f;  // 1/sqrt(2)
  const float2 b0 = make_float2(a[0].x + a[4].x, a[0].y + a[4].y), b1 = make_float2(a[0].x - a[4].x, a[0].y - a[4].y);
  const float2 b2 = make_float2(a[2].x + a[6].x, a[2].y + a[6].y), b3 = make_float2(a[2].x - a[6].x, a[2].y - a[6].y);
  const float2 b4 = make_float2(a[1].x + a[5].x, a[1].y + a[5].y), b5 = make_float2(a[1].x - a[5].x, a[1].y - a[5].y);
  const float2 b6 = make_float2(a[3].x + a[7].x, a[3].y + a[7].y), b7 = make_float2(a[3].x - a[7].x, a[3].y - a[7].y);
  // even part E[k] and odd part O[k], k = 0..3 (i b = (-b.y, b.x))
  const float2 e0 = make_float2(b0.x + b2.x, b0.y + b2.y), e2 = make_float2(b0.x - b2.x, b0.y - b2.y);
  const float2 e1 = make_float2(b1.x - b3.y, b1.y + b3.x), e3 = make_float2(b1.x + b3.y, b1.y - b3.x);
  const float2 o0 = make_float2(b4.x + b6.x, b4.y + b6.y), o2 = make_float2(b4.x - b6.x, b4.y - b6.y);
  const float2 o1 = make_float2(b5.x - b7.y, b5.y + b7.x), o3 = make_float2(b5.x + b7.y, b5.y - b7.x);
  // w^k O[k], w = e^{+i pi / 4}
  const float2 t1 = make_float2((o1.x - o1.y) * r, (o1.x + o1.y) * r);
  const float2 t2 = make_float2(-o2.y, o2.x);
  const float2 t3 = make_float2(-(o3.x + o3.y) * r, (o3.x - o3.y) * r);
  a[0] = make_float2(e0.x + o0.x, e0.y + o0.y);
  a[4] = make_float2(e0.x - o0.x, e0.y - o0.y);
  a[1] = make_float2(e1.x + t1.x, e1.y + t1.y);
  a[5] = make_float2(e1.x - t1.x, e1.y - t1.y);
  a[2] = make_float2(e2.x + t2.x, e2.y + t2.y);
  a[6] = make_float2(e2.x - t2.x, e2.y - t2.y);
  a[3] = make_float2(e3.x + t3.x, e3.y + t3.y);
  a[7] = make_float2(e3.x - t3.x, e3.y - t3.y);
}

// 16-byte asynchronous global -> shared copy (L2 only) and its group fences
__device__ __forceinline__ void cp_async16_cg(void* dst, const void* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait_group() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// One CTA per SM, 512 threads, persistent over tiles (field f, other-axis
// index a, z block zb of C = 16 columns).  A ring of three shared buffers
// of 16 x 513 float2 keeps the two tiles after the current one in flight
// by cp.async (the tile loads overlap the transform: with direct loads the
// pass waited on memory and reached about half of HBM bandwidth).  A tile
// lands row-major ([row][16], 128 B rows in the order of its global rows);
// stage 1 reads it into registers and, after a barrier, writes its output
// column-major (odd pitch: conflict-free columns) into the same buffer.
// Each thread runs R = 2 eight-point transforms per stage; task i = tid +
// 512 r has column c = i % 16, so a half warp covers the 16 columns of one
// row (coalesced global rows, one bank pair per lane in shared memory).
//   stage 1 (c, n1):      x[n1 + 64 n2], n2 = 0..7 -> Y[n1][k2] e^{2 pi i n1 k2 / 512}
//   stage 2 (c, k2, m1):  Y[m1 + 8 m2][k2], m2 = 0..7 -> W[k2][m1][q2] e^{2 pi i m1 q2 / 64}
//   stage 3 (c, k2, q2):  W[k2][m1][q2], m1 = 0..7 -> X[k2 + 8 q2 + 64 q1]
constexpr int kCols = 16, kThreads = 512, kR = kCols * kLen / 8 / kThreads;
__global__ void __launch_bounds__(kThreads, 1)
fft512_cols_kernel(float2* __restrict__ data, int nf, int axis) {
  constexpr int C = kCols, T = kThreads, R = kR, kBuf = C * kPitch;
  extern __shared__ __align__(16) float2 sm[];
  float2* tw = sm + 3 * kBuf;
  for (int j = threadIdx.x; j < kLen; j += T) {
    double sn, cs;
    sincospi((double)j / 256.0, &sn, &cs);
    tw[j] = make_float2((float)cs, (float)sn);
  }
  const long long L = kLen, L2 = L * L, L3 = L2 * L;
  const long long astride = axis == 1 ? L2 : L;
  const long long rstride = axis == 1 ? L : L2;
  const long long ntiles = (long long)nf * L * (L / C);
  auto tile_ptr = [&](long long t) {
    const int zb = (int)(t % (L / C));
    const long long fa = t / (L / C);
    return data + (fa / L) * L3 + (fa % L) * astride + (long long)zb * C;
  };
  // tile t -> buffer (row-major), 4096 16-byte pieces, 8 per 128-byte row
  auto prefetch = [&](long long t, float2* buf) {
    if (t < ntiles) {
      const float2* g = tile_ptr(t);
#pragma unroll
      for (int q = 0; q < 4096 / T; ++q) {
        const int j = threadIdx.x + T * q, row = j >> 3, part = j & 7;
        cp_async16_cg(buf + row * C + 2 * part, g + (long long)row * rstride + 2 * part);
      }
    }
    cp_async_commit();  // an empty group past the end keeps the group count uniform
  };
  long long t = blockIdx.x;
  prefetch(t, sm);
  prefetch(t + gridDim.x, sm + kBuf);
  for (int k = 0; t < ntiles; t += gridDim.x, ++k) {
    float2* buf = sm + (k % 3) * kBuf;
    prefetch(t + 2LL * gridDim.x, sm + ((k + 2) % 3) * kBuf);
    cp_async_wait_group<2>();  // this tile's group is complete (two newer may be in flight)
    __syncthreads();
    float2 v[R][8];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int i = threadIdx.x + T * r, c = i % C, n1 = i / C;
#pragma unroll
      for (int n2 = 0; n2 < 8; ++n2) v[r][n2] = buf[(n1 + 64 * n2) * C + c];
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int i = threadIdx.x + T * r, c = i % C, n1 = i / C;
      idft8(v[r]);
      float2* s = buf + c * kPitch + n1 * 8;
      s[0] = v[r][0];
#pragma unroll
      for (int k2 = 1; k2 < 8; ++k2) s[k2] = cmul(v[r][k2], tw[n1 * k2]);
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int i = threadIdx.x + T * r, c = i % C, rest = i / C, k2 = rest & 7, m1 = rest >> 3;
      const float2* s = buf + c * kPitch + m1 * 8 + k2;
#pragma unroll
      for (int m2 = 0; m2 < 8; ++m2) v[r][m2] = s[64 * m2];
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int i = threadIdx.x + T * r, c = i % C, rest = i / C, k2 = rest & 7, m1 = rest >> 3;
      idft8(v[r]);
      float2* s = buf + c * kPitch + k2 * 64 + m1 * 8;
      s[0] = v[r][0];
#pragma unroll
      for (int q2 = 1; q2 < 8; ++q2) s[q2] = cmul(v[r][q2], tw[8 * m1 * q2]);
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int i = threadIdx.x + T * r, c = i % C, rest = i / C, k2 = rest & 7, q2 = rest >> 3;
      const float2* s = buf + c * kPitch + k2 * 64 + q2;
#pragma unroll
      for (int m1 = 0; m1 < 8; ++m1) v[r][m1] = s[8 * m1];
    }
    __syncthreads();  // buffer free: the next iteration prefetches into it
    float2* g = tile_ptr(t);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int i = threadIdx.x + T * r, c = i % C, rest = i / C, k2 = rest & 7, q2 = rest >> 3;
      idft8(v[r]);
      float2* gp = g + (long long)(k2 + 8 * q2) * rstride + c;
#pragma unroll
      for (int q1 = 0; q1 < 8; ++q1) gp[(long long)(64 * q1) * rstride] = v[r][q1];
    }
  }
  cp_async_wait_group<0>();  // no copy outlives the kernel
}

}  // namespace

// axis 0: x (element stride 512^2), axis 1: y (stride 512).
int fft512_strided_inverse(float2* data, int nf, int axis, cudaStream_t s) {
  constexpr size_t smem = sizeof(float2) * (3 * kCols * (size_t)kPitch + kLen);
  static bool attr_set[64] = {false};
  int dev = 0;
  HERMES_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64 || !attr_set[dev]) {  // once per device, before any stream capture
    HERMES_CUDA_TRY(cudaFuncSetAttribute(fft512_cols_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (dev >= 0 && dev < 64) attr_set[dev] = true;
  }
  int nsm = 0;
  HERMES_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const long long ntiles = (long long)nf * kLen * (kLen / kCols);
  long long grid = nsm;
  if (grid > ntiles) grid = ntiles;
  fft512_cols_kernel<<<(int)grid, kThreads, smem, s>>>(data, nf, axis);
  HERMES_LAUNCH_CHECK("fft512_cols_kernel");
  return HERMES_OK;
}


}  // namespace hermes

extern "C" int hermes_fft512_strided_inverse(void* data, int nfields, int axis, void* stream) {
  if (!data) return hermes::fail(HERMES_ERR_INVALID, "fft512_strided_inverse: data is NULL");
  if (nfields < 1 || nfields > 64)
    return hermes::fail(HERMES_ERR_INVALID, "fft512_strided_inverse: nfields=%d outside [1, 64]", nfields);
  if (axis != 0 && axis != 1)
    return hermes::fail(HERMES_ERR_INVALID, "fft512_strided_inverse: axis=%d must be 0 (x) or 1 (y)", axis);
  return hermes::fft512_strided_inverse(static_cast<float2*>(data), nfields, axis, hermes::as_stream(stream));
}
