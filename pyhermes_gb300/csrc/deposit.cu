// SFC deposit: particles -> scaling-function coefficients eps[L,L,L].
//
// Restates pyhermes/utils/wavelet_grid.py:17-55 (_project_scaling_grid_impl)
// for one GB300.  The reference walks particles sequentially and does 27
// float64 read-modify-writes per particle into the grid.  Here:
//
//   K0 dep_max_kernel     max|w| and max|phi| (order-independent bound)
//   K1 dep_bin_kernel     per particle: float64 cell/frac (bit-identical to the
//                         reference's floor/astype(int32)), packed 16-byte
//                         record, histogram over (home tile, region) buckets
//   K2 dep_scan_*         exclusive scan of the bucket histogram
//   K3 dep_scatter_kernel counting-sort scatter (warp-aggregated slots)
//   K4 dep_accum_kernel   one CTA per output tile: gathers the records of its
//                         own tile and of the <=7 upper-neighbour tiles whose
//                         support reaches it, accumulates each particle's
//                         27-cell stencil into shared-memory int64 fixed-point
//                         cells, then writes the tile once, coalesced.
//
// Each output cell is written exactly once (no zero-fill pass, no global
// atomics on the grid).  Integer accumulation is associative, so the result
// is bitwise independent of particle order and scheduling.  The region code
// of a record marks the axes along which its stencil crosses into the lower
// neighbour tile, so a CTA reads only records that reach it.
#include <math.h>

#include <atomic>
#include <mutex>

#include "hermes_common.cuh"

namespace {

constexpr int kMaxSupport = 4;
constexpr int kTileX = 8, kTileY = 16, kTileZ = 32;  // default tile (cells)
constexpr int kMaxTileCells = 16384;                  // 128 KB int64 + 64 KB counts of shared memory
constexpr int kMaxJ = 10;

// Tile shape per grid level J chosen by hermes_deposit_set_tile (0 = the
// default), packed as tx | ty << 8 | tz << 16 (each a power of two <= 128).
std::atomic<int> g_tile[kMaxJ + 1];

int pack_tile(int tx, int ty, int tz) { return tx | (ty << 8) | (tz << 16); }
constexpr int kAccThreads = 256;
constexpr int kScanChunk = 4096;  // elements per scan block (1024 threads x 4)
constexpr unsigned kRejected = 0xFFFFFFFFu;

struct __align__(16) DepRec {
  uint32_t cell;  // cx << 20 | cy << 10 | cz
  uint32_t frac;  // fx << 20 | fy << 10 | fz
  float w;
  uint32_t key;   // home_tile * 8 + region, or kRejected
};

struct DepGeom {
  int L, S, res;
  int res_log2;       // log2(res) when res is a power of two, else -1
  int tx_log2, ty_log2, tz_log2;
  int tx, ty, tz;     // tile extents (cells)
  int ntx, nty, ntz;  // tiles per axis
  double scale;       // L / box
};

struct DepStatus {
  unsigned long long rejected;  // non-finite or out-of-range particles
  unsigned int wmax_bits;       // max |w| (float, rounded up) as bits
  unsigned int phimax_bits;     // max |phi| (float, rounded up) as bits
  double scale_d;               // fixed-point scale (power of two)
  double inv_d;                 // 1 / scale_d
  float scale_f, inv_f;         // the same as float
};

__device__ __forceinline__ float warp_max(float v) {
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__global__ void dep_max_kernel(const double* __restrict__ w, int64_t n,
                               const double* __restrict__ phi, int n_phi,
                               DepStatus* st) {
  float m = 0.f, pm = 0.f;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    double v = fabs(w[i]);
    if (isfinite(v)) m = fmaxf(m, __double2float_ru(v));
  }
  if (blockIdx.x == 0) {
    for (int i = threadIdx.x; i < n_phi; i += blockDim.x)
      pm = fmaxf(pm, __double2float_ru(fabs(phi[i])));
  }
  m = warp_max(m);
  pm = warp_max(pm);
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&st->wmax_bits, __float_as_uint(m));
    atomicMax(&st->phimax_bits, __float_as_uint(pm));
  }
}

// float64 cell / fraction index of one coordinate, exactly as the reference:
// scaled = x * (L/box); c = floor(scaled); f = int((scaled - c) * res).
__device__ __forceinline__ bool dep_axis(double x, const DepGeom& g, int& c, int& f) {
  double s = __dmul_rn(x, g.scale);
  if (!(fabs(s) < 1073741824.0)) return false;
  double fl = floor(s);
  c = (int)fl;
  f = (int)__dmul_rn(__dsub_rn(s, fl), (double)g.res);
  if (f < 0) f = 0;
  if (f >= g.res) f = g.res - 1;
  c &= (g.L - 1);  // periodic wrap (matches the reference's negative-index wrap)
  return true;
}

// Same result as dep_axis for s = x*scale >= 0 and a power-of-two res, from
// the bits of s: the integer part and the top log2(res) fraction bits of the
// float64 mantissa are exactly floor(s) and int((s - floor(s)) * res).
// Only the multiply is float64 (GB300 float64 throughput is low).
__device__ __forceinline__ bool dep_axis_fast(double x, const DepGeom& g, int& c, int& f) {
  const double s = __dmul_rn(x, g.scale);
  const unsigned long long b = (unsigned long long)__double_as_longlong(s);
  if ((b >> 63) || g.res_log2 < 0) return dep_axis(x, g, c, f);
  const int ex = (int)(b >> 52);
  if (ex >= 1023 + 30) return false;  // >= 2^30, inf or nan
  const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (ex ? (1ull << 52) : 0ull);
  const int sh = ex ? 1075 - ex : 1074;  // s = m * 2^-sh, sh >= 23
  c = sh >= 64 ? 0 : (int)(m >> sh);
  const int t = sh - g.res_log2;
  f = t >= 64 ? 0 : (int)((m >> t) & (unsigned long long)(g.res - 1));
  c &= (g.L - 1);
  return true;
}

__device__ __forceinline__ unsigned dep_key(int cx, int cy, int cz, const DepGeom& g) {
  int hx = cx / g.tx, hy = cy / g.ty, hz = cz / g.tz;
  unsigned region = 0;
  if (g.ntx > 1 && (cx - hx * g.tx) < g.S - 1) region |= 1u;
  if (g.nty > 1 && (cy - hy * g.ty) < g.S - 1) region |= 2u;
  if (g.ntz > 1 && (cz - hz * g.tz) < g.S - 1) region |= 4u;
  unsigned tile = ((unsigned)hx * g.nty + hy) * g.ntz + hz;
  return tile * 8u + region;
}

// Warp-aggregated atomicAdd of 1 per lane on ctr[key]; returns each lane's
// slot.  All 32 lanes must call it; lanes with key == kRejected get nothing.
__device__ __forceinline__ unsigned warp_agg_slot(unsigned* ctr, unsigned key) {
  unsigned lane = threadIdx.x & 31;
  unsigned peers = __match_any_sync(0xffffffffu, key);
  int leader = __ffs(peers) - 1;
  unsigned rank = __popc(peers & ((1u << lane) - 1u));
  unsigned base = 0;
  if ((int)lane == leader && key != kRejected) base = atomicAdd(&ctr[key], (unsigned)__popc(peers));
  base = __shfl_sync(0xffffffffu, base, leader);
  return base + rank;
}

__global__ void dep_bin_kernel(const double* __restrict__ pos, const double* __restrict__ w,
                               int64_t n, DepGeom g, DepRec* __restrict__ rec,
                               unsigned* __restrict__ counts, DepStatus* st) {
  int64_t warp_stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += warp_stride) {
    int64_t i = base + threadIdx.x;
    unsigned key = kRejected;
    if (i < n) {
      double x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
      double wi = w[i];
      int cx, cy, cz, fx, fy, fz;
      bool ok = isfinite(x) && isfinite(y) && isfinite(z) && isfinite(wi) &&
                dep_axis_fast(x, g, cx, fx) && dep_axis_fast(y, g, cy, fy) && dep_axis_fast(z, g, cz, fz);
      DepRec r;
      if (ok) {
        key = dep_key(cx, cy, cz, g);
        r.cell = ((unsigned)cx << 20) | ((unsigned)cy << 10) | (unsigned)cz;
        r.frac = ((unsigned)fx << 20) | ((unsigned)fy << 10) | (unsigned)fz;
        r.w = (float)wi;
      } else {
        r.cell = 0;
        r.frac = 0;
        r.w = 0.f;
        atomicAdd(&st->rejected, 1ULL);
      }
      r.key = key;
      rec[i] = r;
    }
    warp_agg_slot(counts, key);
  }
}

// Scan phase 1: per-chunk sums.
__global__ void dep_scan_sums_kernel(const unsigned* __restrict__ counts, int nb,
                                     unsigned* __restrict__ chunk_sums) {
  __shared__ unsigned warp_tot[32];
  int beg = blockIdx.x * kScanChunk;
  unsigned s = 0;
  for (int k = 0; k < 4; ++k) {
    int i = beg + k * 1024 + threadIdx.x;
    if (i < nb) s += counts[i];
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) warp_tot[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    unsigned v = warp_tot[threadIdx.x];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) chunk_sums[blockIdx.x] = v;
  }
}

// Block-wide exclusive scan of one value per thread (1024 threads).
__device__ unsigned block_excl_scan_1024(unsigned v, unsigned* total) {
  __shared__ unsigned warp_part[32];
  unsigned lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned inc = v;
  for (int o = 1; o < 32; o <<= 1) {
    unsigned t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= (unsigned)o) inc += t;
  }
  if (lane == 31) warp_part[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    unsigned p = warp_part[lane];
    unsigned pinc = p;
    for (int o = 1; o < 32; o <<= 1) {
      unsigned t = __shfl_up_sync(0xffffffffu, pinc, o);
      if (lane >= (unsigned)o) pinc += t;
    }
    warp_part[lane] = pinc - p;  // exclusive warp prefix
    if (lane == 31) *total = pinc;
  }
  __syncthreads();
  unsigned r = warp_part[wid] + inc - v;
  __syncthreads();
  return r;
}

__device__ __forceinline__ double dep_fixed_scale(const DepStatus* st, int64_t n) {
  double wmax = (double)__uint_as_float(st->wmax_bits);
  double pmax = (double)__uint_as_float(st->phimax_bits);
  double bound = (double)n * wmax * pmax * pmax * pmax;
  int e = -60;
  if (bound > 0.0) {
    frexp(bound, &e);  // bound < 2^e
    if (e < -60) e = -60;
  }
  return ldexp(1.0, 62 - e);  // bound * scale < 2^62
}

// Scan phase 2: exclusive scan of chunk sums (single block, serial over
// groups of 1024).  Also fixes the fixed-point scale and the float32 copy of
// phi used by the accumulation.
__global__ void dep_scan_chunks_kernel(unsigned* chunk_sums, int nchunks, DepStatus* st, int64_t n,
                                       const double* __restrict__ phi, int n_phi,
                                       float* __restrict__ phi_f) {
  if (threadIdx.x == 0) {
    const double sc = dep_fixed_scale(st, n);
    st->scale_d = sc;
    st->inv_d = 1.0 / sc;
    st->scale_f = (float)sc;
    st->inv_f = (float)(1.0 / sc);
  }
  for (int i = threadIdx.x; i < n_phi; i += blockDim.x) phi_f[i] = __double2float_rn(phi[i]);
  __shared__ unsigned total;
  unsigned carry = 0;
  for (int beg = 0; beg < nchunks; beg += 1024) {
    int i = beg + threadIdx.x;
    unsigned v = i < nchunks ? chunk_sums[i] : 0u;
    unsigned ex = block_excl_scan_1024(v, &total);
    if (i < nchunks) chunk_sums[i] = carry + ex;
    carry += total;
    __syncthreads();
  }
}

// Scan phase 3: rescan each chunk with its prefix; writes offsets and the
// scatter cursor, and offsets[nb] = grand total.
__global__ void dep_scan_apply_kernel(const unsigned* __restrict__ counts, int nb,
                                      const unsigned* __restrict__ chunk_prefix,
                                      unsigned* __restrict__ offsets,
                                      unsigned* __restrict__ cursor) {
  __shared__ unsigned total;
  int beg = blockIdx.x * kScanChunk + threadIdx.x * 4;
  unsigned v[4];
  unsigned s = 0;
  for (int k = 0; k < 4; ++k) {
    v[k] = (beg + k < nb) ? counts[beg + k] : 0u;
    s += v[k];
  }
  unsigned ex = block_excl_scan_1024(s, &total) + chunk_prefix[blockIdx.x];
  for (int k = 0; k < 4; ++k) {
    if (beg + k < nb) {
      offsets[beg + k] = ex;
      cursor[beg + k] = ex;
    }
    ex += v[k];
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 1023) offsets[nb] = ex;
}

__global__ void dep_scatter_kernel(const DepRec* __restrict__ rec, int64_t n,
                                   unsigned* __restrict__ cursor,
                                   DepRec* __restrict__ sorted) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
    int64_t i = base + threadIdx.x;
    DepRec r;
    unsigned key = kRejected;
    if (i < n) {
      r = rec[i];
      key = r.key;
    }
    unsigned slot = warp_agg_slot(cursor, key);
    if (key != kRejected) sorted[slot] = r;
  }
}

// Round-to-nearest int64 of a float32 value |v| < 2^62 with integer ops only
// (float -> int64 conversion instructions are slow on this part).
__device__ __forceinline__ long long f32_to_ll_rn(float v) {
  const int b = __float_as_int(v);
  const int e = (b >> 23) & 0xFF;
  if (e == 0) return 0;  // zero / subnormal: below one quantum
  const long long m = (long long)((b & 0x7FFFFF) | 0x800000);
  long long q;
  if (e >= 150) {
    q = m << (e - 150);
  } else {
    const int sh = 150 - e;
    q = sh >= 25 ? 0 : ((m + (1LL << (sh - 1))) >> sh);
  }
  return b < 0 ? -q : q;
}

// int64 -> float32 via two 32-bit conversions (at most one rounding step
// beyond round-to-nearest; the result is a float32 field anyway).
__device__ __forceinline__ float ll_to_f32(long long a) {
  const float hi = (float)(int)(a >> 32);
  const float lo = (float)(unsigned)(a & 0xFFFFFFFFLL);
  return fmaf(hi, 4294967296.0f, lo);
}

// ll_to_f32(HI * 2^sb + LO) from the two words in 32-bit integer arithmetic
// (8 <= sb <= 31; LO is the unsigned sum of many parts, so any 32-bit
// value): HI * 2^sb has upper 32 bits HI >> (32 - sb) (arithmetic shift:
// floor division) and lower 32 bits HI << sb; adding LO to the lower word
// carries one into the upper word when the 32-bit sum wraps.  The two words
// are those of the int64 total, so the result is the same float bit for bit.
__device__ __forceinline__ float split_to_f32(int hi, unsigned lo, int sb) {
  const unsigned low = ((unsigned)hi << sb) + lo;
  const int up = (hi >> (32 - sb)) + (low < lo ? 1 : 0);
  return fmaf((float)up, 4294967296.0f, (float)low);
}

// The (hi, lo) words of q = f32_to_ll_rn(v) split at bit sb, for
// |q| < 2^(31 + sb), in 32-bit arithmetic: with a = |v|, qa = floor(a) +
// (a - floor(a) >= 1/2) is the same round-half-away magnitude (floor(a) and
// a - floor(a) are exact), hi_a = qa >> sb and lo_a = qa - hi_a 2^sb are
// exact in float32 (qa has at most 24 significant bits), and a negative q
// takes hi = -hi_a - (lo_a != 0), lo = 2^sb - lo_a (two's complement).
__device__ __forceinline__ void split_q(float v, float two_sb, float inv_two_sb, unsigned lo_one, int& hi,
                                        unsigned& lo) {
  const float a = fabsf(v);
  const float fl = floorf(a);
  const float qa = (a - fl >= 0.5f) ? fl + 1.0f : fl;
  const int ha = __float2int_rz(qa * inv_two_sb);
  const unsigned la = __float2uint_rz(fmaf(-(float)ha, two_sb, qa));
  if (v < 0.f) {
    hi = -ha - (la != 0u ? 1 : 0);
    lo = la != 0u ? lo_one - la : 0u;
  } else {
    hi = ha;
    lo = la;
  }
}

// The split point sb of the two-word accumulation for a tile reached by T
// records (0: int64 atomics), see dep_accum_kernel.
__device__ __forceinline__ int split_bits(unsigned total, const DepStatus* __restrict__ st) {
  const int clog = total > 1u ? 32 - __clz((int)(total - 1u)) : 0;  // ceil(log2 T)
  const int cand = 32 - clog;
  if (cand < 8 || cand > 31) return 0;
  const double pm = (double)__uint_as_float(st->phimax_bits);
  const double qmax = (double)__uint_as_float(st->wmax_bits) * pm * pm * pm * st->scale_d;
  // factor 2 margin for the float32 rounding of each product
  return (double)total * (2.0 * ldexp(qmax, -cand) + 1.0) < 2147483648.0 ? cand : 0;
}

template <int S, bool kF64Out>
__global__ void __launch_bounds__(kAccThreads, 5)
dep_accum_kernel(const DepRec* __restrict__ sorted, const unsigned* __restrict__ offsets,
                 const float* __restrict__ phif, DepGeom g,
                 const DepStatus* __restrict__ st, float* __restrict__ out32,
                 double* __restrict__ out64, unsigned* __restrict__ counts_out) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int ncell = g.tx * g.ty * g.tz;
  long long* acc = reinterpret_cast<long long*>(smem);
  unsigned* cnt = reinterpret_cast<unsigned*>(acc + ncell);
  __shared__ unsigned r_start[64], r_pref[65], r_home[64];
  __shared__ int n_ranges, s_sb;

  const int tile = blockIdx.x;
  const int hz = tile % g.ntz, hy = (tile / g.ntz) % g.nty, hx = tile / (g.ntz * g.nty);
  const int x0 = hx * g.tx, y0 = hy * g.ty, z0 = hz * g.tz;
  const int tzl = g.tz_log2, tyzl = g.ty_log2 + g.tz_log2;

  // Zero the accumulators in every thread while warp 0 builds the range
  // table below (both before the first barrier; an empty tile then skips
  // shared memory when it writes).
  for (int i = 2 * threadIdx.x; i < ncell; i += 2 * blockDim.x) {
    *reinterpret_cast<longlong2*>(acc + i) = make_longlong2(0, 0);
    if (counts_out) *reinterpret_cast<uint2*>(cnt + i) = make_uint2(0u, 0u);
  }
  // Range table: warp 0 handles the 64 (neighbour d, region r) combinations,
  // two per lane, with independent loads, then compacts them with a ballot.
  if (threadIdx.x < 32) {
    const unsigned lane = threadIdx.x;
    unsigned len[2], st0[2], home[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int combo = 2 * (int)lane + h;
      const int d = combo >> 3;
      const unsigned r = (unsigned)(combo & 7), D = (unsigned)d;
      const int dx = d & 1, dy = (d >> 1) & 1, dz = (d >> 2) & 1;
      len[h] = 0;
      st0[h] = 0;
      home[h] = (d == 0);
      const bool ok = !((dx && g.ntx == 1) || (dy && g.nty == 1) || (dz && g.ntz == 1)) && ((r & D) == D);
      if (ok) {
        const int nx_ = (hx + dx) % g.ntx, ny_ = (hy + dy) % g.nty, nz_ = (hz + dz) % g.ntz;
        const unsigned b = (((unsigned)nx_ * g.nty + ny_) * g.ntz + nz_) * 8u + r;
        const unsigned s0 = offsets[b], s1 = offsets[b + 1];
        st0[h] = s0;
        len[h] = s1 - s0;
      }
    }
    // inclusive scan over the 64 lengths (lane order, two per lane)
    const unsigned pair_sum = len[0] + len[1];
    unsigned inc = pair_sum;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= (unsigned)o) inc += t;
    }
    const unsigned excl = inc - pair_sum;
    const unsigned v0 = __ballot_sync(0xffffffffu, len[0] > 0), v1 = __ballot_sync(0xffffffffu, len[1] > 0);
    const unsigned below = (1u << lane) - 1u;
    unsigned slot = __popc(v0 & below) + __popc(v1 & below);
    unsigned pref = excl;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if (len[h] > 0) {
        r_start[slot] = st0[h];
        r_pref[slot] = pref;
        r_home[slot] = home[h];
        ++slot;
      }
      pref += len[h];
    }
    if (lane == 31) {
      const int nr = __popc(v0) + __popc(v1);
      r_pref[nr] = inc;
      n_ranges = nr;
      s_sb = split_bits(inc, st);
    }
  }
  __syncthreads();
  const int nr = n_ranges;
  const unsigned total = r_pref[nr];

  if (total == 0) {  // empty tile: write zeros, skip shared memory
    for (int i = 4 * threadIdx.x; i < ncell; i += 4 * blockDim.x) {
      const int lz_ = i & (g.tz - 1), ly_ = (i >> tzl) & (g.ty - 1), lx_ = i >> tyzl;
      const size_t gi = ((size_t)(x0 + lx_) * g.L + (y0 + ly_)) * g.L + (z0 + lz_);
      if (kF64Out) {
        reinterpret_cast<double2*>(out64 + gi)[0] = make_double2(0.0, 0.0);
        reinterpret_cast<double2*>(out64 + gi)[1] = make_double2(0.0, 0.0);
      } else {
        *reinterpret_cast<float4*>(out32 + gi) = make_float4(0.f, 0.f, 0.f, 0.f);
      }
      if (counts_out) *reinterpret_cast<uint4*>(counts_out + gi) = make_uint4(0u, 0u, 0u, 0u);
    }
    return;
  }

  const float scale_f = st->scale_f;
  const int Lm = g.L - 1;
  // Split accumulation.  A 64-bit shared-memory atomic add costs about four
  // 32-bit ones on this part, so when the tile's sums allow it each int64
  // contribution q = hi * 2^sb + lo (0 <= lo < 2^sb, hi = q >> sb) goes into
  // two 32-bit words per cell: LO += lo (unsigned) and HI += hi (two's
  // complement).  With T records reaching the tile no cell gets more than T
  // contributions, so LO is exact when T * (2^sb - 1) < 2^32, and HI's final
  // value is exact (wrap-around addition is associative) when the true sum
  // of the hi parts fits in 31 bits: |sum hi| <= T * (qmax / 2^sb + 1), with
  // qmax = max|w| * max|phi|^3 * scale the largest |q|.  The cell total
  // HI * 2^sb + LO is then the same int64 as the plain path's, bit for bit.
  // Otherwise (dense tiles) sb = 0 and the tile uses int64 atomics.  The
  // same bound gives |q| / 2^sb < 2^31 for every contribution, which
  // split_q needs.
  const int sb = s_sb;  // chosen once per tile by the range-table warp (float64 is slow on this part)
  if (sb > 0) {
    unsigned* acc_lo = reinterpret_cast<unsigned*>(acc);
    int* acc_hi = reinterpret_cast<int*>(acc) + ncell;
    const float two_sb = ldexpf(1.0f, sb), inv_two_sb = ldexpf(1.0f, -sb);
    const unsigned lo_one = 1u << sb;
    for (unsigned k = threadIdx.x; k < total; k += blockDim.x) {
      int lo = 0, hi = nr - 1;  // largest r with r_pref[r] <= k
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (r_pref[mid] <= k) lo = mid; else hi = mid - 1;
      }
      const int r = lo;
      const DepRec rec = sorted[r_start[r] + (k - r_pref[r])];
      const int cx = rec.cell >> 20, cy = (rec.cell >> 10) & 1023, cz = rec.cell & 1023;
      const int fx = rec.frac >> 20, fy = (rec.frac >> 10) & 1023, fz = rec.frac & 1023;
      int lx[S], ly[S], lz[S];
      float px[S], py[S], pz[S];
#pragma unroll
      for (int s = 0; s < S; ++s) {
        lx[s] = (cx - s - x0) & Lm;
        ly[s] = (cy - s - y0) & Lm;
        lz[s] = (cz - s - z0) & Lm;
        px[s] = rec.w * __ldg(&phif[fx + g.res * s]);
        py[s] = __ldg(&phif[fy + g.res * s]);
        pz[s] = __ldg(&phif[fz + g.res * s]);
      }
      // every lane runs all S^3 terms and predicates the adds on the term's
      // cell lying in this tile (no divergent skips between the lanes'
      // particles)
#pragma unroll
      for (int a = 0; a < S; ++a) {
        const bool va = lx[a] < g.tx;
#pragma unroll
        for (int b = 0; b < S; ++b) {
          const bool vb = va && ly[b] < g.ty;
          const float pxy = px[a] * py[b];
          const int row = (lx[a] << tyzl) + (ly[b] << tzl);
#pragma unroll
          for (int c = 0; c < S; ++c) {
            const bool v = vb && lz[c] < g.tz;
            int qh;
            unsigned ql;
            split_q(pxy * pz[c] * scale_f, two_sb, inv_two_sb, lo_one, qh, ql);
            const int cell = row + lz[c];
            if (v && ql != 0u) atomicAdd(&acc_lo[cell], ql);
            if (v && qh != 0) atomicAdd(&acc_hi[cell], qh);
          }
        }
      }
      if (counts_out && r_home[r]) {
        atomicAdd(&cnt[((cx - x0) << tyzl) + ((cy - y0) << tzl) + (cz - z0)], 1u);
      }
    }
  } else
  for (unsigned k = threadIdx.x; k < total; k += blockDim.x) {
    int lo = 0, hi = nr - 1;  // largest r with r_pref[r] <= k
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (r_pref[mid] <= k) lo = mid; else hi = mid - 1;
    }
    const int r = lo;
    const DepRec rec = sorted[r_start[r] + (k - r_pref[r])];
    const int cx = rec.cell >> 20, cy = (rec.cell >> 10) & 1023, cz = rec.cell & 1023;
    const int fx = rec.frac >> 20, fy = (rec.frac >> 10) & 1023, fz = rec.frac & 1023;
    int lx[S], ly[S], lz[S];
    float px[S], py[S], pz[S];
#pragma unroll
    for (int s = 0; s < S; ++s) {
      lx[s] = (cx - s - x0) & Lm;
      ly[s] = (cy - s - y0) & Lm;
      lz[s] = (cz - s - z0) & Lm;
      px[s] = rec.w * __ldg(&phif[fx + g.res * s]);
      py[s] = __ldg(&phif[fy + g.res * s]);
      pz[s] = __ldg(&phif[fz + g.res * s]);
    }
#pragma unroll
    for (int a = 0; a < S; ++a) {
      const bool va = lx[a] < g.tx;
#pragma unroll
      for (int b = 0; b < S; ++b) {
        const bool vb = va && ly[b] < g.ty;
        const float pxy = px[a] * py[b];
        const int row = (lx[a] << tyzl) + (ly[b] << tzl);
#pragma unroll
        for (int c = 0; c < S; ++c) {
          const bool v = vb && lz[c] < g.tz;
          const long long q = f32_to_ll_rn(pxy * pz[c] * scale_f);
          if (v && q != 0)
            atomicAdd(reinterpret_cast<unsigned long long*>(&acc[row + lz[c]]), static_cast<unsigned long long>(q));
        }
      }
    }
    if (counts_out && r_home[r]) {
      atomicAdd(&cnt[((cx - x0) << tyzl) + ((cy - y0) << tzl) + (cz - z0)], 1u);
    }
  }
  __syncthreads();

  const float inv_f = st->inv_f;
  const double inv_d = st->inv_d;
  for (int i = 4 * threadIdx.x; i < ncell; i += 4 * blockDim.x) {
    const int lz_ = i & (g.tz - 1), ly_ = (i >> tzl) & (g.ty - 1), lx_ = i >> tyzl;
    const size_t gi = ((size_t)(x0 + lx_) * g.L + (y0 + ly_)) * g.L + (z0 + lz_);
    if (!kF64Out && sb > 0) {  // float32 field from the two words, no 64-bit arithmetic
      const uint4 l4 = *reinterpret_cast<const uint4*>(reinterpret_cast<const unsigned*>(acc) + i);
      const int4 h4 = *reinterpret_cast<const int4*>(reinterpret_cast<const int*>(acc) + ncell + i);
      *reinterpret_cast<float4*>(out32 + gi) =
          make_float4(split_to_f32(h4.x, l4.x, sb) * inv_f, split_to_f32(h4.y, l4.y, sb) * inv_f,
                      split_to_f32(h4.z, l4.z, sb) * inv_f, split_to_f32(h4.w, l4.w, sb) * inv_f);
      if (counts_out) *reinterpret_cast<uint4*>(counts_out + gi) = *reinterpret_cast<const uint4*>(cnt + i);
      continue;
    }
    longlong2 a01, a23;
    if (sb > 0) {  // cell total = HI * 2^sb + LO
      const uint4 l4 = *reinterpret_cast<const uint4*>(reinterpret_cast<const unsigned*>(acc) + i);
      const int4 h4 = *reinterpret_cast<const int4*>(reinterpret_cast<const int*>(acc) + ncell + i);
      const long long m = 1LL << sb;
      a01 = make_longlong2((long long)h4.x * m + l4.x, (long long)h4.y * m + l4.y);
      a23 = make_longlong2((long long)h4.z * m + l4.z, (long long)h4.w * m + l4.w);
    } else {
      a01 = *reinterpret_cast<const longlong2*>(acc + i);
      a23 = *reinterpret_cast<const longlong2*>(acc + i + 2);
    }
    if (kF64Out) {
      reinterpret_cast<double2*>(out64 + gi)[0] = make_double2((double)a01.x * inv_d, (double)a01.y * inv_d);
      reinterpret_cast<double2*>(out64 + gi)[1] = make_double2((double)a23.x * inv_d, (double)a23.y * inv_d);
    } else {
      *reinterpret_cast<float4*>(out32 + gi) =
          make_float4(ll_to_f32(a01.x) * inv_f, ll_to_f32(a01.y) * inv_f,
                      ll_to_f32(a23.x) * inv_f, ll_to_f32(a23.y) * inv_f);
    }
    if (counts_out) *reinterpret_cast<uint4*>(counts_out + gi) = *reinterpret_cast<const uint4*>(cnt + i);
  }
}

template <int S>
int dep_launch_accum(const DepRec* sorted, const unsigned* offsets, const float* phif,
                     const DepGeom& g, const DepStatus* st, float* eps_out,
                     double* eps_f64_out, unsigned* counts_out, int ntiles, size_t smem,
                     cudaStream_t s) {
  if (eps_f64_out) {
    HERMES_CUDA_TRY(cudaFuncSetAttribute(dep_accum_kernel<S, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dep_accum_kernel<S, true><<<ntiles, kAccThreads, smem, s>>>(sorted, offsets, phif, g, st,
                                                                nullptr, eps_f64_out, counts_out);
  } else {
    HERMES_CUDA_TRY(cudaFuncSetAttribute(dep_accum_kernel<S, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dep_accum_kernel<S, false><<<ntiles, kAccThreads, smem, s>>>(sorted, offsets, phif, g, st,
                                                                 eps_out, nullptr, counts_out);
  }
  return HERMES_OK;
}

struct DepPlan {
  DepGeom g;
  int nbuckets;
  int nchunks;
  size_t ws_bytes;
};

// tile: packed tile shape, 0 for the default.
int dep_plan(int64_t n, int J, int S, int res, DepPlan* p, int tile) {
  if (J < 2 || J > kMaxJ) return hermes::fail(HERMES_ERR_INVALID, "deposit: J=%d outside [2,%d]", J, kMaxJ);
  if (n < 0 || n > 0x7FFFFFFFLL) return hermes::fail(HERMES_ERR_INVALID, "deposit: n=%lld outside [0,2^31)", (long long)n);
  if (S < 1 || S > kMaxSupport) return hermes::fail(HERMES_ERR_INVALID, "deposit: phi support %d outside [1,%d]", S, kMaxSupport);
  if (res < 1 || res > 1024) return hermes::fail(HERMES_ERR_INVALID, "deposit: phi_res %d outside [1,1024]", res);
  DepGeom& g = p->g;
  g.L = 1 << J;
  g.S = S;
  g.res = res;
  const int tx = tile ? (tile & 0xFF) : kTileX, ty = tile ? ((tile >> 8) & 0xFF) : kTileY,
            tz = tile ? ((tile >> 16) & 0xFF) : kTileZ;
  g.tx = g.L < tx ? g.L : tx;
  g.ty = g.L < ty ? g.L : ty;
  g.tz = g.L < tz ? g.L : tz;
  if (S - 1 > g.tx) return hermes::fail(HERMES_ERR_INVALID, "deposit: grid too small for support");
  g.res_log2 = (res & (res - 1)) == 0 ? __builtin_ctz((unsigned)res) : -1;
  g.tx_log2 = __builtin_ctz((unsigned)g.tx);
  g.ty_log2 = __builtin_ctz((unsigned)g.ty);
  g.tz_log2 = __builtin_ctz((unsigned)g.tz);
  g.ntx = g.L / g.tx;
  g.nty = g.L / g.ty;
  g.ntz = g.L / g.tz;
  const int ntiles = g.ntx * g.nty * g.ntz;
  p->nbuckets = ntiles * 8;
  p->nchunks = (p->nbuckets + kScanChunk - 1) / kScanChunk;
  hermes::Carver c(nullptr, 0);
  c.take<DepStatus>(1);
  c.take<unsigned>(p->nbuckets);      // counts
  c.take<unsigned>(p->nbuckets + 1);  // offsets
  c.take<unsigned>(p->nbuckets);      // cursor
  c.take<unsigned>(p->nchunks);       // chunk sums
  c.take<float>(kMaxSupport * 1024);  // float32 phi
  c.take<DepRec>((size_t)(n > 0 ? n : 1));  // unsorted records
  c.take<DepRec>((size_t)(n > 0 ? n : 1));  // sorted records
  p->ws_bytes = c.used;
  return HERMES_OK;
}

// the tile set for level J (0: default)
int tile_for(int J) { return (J >= 0 && J <= kMaxJ) ? g_tile[J].load(std::memory_order_relaxed) : 0; }

int workspace_size(int64_t n, int J, int tile, size_t* bytes) {
  if (!bytes) return hermes::fail(HERMES_ERR_INVALID, "deposit: bytes is NULL");
  DepPlan p;
  int rc = dep_plan(n, J, 3, 1024, &p, tile);
  if (rc) return rc;
  *bytes = p.ws_bytes;
  return HERMES_OK;
}

}  // namespace

extern "C" int hermes_deposit_set_tile(int J, int tx, int ty, int tz) {
  if (J < 2 || J > kMaxJ) return hermes::fail(HERMES_ERR_INVALID, "deposit_set_tile: J=%d outside [2,%d]", J, kMaxJ);
  if (tx == 0 && ty == 0 && tz == 0) {
    g_tile[J].store(0);
    return HERMES_OK;
  }
  auto pow2 = [](int v) { return v > 0 && (v & (v - 1)) == 0; };
  if (!pow2(tx) || !pow2(ty) || !pow2(tz) || tx < kMaxSupport || ty < kMaxSupport || tz < 4 || tx > 128 ||
      ty > 128 || tz > 128 || tx * ty * tz > kMaxTileCells)
    return hermes::fail(HERMES_ERR_INVALID,
                        "deposit_set_tile: tile %dx%dx%d must be powers of two, x and y in [%d, 128], z in [4, 128], "
                        "at most %d cells", tx, ty, tz, kMaxSupport, kMaxTileCells);
  g_tile[J].store(pack_tile(tx, ty, tz));
  return HERMES_OK;
}

extern "C" int hermes_deposit_get_tile(int J, int* tx, int* ty, int* tz) {
  if (J < 2 || J > kMaxJ || !tx || !ty || !tz) return hermes::fail(HERMES_ERR_INVALID, "deposit_get_tile: bad argument");
  const int t = tile_for(J);
  const int L = 1 << J;
  const int x = t ? (t & 0xFF) : kTileX, y = t ? ((t >> 8) & 0xFF) : kTileY, z = t ? ((t >> 16) & 0xFF) : kTileZ;
  *tx = x < L ? x : L;
  *ty = y < L ? y : L;
  *tz = z < L ? z : L;
  return HERMES_OK;
}

extern "C" int hermes_deposit_workspace_size(int64_t n, int J, size_t* bytes) {
  return workspace_size(n, J, tile_for(J), bytes);
}

namespace {

struct DepBuffers {
  DepStatus* st;
  unsigned* counts;
  unsigned* offsets;
  unsigned* cursor;
  unsigned* chunk_sums;
  float* phif;
  DepRec* rec;
  DepRec* sorted;
};

int dep_prepare(int64_t n, int J, double box, int n_phi, int phi_res, const double* phi,
                void* workspace, size_t workspace_bytes, DepPlan* p, DepBuffers* b, int tile) {
  if (!(box > 0.0) || !isfinite(box)) return hermes::fail(HERMES_ERR_INVALID, "deposit: box must be finite and > 0");
  if (!phi || phi_res <= 0 || n_phi <= 0 || n_phi % phi_res)
    return hermes::fail(HERMES_ERR_INVALID, "deposit: n_phi=%d must be a positive multiple of phi_res=%d", n_phi, phi_res);
  int rc = dep_plan(n, J, n_phi / phi_res, phi_res, p, tile);
  if (rc) return rc;
  p->g.scale = (double)p->g.L / box;
  if (!workspace || workspace_bytes < p->ws_bytes)
    return hermes::fail(HERMES_ERR_WORKSPACE, "deposit: workspace %zu < required %zu", workspace_bytes, p->ws_bytes);
  hermes::Carver c(workspace, workspace_bytes);
  b->st = c.take<DepStatus>(1);
  b->counts = c.take<unsigned>(p->nbuckets);
  b->offsets = c.take<unsigned>(p->nbuckets + 1);
  b->cursor = c.take<unsigned>(p->nbuckets);
  b->chunk_sums = c.take<unsigned>(p->nchunks);
  b->phif = c.take<float>(kMaxSupport * 1024);
  b->rec = c.take<DepRec>((size_t)(n > 0 ? n : 1));
  b->sorted = c.take<DepRec>((size_t)(n > 0 ? n : 1));
  return HERMES_OK;
}

int deposit_sort(const double* pos, const double* w, int64_t n, int J, double box, const double* phi, int n_phi,
                 int phi_res, void* workspace, size_t workspace_bytes, void* stream, int tile) {
  if (n > 0 && (!pos || !w)) return hermes::fail(HERMES_ERR_INVALID, "deposit: pos/w NULL");
  DepPlan p;
  DepBuffers b;
  int rc = dep_prepare(n, J, box, n_phi, phi_res, phi, workspace, workspace_bytes, &p, &b, tile);
  if (rc) return rc;
  cudaStream_t s = hermes::as_stream(stream);
  HERMES_CUDA_TRY(cudaMemsetAsync(b.st, 0, sizeof(DepStatus), s));
  HERMES_CUDA_TRY(cudaMemsetAsync(b.counts, 0, sizeof(unsigned) * p.nbuckets, s));
  int dev = 0, nsm = 148;
  HERMES_CUDA_TRY(cudaGetDevice(&dev));
  HERMES_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int64_t want = (n + 255) / 256;
  const int grid_p = (int)(want < 1 ? 1 : (want < (int64_t)nsm * 8 ? want : (int64_t)nsm * 8));

  dep_max_kernel<<<grid_p, 256, 0, s>>>(w, n, phi, n_phi, b.st);
  HERMES_LAUNCH_CHECK("dep_max_kernel");
  if (n > 0) {
    dep_bin_kernel<<<grid_p, 256, 0, s>>>(pos, w, n, p.g, b.rec, b.counts, b.st);
    HERMES_LAUNCH_CHECK("dep_bin_kernel");
  }
  dep_scan_sums_kernel<<<p.nchunks, 1024, 0, s>>>(b.counts, p.nbuckets, b.chunk_sums);
  HERMES_LAUNCH_CHECK("dep_scan_sums_kernel");
  dep_scan_chunks_kernel<<<1, 1024, 0, s>>>(b.chunk_sums, p.nchunks, b.st, n, phi, n_phi, b.phif);
  HERMES_LAUNCH_CHECK("dep_scan_chunks_kernel");
  dep_scan_apply_kernel<<<p.nchunks, 1024, 0, s>>>(b.counts, p.nbuckets, b.chunk_sums, b.offsets, b.cursor);
  HERMES_LAUNCH_CHECK("dep_scan_apply_kernel");
  if (n > 0) {
    dep_scatter_kernel<<<grid_p, 256, 0, s>>>(b.rec, n, b.cursor, b.sorted);
    HERMES_LAUNCH_CHECK("dep_scatter_kernel");
  }
  return HERMES_OK;
}

int deposit_accumulate(int64_t n, int J, double box, const double* phi, int n_phi, int phi_res, float* eps_out,
                       double* eps_f64_out, uint32_t* counts_out, void* workspace, size_t workspace_bytes,
                       void* stream, int tile) {
  if ((eps_out == nullptr) == (eps_f64_out == nullptr))
    return hermes::fail(HERMES_ERR_INVALID, "deposit: give exactly one of eps_out / eps_f64_out");
  DepPlan p;
  DepBuffers b;
  int rc = dep_prepare(n, J, box, n_phi, phi_res, phi, workspace, workspace_bytes, &p, &b, tile);
  if (rc) return rc;
  cudaStream_t s = hermes::as_stream(stream);
  const int ncell = p.g.tx * p.g.ty * p.g.tz;
  const size_t smem = (size_t)ncell * 8 + (counts_out ? (size_t)ncell * 4 : 0);
  if (smem > 227 * 1024) return hermes::fail(HERMES_ERR_UNSUPPORTED, "deposit: shared memory %zu too large", smem);
  const int ntiles = p.g.ntx * p.g.nty * p.g.ntz;
  DepRec* sorted = b.sorted;
  unsigned* offsets = b.offsets;
  DepStatus* st = b.st;
  int lrc = HERMES_OK;
  switch (p.g.S) {
    case 1: lrc = dep_launch_accum<1>(sorted, offsets, b.phif, p.g, st, eps_out, eps_f64_out, counts_out, ntiles, smem, s); break;
    case 2: lrc = dep_launch_accum<2>(sorted, offsets, b.phif, p.g, st, eps_out, eps_f64_out, counts_out, ntiles, smem, s); break;
    case 3: lrc = dep_launch_accum<3>(sorted, offsets, b.phif, p.g, st, eps_out, eps_f64_out, counts_out, ntiles, smem, s); break;
    default: lrc = dep_launch_accum<4>(sorted, offsets, b.phif, p.g, st, eps_out, eps_f64_out, counts_out, ntiles, smem, s); break;
  }
  if (lrc) return lrc;
  HERMES_LAUNCH_CHECK("dep_accum_kernel");
  return HERMES_OK;
}

int deposit_full(const double* pos, const double* w, int64_t n, int J, double box, const double* phi, int n_phi,
                 int phi_res, float* eps_out, double* eps_f64_out, uint32_t* counts_out, void* workspace,
                 size_t workspace_bytes, void* stream, int tile) {
  if ((eps_out == nullptr) == (eps_f64_out == nullptr))
    return hermes::fail(HERMES_ERR_INVALID, "deposit: give exactly one of eps_out / eps_f64_out");
  int rc = deposit_sort(pos, w, n, J, box, phi, n_phi, phi_res, workspace, workspace_bytes, stream, tile);
  if (rc) return rc;
  return deposit_accumulate(n, J, box, phi, n_phi, phi_res, eps_out, eps_f64_out, counts_out, workspace,
                            workspace_bytes, stream, tile);
}

}  // namespace

extern "C" int hermes_deposit_sort(const double* pos, const double* w, int64_t n, int J,
                                   double box, const double* phi, int n_phi, int phi_res,
                                   void* workspace, size_t workspace_bytes, void* stream) {
  return deposit_sort(pos, w, n, J, box, phi, n_phi, phi_res, workspace, workspace_bytes, stream, tile_for(J));
}

extern "C" int hermes_deposit_accumulate(int64_t n, int J, double box, const double* phi,
                                         int n_phi, int phi_res, float* eps_out,
                                         double* eps_f64_out, uint32_t* counts_out,
                                         void* workspace, size_t workspace_bytes, void* stream) {
  return deposit_accumulate(n, J, box, phi, n_phi, phi_res, eps_out, eps_f64_out, counts_out, workspace,
                            workspace_bytes, stream, tile_for(J));
}

extern "C" int hermes_deposit(const double* pos, const double* w, int64_t n, int J,
                              double box, const double* phi, int n_phi, int phi_res,
                              float* eps_out, double* eps_f64_out, uint32_t* counts_out,
                              void* workspace, size_t workspace_bytes, void* stream) {
  return deposit_full(pos, w, n, J, box, phi, n_phi, phi_res, eps_out, eps_f64_out, counts_out, workspace,
                      workspace_bytes, stream, tile_for(J));
}

extern "C" int hermes_deposit_status(const void* workspace, int64_t* n_rejected, void* stream) {
  if (!workspace || !n_rejected) return hermes::fail(HERMES_ERR_INVALID, "deposit_status: NULL argument");
  DepStatus st;
  cudaStream_t s = hermes::as_stream(stream);
  HERMES_CUDA_TRY(cudaMemcpyAsync(&st, workspace, sizeof(st), cudaMemcpyDeviceToHost, s));
  HERMES_CUDA_TRY(cudaStreamSynchronize(s));
  *n_rejected = (int64_t)st.rejected;
  return HERMES_OK;
}

// ---- deposit without any device allocation ---------------------------------
// Some callers cannot allocate device memory at all: code that runs inside an
// allocator's own callbacks, plug-ins of hosts that own and budget every byte
// of HBM, or programs that must never hit an allocation failure mid-run.  For
// them hermes_deposit_noalloc runs the same deposit kernels with their scratch
// (the sort buckets and particle records that hermes_deposit takes from a
// caller workspace) in the fixed array below, compiled into this library.
//
// Limits: n <= kNoAllocMaxParticles and J <= kNoAllocMaxJ.  The array holds
// kNoAllocScratchBytes (4.5 MiB) on every GPU that loads the library, until
// the process exits.
constexpr int64_t kNoAllocMaxParticles = 131072;
constexpr int kNoAllocMaxJ = 8;
constexpr size_t kNoAllocScratchBytes = 4718592;
static __device__ __align__(256) unsigned char g_deposit_noalloc_scratch[kNoAllocScratchBytes];

namespace {
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kNoAllocMaxDevices] = {};

// Device address of the scratch array on the current device.  The array's
// name in host code is only a host-side stand-in, so the address is looked
// up once per device with cudaGetSymbolAddress and cached.
int noalloc_scratch(void** out) {
  int dev = 0;
  HERMES_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoAllocMaxDevices)
    return hermes::fail(HERMES_ERR_UNSUPPORTED, "deposit_noalloc: device %d beyond the supported %d", dev,
                        kNoAllocMaxDevices);
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_deposit_noalloc_scratch);
    if (e != cudaSuccess) return hermes::cuda_fail(e, "cudaGetSymbolAddress(g_deposit_noalloc_scratch)");
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return HERMES_OK;
}
}  // namespace

extern "C" int hermes_deposit_noalloc(const double* pos, const double* w, int64_t n, int J, double box,
                                      const double* phi, int n_phi, int phi_res, float* eps_out,
                                      double* eps_f64_out, uint32_t* counts_out, void* stream) {
  if (n < 0 || n > kNoAllocMaxParticles)
    return hermes::fail(HERMES_ERR_INVALID, "deposit_noalloc: n=%lld outside [0, %lld] (the built-in scratch limit)",
                        (long long)n, (long long)kNoAllocMaxParticles);
  if (J > kNoAllocMaxJ)
    return hermes::fail(HERMES_ERR_INVALID, "deposit_noalloc: J=%d above %d (the built-in scratch limit)", J,
                        kNoAllocMaxJ);
  size_t need = 0;
  int rc = workspace_size(n, J, 0, &need);  // always the default tile (the limits above assume it)
  if (rc) return rc;
  if (need > kNoAllocScratchBytes)
    return hermes::fail(HERMES_ERR_INVALID, "deposit_noalloc: needs %zu scratch bytes, built-in array has %zu",
                        need, kNoAllocScratchBytes);
  void* scratch = nullptr;
  rc = noalloc_scratch(&scratch);
  if (rc) return rc;
  // hermes_deposit_sort clears the status word and bucket counts it relies on;
  // everything else in the scratch is written before it is read.
  return deposit_full(pos, w, n, J, box, phi, n_phi, phi_res, eps_out, eps_f64_out, counts_out, scratch,
                      kNoAllocScratchBytes, stream, 0);
}
