// Pointing projections: map2tod (gather) and tod2map (scatter-add).
//
//   map2tod  dat[i] (+)= map[ipix[i]]  -- minkasi/lib/minkasi.c:116-144
//   tod2map  map[ipix[i]] += dat[i]    -- minkasi/lib/minkasi.c:50-112
//
// Both are HBM-bound streams over the TOD: per sample 4 B of ipix plus one
// dat element read or written.  The map (<= 2048^2 doubles = 32 MB) stays
// resident in the 129 MB L2, so the map side costs L2 bandwidth, not HBM.
// Streams are read and written with evict-first hints (ld.global.cs /
// st.global.cs) so they do not push the map out of L2.
#include <cub/device/device_radix_sort.cuh>

#include <mutex>

#include "mk_async.cuh"
#include "mk_common.cuh"

namespace {

constexpr unsigned FULL = 0xffffffffu;

template <typename T>
__device__ __forceinline__ T gather(const T *__restrict__ map, int32_t p, int64_t npix) {
  return ((uint32_t)p < (uint64_t)npix) ? __ldg(map + p) : T(0);
}

// ---- map2tod --------------------------------------------------------------
// Vector body: a warp takes 32 x MU consecutive 16-byte ipix groups (4
// samples each) and lane l the groups l, l + 32, ... of it, so every load and
// store instruction of the warp covers a contiguous span.  The MU index loads
// are all issued before the dependent map gathers: one 16-byte load in flight
// per thread leaves the stream latency-bound (about 32 KB in flight per SM at
// full occupancy, below what HBM needs), MU = 4 gives 64 B per thread.  The
// gathers then bound the kernel through the L1 (81 % busy against 47 % DRAM
// on the 256 x 130,978 TOD), so equal consecutive pixels are loaded once.
// Requires ipix and dat 16-byte aligned; the host falls back to the scalar
// kernel otherwise.
constexpr int MU = 4;

template <typename T, bool ADD>
__global__ void __launch_bounds__(256) k_map2tod_vec(T *__restrict__ dat, const T *__restrict__ map,
                                                     const int32_t *__restrict__ ipix, int64_t n,
                                                     int64_t npix) {
  const int64_t n4 = n >> 2;
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int4 *ip4 = reinterpret_cast<const int4 *>(ipix);
  for (int64_t base = warp * (32 * MU); base < n4; base += nwarp * (32 * MU)) {
    int4 p[MU];
#pragma unroll
    for (int u = 0; u < MU; u++) {
      const int64_t g = base + 32 * u + lane;
      p[u] = g < n4 ? __ldcs(ip4 + g) : make_int4(-1, -1, -1, -1);
    }
    T v[MU][4];
    // a sample on the same pixel as the one before it (runs average about
    // 5 samples) reuses that value: fewer L1 requests for the gathers,
    // which otherwise bound the kernel
#pragma unroll
    for (int u = 0; u < MU; u++) {
      const T a = gather(map, p[u].x, npix);
      const T b = p[u].y == p[u].x ? a : gather(map, p[u].y, npix);
      const T c = p[u].z == p[u].y ? b : gather(map, p[u].z, npix);
      const T d = p[u].w == p[u].z ? c : gather(map, p[u].w, npix);
      v[u][0] = a;
      v[u][1] = b;
      v[u][2] = c;
      v[u][3] = d;
    }
#pragma unroll
    for (int u = 0; u < MU; u++) {
      const int64_t g = base + 32 * u + lane;
      if (g >= n4) continue;
      if constexpr (sizeof(T) == 8) {
        double2 *d2 = reinterpret_cast<double2 *>(dat) + 2 * g;
        if (ADD) {
          const double2 a = __ldcs(d2), b = __ldcs(d2 + 1);
          v[u][0] += a.x; v[u][1] += a.y; v[u][2] += b.x; v[u][3] += b.y;
        }
        __stcs(d2, make_double2(v[u][0], v[u][1]));
        __stcs(d2 + 1, make_double2(v[u][2], v[u][3]));
      } else {
        float4 *d4 = reinterpret_cast<float4 *>(dat) + g;
        if (ADD) {
          const float4 a = __ldcs(d4);
          v[u][0] += a.x; v[u][1] += a.y; v[u][2] += a.z; v[u][3] += a.w;
        }
        __stcs(d4, make_float4(v[u][0], v[u][1], v[u][2], v[u][3]));
      }
    }
  }
  // tail (n % 4 samples), handled by the first threads of block 0
  if (blockIdx.x == 0 && threadIdx.x < (n & 3)) {
    int64_t i = (n4 << 2) + threadIdx.x;
    T v = gather(map, ipix[i], npix);
    dat[i] = ADD ? dat[i] + v : v;
  }
}

template <typename T, bool ADD>
__global__ void __launch_bounds__(256) k_map2tod_scalar(T *__restrict__ dat, const T *__restrict__ map,
                                                        const int32_t *__restrict__ ipix, int64_t n,
                                                        int64_t npix) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    T v = gather(map, ipix[i], npix);
    dat[i] = ADD ? dat[i] + v : v;
  }
}

// ---- tod2map: warp-aggregated atomics -------------------------------------
// A warp reads 32 consecutive samples (coalesced).  Consecutive samples of a
// scanning detector often fall in the same pixel, so runs of equal pixel
// index are summed with a segmented shuffle scan and only the last lane of
// each run issues the (L2) atomic add.
template <typename T>
__device__ __forceinline__ void warp_run_add(T *__restrict__ map, int32_t key, T val, int lane,
                                             int64_t npix) {
  int32_t prev = __shfl_up_sync(FULL, key, 1);
  bool head = (lane == 0) || (prev != key);
  unsigned heads = __ballot_sync(FULL, head);
  unsigned upto = heads & (FULL >> (31 - lane));  // run heads at lanes <= mine
  int start = 31 - __clz(upto);
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    T up = __shfl_up_sync(FULL, val, off);
    if (lane - off >= start) val += up;
  }
  bool tail = (lane == 31) ? true : (((heads >> (lane + 1)) & 1u) != 0u);
  if (tail && (uint32_t)key < (uint64_t)npix) atomicAdd(map + key, val);
}

// ROWS: the value of sample i is rowval[i / ndata] (1 if rowval is NULL);
// used for hit maps, where no TOD-sized array of ones is materialised.
template <typename T, bool ROWS, int U>
__global__ void __launch_bounds__(256) k_tod2map_atomic(T *__restrict__ map, const T *__restrict__ dat,
                                                        const int32_t *__restrict__ ipix, int64_t n,
                                                        int64_t npix, const T *__restrict__ rowval,
                                                        int64_t ndata) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t base = warp * (32 * U); base < n; base += nwarp * (32 * U)) {
    int32_t p[U];
    T v[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      int64_t i = base + u * 32 + lane;
      if (i < n) {
        p[u] = __ldcs(ipix + i);
        if (ROWS)
          v[u] = rowval ? rowval[i / ndata] : T(1);
        else
          v[u] = __ldcs(dat + i);
      } else {
        p[u] = -1;
        v[u] = T(0);
      }
    }
#pragma unroll
    for (int u = 0; u < U; u++) warp_run_add(map, p[u], v[u], lane, npix);
  }
}

__global__ void k_count_bad(const int32_t *__restrict__ ipix, int64_t n, int64_t npix,
                            unsigned long long *nbad) {
  unsigned long long mine = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    mine += ((uint32_t)ipix[i] >= (uint64_t)npix) ? 1ull : 0ull;
  for (int off = 16; off > 0; off >>= 1) mine += __shfl_xor_sync(FULL, mine, off);
  if ((threadIdx.x & 31) == 0 && mine) atomicAdd(nbad, mine);
}

// ---- deterministic tod2map via a pixel plan --------------------------------
__global__ void k_iota(int32_t *v, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) v[i] = (int32_t)i;
}

// offsets[p] = first position in the sorted key list with key >= p, p in [0, npix]
__global__ void k_pix_offsets(const int32_t *__restrict__ keys, int64_t n, int32_t *__restrict__ off,
                              int64_t npix) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p <= npix; p += stride) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
      int64_t mid = (lo + hi) >> 1;
      if ((int64_t)keys[mid] < p) lo = mid + 1; else hi = mid;
    }
    off[p] = (int32_t)lo;
  }
}

// One warp per pixel: lane l sums the pixel's samples l, l+32, ... in sample
// order, then a fixed xor tree combines the lanes -> reproducible bits.
template <typename T>
__global__ void __launch_bounds__(256) k_tod2map_sorted(T *__restrict__ map, const T *__restrict__ dat,
                                                        const int32_t *__restrict__ perm,
                                                        const int32_t *__restrict__ off, int64_t npix) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t p = warp; p < npix; p += nwarp) {
    int32_t b = off[p], e = off[p + 1];
    if (b == e) continue;
    T acc = T(0);
    for (int32_t j = b + lane; j < e; j += 32) acc += __ldg(dat + __ldg(perm + j));
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) acc += __shfl_xor_sync(FULL, acc, s);
    if (lane == 0) map[p] += acc;
  }
}

// ---- deterministic tod2map by 64-bit fixed-point accumulation ------------
// Integer addition is associative, so the accumulated map is bitwise the
// same whatever order the atomics land in.  Scale: with D = max|dat| < 2^(e+1)
// and every pixel hit at most hmax <= 2^hbits times, each term
// llrint(dat * 2^s) is below 2^(e+1+s) and a pixel's sum below
// 2^(e+1+s+hbits) = 2^62 for s = 61 - e - hbits.
// Header words of the scratch: [0] max|dat| over the finite samples, as the
// bits of a non-negative double (atomicMax on the bit pattern orders like the
// value), [1] the shift s chosen by the scatter pass.
// Non-finite samples (NaN, +-inf) bypass the integers: each is added straight
// into its own pixel of the map with a floating-point atomic, so a pixel ends
// up NaN / +-inf exactly when the reference's serial sum would (the IEEE sum
// of the special values a pixel receives does not depend on their order),
// and every other pixel is untouched by them.
struct FixHdr {
  unsigned long long dmax_bits;
  long long shift;
  unsigned long long pad[30];
};

// Integer-only fixed-point conversion.  GB300's FP64 units are a small
// fraction of its integer throughput, so the per-sample path touches no FP64
// arithmetic: |x| is compared as a bit pattern, and x * 2^s is formed by
// shifting the mantissa (round half away from zero).  The same helpers serve
// the aligned and unaligned kernels, so both give identical bits.
__device__ __forceinline__ unsigned long long abs_bits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
}
__device__ __forceinline__ unsigned int abs_bits(float x) { return __float_as_uint(x) & 0x7FFFFFFFu; }
// |x| bit patterns at or above these are +inf or NaN
__device__ __forceinline__ bool nonfinite_bits(unsigned long long a) { return a >= 0x7FF0000000000000ull; }
__device__ __forceinline__ bool nonfinite_bits(unsigned int a) { return a >= 0x7F800000u; }

__device__ __forceinline__ long long shift_round(unsigned long long m, int sh, bool neg) {
  unsigned long long r;
  if (sh >= 0)
    r = m << sh;  // sh <= 9 (double) / 38 (float) by the choice of s: no overflow
  else if (sh > -64)
    r = (m + (1ull << (-sh - 1))) >> (-sh);
  else
    r = 0;
  return neg ? -(long long)r : (long long)r;
}

// round(x * 2^s) for a finite double
__device__ __forceinline__ long long to_fixed(double x, int s) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int ef = (int)((b >> 52) & 0x7FF);
  unsigned long long m = b & 0x000FFFFFFFFFFFFFull;
  if (ef) m |= 0x0010000000000000ull;
  return shift_round(m, (ef ? ef : 1) - 1075 + s, (b >> 63) != 0);
}

// round(x * 2^s) for a finite float
__device__ __forceinline__ long long to_fixed(float x, int s) {
  const unsigned int b = __float_as_uint(x);
  const int ef = (int)((b >> 23) & 0xFF);
  unsigned long long m = b & 0x7FFFFFu;
  if (ef) m |= 0x800000u;
  return shift_round(m, (ef ? ef : 1) - 150 + s, (b >> 31) != 0);
}

template <typename T>
struct AbsBits;
template <>
struct AbsBits<double> {
  using U = unsigned long long;
  static __device__ __forceinline__ unsigned long long as_double_bits(U u) { return u; }
};
template <>
struct AbsBits<float> {
  using U = unsigned int;
  static __device__ __forceinline__ unsigned long long as_double_bits(U u) {
    return (unsigned long long)__double_as_longlong((double)__uint_as_float(u));
  }
};

// block max of bit patterns -> one atomicMax into the header (as double bits)
template <typename T>
__device__ __forceinline__ void absmax_finish(typename AbsBits<T>::U m, FixHdr *h) {
  unsigned long long b = AbsBits<T>::as_double_bits(m);
  for (int off = 16; off > 0; off >>= 1) {
    unsigned long long o = __shfl_xor_sync(FULL, b, off);
    b = o > b ? o : b;
  }
  __shared__ unsigned long long sh[32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = b;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) b = sh[w] > b ? sh[w] : b;
    atomicMax(&h->dmax_bits, b);
  }
}

__device__ __forceinline__ void flush_i64(unsigned long long *__restrict__ acc, int32_t key, long long v,
                                          int64_t npix) {
  if (v != 0 && (uint32_t)key < (uint64_t)npix) atomicAdd(acc + key, (unsigned long long)v);
}

// shift s from the header; any s when every finite sample is zero
__device__ __forceinline__ int fixed_shift(const FixHdr *h, int hbits) {
  const double dmax = __longlong_as_double((long long)h->dmax_bits);
  if (!(dmax > 0.0)) return 0;
  return 61 - ilogb(dmax) - hbits;
}

// The fixed-point term of one sample; a non-finite sample is added to its
// pixel of the map directly and contributes nothing to the accumulator.
template <typename T>
__device__ __forceinline__ long long fixed_term(T *__restrict__ map, int32_t key, T x, int s, int64_t npix) {
  if (nonfinite_bits(abs_bits(x))) {
    if ((uint32_t)key < (uint64_t)npix) atomicAdd(map + key, x);
    return 0;
  }
  return to_fixed(x, s);
}


template <typename T>
__global__ void __launch_bounds__(256) k_absmax(const T *__restrict__ dat, int64_t n, FixHdr *h) {
  using U = typename AbsBits<T>::U;
  U m = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    U a = abs_bits(__ldcs(dat + i));
    m = (a > m && !nonfinite_bits(a)) ? a : m;
  }
  absmax_finish<T>(m, h);
}

__device__ __forceinline__ void warp_run_add_i64(unsigned long long *__restrict__ acc, int32_t key,
                                                 long long val, int lane, int64_t npix) {
  int32_t prev = __shfl_up_sync(FULL, key, 1);
  bool head = (lane == 0) || (prev != key);
  unsigned heads = __ballot_sync(FULL, head);
  unsigned upto = heads & (FULL >> (31 - lane));
  int start = 31 - __clz(upto);
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    long long up = __shfl_up_sync(FULL, val, off);
    if (lane - off >= start) val += up;
  }
  bool tail = (lane == 31) ? true : (((heads >> (lane + 1)) & 1u) != 0u);
  if (tail && val != 0 && (uint32_t)key < (uint64_t)npix) atomicAdd(acc + key, (unsigned long long)val);
}

template <typename T, int U>
__global__ void __launch_bounds__(256) k_scatter_fixed(unsigned long long *__restrict__ acc, T *__restrict__ map,
                                                       const T *__restrict__ dat,
                                                       const int32_t *__restrict__ ipix, int64_t n,
                                                       int64_t npix, int hbits, FixHdr *h) {
  const int s = fixed_shift(h, hbits);
  if (blockIdx.x == 0 && threadIdx.x == 0) h->shift = s;
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t base = warp * (32 * U); base < n; base += nwarp * (32 * U)) {
    int32_t p[U];
    long long v[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      int64_t i = base + u * 32 + lane;
      if (i < n) {
        p[u] = __ldcs(ipix + i);
        v[u] = fixed_term(map, p[u], __ldcs(dat + i), s, npix);
      } else {
        p[u] = -1;
        v[u] = 0;
      }
    }
#pragma unroll
    for (int u = 0; u < U; u++) warp_run_add_i64(acc, p[u], v[u], lane, npix);
  }
}

// ---- vectorised forms (ipix and dat 16-byte aligned) -----------------------
// Each thread owns 8 consecutive samples: two 16-byte ipix loads and 16/32
// bytes of dat per load instruction (a warp covers 256 consecutive samples,
// fully coalesced).  Runs of equal pixels inside the 8 are summed in a
// register; one integer atomic per run.  This trades the warp-wide scan
// (~25 instructions per sample) for ~6, which matters because the scan
// version is issue-bound.
template <typename T>
__device__ __forceinline__ void load8(const T *__restrict__ p, T (&v)[8]) {
  if constexpr (sizeof(T) == 8) {
    const double2 *q = reinterpret_cast<const double2 *>(p);
#pragma unroll
    for (int k = 0; k < 4; k++) {
      double2 a = __ldcs(q + k);
      v[2 * k] = a.x;
      v[2 * k + 1] = a.y;
    }
  } else {
    const float4 *q = reinterpret_cast<const float4 *>(p);
#pragma unroll
    for (int k = 0; k < 2; k++) {
      float4 a = __ldcs(q + k);
      v[4 * k] = a.x;
      v[4 * k + 1] = a.y;
      v[4 * k + 2] = a.z;
      v[4 * k + 3] = a.w;
    }
  }
}

__device__ __forceinline__ void load8i(const int32_t *__restrict__ p, int32_t (&k)[8]) {
  const int4 *q = reinterpret_cast<const int4 *>(p);
  int4 a = __ldcs(q), b = __ldcs(q + 1);
  k[0] = a.x; k[1] = a.y; k[2] = a.z; k[3] = a.w;
  k[4] = b.x; k[5] = b.y; k[6] = b.z; k[7] = b.w;
}

template <typename T>
__global__ void __launch_bounds__(256, 8) k_absmax8(const T *__restrict__ dat, int64_t n, FixHdr *h) {
  using U = typename AbsBits<T>::U;
  U m = 0;
  const int64_t n8 = n >> 3;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n8; g += stride) {
    T v[8];
    load8(dat + 8 * g, v);
#pragma unroll
    for (int k = 0; k < 8; k++) {
      U a = abs_bits(v[k]);
      m = (a > m && !nonfinite_bits(a)) ? a : m;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x < (n & 7)) {
    U a = abs_bits(dat[(n8 << 3) + threadIdx.x]);
    m = (a > m && !nonfinite_bits(a)) ? a : m;
  }
  absmax_finish<T>(m, h);
}

template <typename T>
__global__ void __launch_bounds__(256) k_scatter_fixed8(unsigned long long *__restrict__ acc,
                                                        T *__restrict__ map, const T *__restrict__ dat,
                                                        const int32_t *__restrict__ ipix, int64_t n,
                                                        int64_t npix, int hbits, FixHdr *h) {
  const int s = fixed_shift(h, hbits);
  if (blockIdx.x == 0 && threadIdx.x == 0) h->shift = s;
  const int64_t n8 = n >> 3;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n8; g += stride) {
    int32_t p[8];
    T v[8];
    load8i(ipix + 8 * g, p);
    load8(dat + 8 * g, v);
    int32_t key = p[0];
    long long cur = fixed_term(map, p[0], v[0], s, npix);
#pragma unroll
    for (int k = 1; k < 8; k++) {
      long long t = fixed_term(map, p[k], v[k], s, npix);
      if (p[k] == key) {
        cur += t;
      } else {
        flush_i64(acc, key, cur, npix);
        key = p[k];
        cur = t;
      }
    }
    flush_i64(acc, key, cur, npix);
  }
  if (blockIdx.x == 0 && threadIdx.x < (n & 7)) {
    int64_t i = (n8 << 3) + threadIdx.x;
    flush_i64(acc, ipix[i], fixed_term(map, ipix[i], dat[i], s, npix), npix);
  }
}

// map += acc * 2^-s, acc cleared (a pixel already made NaN / inf by a
// non-finite sample stays so)
template <typename T>
__global__ void k_fixed_finalize(T *__restrict__ map, unsigned long long *__restrict__ acc, int64_t npix,
                                 FixHdr *h, int64_t nsamp) {
  const double inv = ldexp(1.0, -(int)h->shift);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += stride) {
    long long a = (long long)acc[p];
    if (a != 0) {
      map[p] = (T)((double)map[p] + (double)a * inv);
      acc[p] = 0ull;
    }
  }
}

template <typename T>
__global__ void k_fixed_reset(FixHdr *h) {
  h->dmax_bits = 0ull;
}

template <typename T>
int map2tod_t(void *dat, const void *map, const int32_t *ipix, int64_t n, int64_t npix, int do_add,
              cudaStream_t st) {
  bool vec = ((uintptr_t)dat % 16 == 0) && ((uintptr_t)ipix % 16 == 0) && n >= 4;
  const int B = 256;
  if (vec) {
    if (do_add)
      k_map2tod_vec<T, true><<<mk_grid_fit(k_map2tod_vec<T, true>, ((n >> 2) + MU - 1) / MU, B), B, 0, st>>>(
          (T *)dat, (const T *)map, ipix, n, npix);
    else
      k_map2tod_vec<T, false><<<mk_grid_fit(k_map2tod_vec<T, false>, ((n >> 2) + MU - 1) / MU, B), B, 0, st>>>(
          (T *)dat, (const T *)map, ipix, n, npix);
  } else {
    if (do_add)
      k_map2tod_scalar<T, true><<<mk_grid_fit(k_map2tod_scalar<T, true>, n, B), B, 0, st>>>(
          (T *)dat, (const T *)map, ipix, n, npix);
    else
      k_map2tod_scalar<T, false><<<mk_grid_fit(k_map2tod_scalar<T, false>, n, B), B, 0, st>>>(
          (T *)dat, (const T *)map, ipix, n, npix);
  }
  return mk::launch_status("mk_map2tod");
}

// Scatter with runs of equal pixel joined across the lanes of a warp: each
// warp takes windows of 256 consecutive samples (8 per lane, 16-byte loads),
// each lane sums its runs in registers, and warp_runs joins the runs that cross
// lanes, so a run costs one L2 atomic whatever its alignment.  On GB300 the
// scatter is bound by the L2 atomic rate, not by HBM: the same loads without
// atomics stream at 7 TB/s, and one atomic per sample runs at 2.1 TB/s.
//
// warp_runs: lane l holds samples 8l .. 8l+7 of the window, the first m of
// them valid (0 <= m <= 8; the valid samples of a window are a prefix of it).
// Each lane sums its own runs and issues the atomics of the runs that start
// and end inside it; the runs that cross lane boundaries are joined by a
// segmented scan over the lanes, and each is added once, by the lane where it
// ends.  With daisy scans a run of equal pixels is ~5 samples long, so joining
// the runs cut by the 8-sample lane windows removes about 40 % of the atomics.
template <typename T>
__device__ __forceinline__ void warp_runs(T *__restrict__ map, const int32_t (&p)[8], const T (&v)[8], int m,
                                          int lane, int64_t npix) {
  int32_t kf = INT32_MIN, kl = INT32_MIN;  // first / last run keys of this lane
  T sf = T(0), sl = T(0);
  bool single = true;  // the lane's samples are one run
  if (m > 0) {
    int32_t key = p[0];
    T cur = v[0];
    kf = key;
#pragma unroll
    for (int j = 1; j < 8; j++) {
      if (j < m) {
        if (p[j] == key) {
          cur += v[j];
        } else {
          if (single) {
            sf = cur;
            single = false;
          } else if ((uint32_t)key < (uint64_t)npix) {
            atomicAdd(map + key, cur);  // a run inside the lane
          }
          key = p[j];
          cur = v[j];
        }
      }
    }
    kl = key;
    sl = cur;
    if (single) sf = cur;
  }
  const int32_t kl_prev = __shfl_up_sync(FULL, kl, 1);
  const int32_t kf_next = __shfl_down_sync(FULL, kf, 1);
  const bool cont_in = lane > 0 && m > 0 && kl_prev == kf;
  const bool cont_out = lane < 31 && kf_next == kl && m > 0;
  // out_l = y_l + [single_l and cont_in_l] out_{l-1}, y = the part handed on.
  // A run passes through a lane only if the lane is one run that continues
  // a run from the previous lane; when no lane of the warp does (the common
  // case), out = y and one shuffle suffices.  The segmented scan, whose FP64
  // adds are costly on GB300's narrow FP64 pipe, runs only otherwise.
  T out = single ? sf : sl;
  if (__ballot_sync(FULL, single && cont_in) != 0u) {
    bool head = !(single && cont_in);
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const T up = __shfl_up_sync(FULL, out, off);
      const bool hup = __shfl_up_sync(FULL, (int)head, off) != 0;
      if (lane >= off) {
        if (!head) out += up;
        head = head || hup;
      }
    }
  }
  const T prev = __shfl_up_sync(FULL, out, 1);
  if (m == 0) return;
  const T first = cont_in ? prev + sf : sf;  // the first run, with what flows in
  if (single) {
    if (!cont_out && (uint32_t)kf < (uint64_t)npix) atomicAdd(map + kf, first);
  } else {
    if ((uint32_t)kf < (uint64_t)npix) atomicAdd(map + kf, first);
    if (!cont_out && (uint32_t)kl < (uint64_t)npix) atomicAdd(map + kl, sl);
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_tod2map_atomic8(T *__restrict__ map, const T *__restrict__ dat,
                                                         const int32_t *__restrict__ ipix, int64_t n,
                                                         int64_t npix) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t base = warp * 256; base < n; base += nwarp * 256) {
    const int64_t i0 = base + 8 * lane;
    const int64_t r = n - i0;
    const int m = r <= 0 ? 0 : (r >= 8 ? 8 : (int)r);
    int32_t p[8];
    T v[8];
    if (m == 8) {
      load8i(ipix + i0, p);
      load8(dat + i0, v);
    } else {
#pragma unroll
      for (int j = 0; j < 8; j++) {
        p[j] = j < m ? ipix[i0 + j] : INT32_MIN;
        v[j] = j < m ? dat[i0 + j] : T(0);
      }
    }
    warp_runs<T>(map, p, v, m, lane, npix);
  }
}

template <typename T, bool ROWS>
int tod2map_t(void *map, const void *dat, const int32_t *ipix, int64_t n, int64_t npix,
              const void *rowval, int64_t ndata, cudaStream_t st) {
  const int B = 256;
  if (!ROWS && (uintptr_t)dat % 16 == 0 && (uintptr_t)ipix % 16 == 0) {
    // more CTAs than fit at once: the warps' windows are short, and a deep
    // queue of CTAs keeps every SM's atomic issue busy to the end
    k_tod2map_atomic8<T><<<mk_grid((n + 7) / 8, B, 16), B, 0, st>>>((T *)map, (const T *)dat, ipix, n, npix);
    return mk::launch_status("mk_tod2map");
  }
  constexpr int U = 4;
  unsigned g = mk_grid_fit(k_tod2map_atomic<T, ROWS, U>, (n + U - 1) / U, B);
  k_tod2map_atomic<T, ROWS, U><<<g, B, 0, st>>>((T *)map, (const T *)dat, ipix, n, npix,
                                                 (const T *)rowval, ndata);
  return mk::launch_status("mk_tod2map");
}

// ---- tod2map, bulk-staged, warp-specialised ---------------------------------
// A persistent CTA streams chunks of SCH consecutive samples (pixel indices
// and values) through a ring of SSTG shared-memory stages.  One producer
// warp issues the cp.async.bulk copies of each chunk; they complete on the
// stage's "full" mbarrier.  SCW consumer warps each reduce their 256 samples
// of the chunk (8 consecutive samples per lane; runs of equal pixels summed in
// registers and joined across lanes by warp_runs, one L2 atomic per run) and arrive on the
// stage's "empty" mbarrier, which the producer waits on before refilling the
// stage.  No CTA-wide barrier sits in the loop, so the consumer warps drift
// freely and several chunks per CTA are in flight from HBM at any time.
// Chunk c holds samples [c*SCH, min(c*SCH + SCH, n4)), n4 = n rounded down to
// a multiple of 4 so every copy is a multiple of 16 bytes; CTA 0 adds the last
// n - n4 samples with plain loads.  Needs ipix and dat 16-byte aligned device
// memory.  Every wait is bounded; on a timeout the CTA records it in
// g_staged_err, the producer stops issuing and waits (bounded) for its copies
// in flight, and every warp leaves its loop.
constexpr int SCW = 8;                    // consumer warps
constexpr int SCH = SCW * 32 * 8;         // samples per chunk (2048)
constexpr int SSTG = 3;                   // stages in the ring
constexpr int STHREADS = (SCW + 1) * 32;  // + one producer warp

template <typename T>
struct StagedSmem {
  int32_t pix[SSTG][SCH];
  T val[SSTG][SCH];
  uint64_t full[SSTG];
  uint64_t empty[SSTG];
  int abort;
};

// 1 once a bounded wait of k_tod2map_staged timed out (mk_tod2map_status)
__device__ int g_staged_err = 0;

template <typename T>
__device__ __forceinline__ void staged_issue(StagedSmem<T> &sm, int s, int64_t c, int64_t n4,
                                             const int32_t *ipix, const T *dat, uint64_t pol) {
  const int64_t base = c * SCH;
  const int64_t rem = n4 - base;
  const uint32_t cnt = (uint32_t)(rem < SCH ? rem : SCH);
  mk::mbar_expect_tx(&sm.full[s], cnt * (uint32_t)(sizeof(int32_t) + sizeof(T)));
  mk::bulk_g2s_hint(sm.pix[s], ipix + base, cnt * (uint32_t)sizeof(int32_t), &sm.full[s], pol);
  mk::bulk_g2s_hint(sm.val[s], dat + base, cnt * (uint32_t)sizeof(T), &sm.full[s], pol);
}

template <typename V>
__device__ __forceinline__ V pick4(V a, V b, V c, V d, int i) {
  return i == 0 ? a : (i == 1 ? b : (i == 2 ? c : d));
}

// Thread t's 8 samples at sp[8t..8t+7] / sv[8t..8t+7].  The 16-byte
// shared-memory loads are issued in a per-thread rotated order so that each
// group of 8 threads served together touches all 32 banks (no conflicts),
// then put back in sample order with selects.
template <typename T>
__device__ __forceinline__ void smem_load8(const int32_t *sp, const T *sv, int t, int32_t (&p)[8], T (&v)[8]) {
  const int4 *qp = reinterpret_cast<const int4 *>(sp + 8 * t);
  const int r1 = (t >> 2) & 1;
  int4 a = qp[r1], b = qp[r1 ^ 1];
  int4 lo = r1 ? b : a, hi = r1 ? a : b;
  p[0] = lo.x; p[1] = lo.y; p[2] = lo.z; p[3] = lo.w;
  p[4] = hi.x; p[5] = hi.y; p[6] = hi.z; p[7] = hi.w;
  if constexpr (sizeof(T) == 8) {
    const double2 *qv = reinterpret_cast<const double2 *>(sv + 8 * t);
    const int r = (t >> 1) & 3;
    double2 L0 = qv[r], L1 = qv[(1 + r) & 3], L2 = qv[(2 + r) & 3], L3 = qv[(3 + r) & 3];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      double2 P = pick4(L0, L1, L2, L3, (j - r) & 3);
      v[2 * j] = P.x;
      v[2 * j + 1] = P.y;
    }
  } else {
    const float4 *qv = reinterpret_cast<const float4 *>(sv + 8 * t);
    float4 c = qv[r1], d = qv[r1 ^ 1];
    float4 vl = r1 ? d : c, vh = r1 ? c : d;
    v[0] = vl.x; v[1] = vl.y; v[2] = vl.z; v[3] = vl.w;
    v[4] = vh.x; v[5] = vh.y; v[6] = vh.z; v[7] = vh.w;
  }
}

template <typename T>
__global__ void __launch_bounds__(STHREADS) k_tod2map_staged(T *__restrict__ map, const T *__restrict__ dat,
                                                             const int32_t *__restrict__ ipix, int64_t n,
                                                             int64_t npix) {
  extern __shared__ __align__(128) unsigned char smraw[];
  StagedSmem<T> &sm = *reinterpret_cast<StagedSmem<T> *>(smraw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t n4 = n & ~(int64_t)3;
  const int64_t nchunk = (n4 + SCH - 1) / SCH;
  const int64_t G = gridDim.x;
  if (tid == 0) {
    for (int s = 0; s < SSTG; s++) {
      mk::mbar_init(&sm.full[s], 1);
      mk::mbar_init(&sm.empty[s], SCW);
    }
    sm.abort = 0;
    mk::mbar_init_fence();
  }
  __syncthreads();
  volatile int *abort_flag = &sm.abort;
  int64_t issued = 0;

  if (warp == SCW) {
    // ---- producer
    if (lane == 0) {
      const uint64_t pol = mk::l2_evict_first_policy();
      for (int64_t c = blockIdx.x; c < nchunk; c += G, issued++) {
        const int s = (int)(issued % SSTG);
        if (issued >= SSTG) {
          // wait until every consumer warp released the stage's previous chunk
          if (!mk::mbar_wait(&sm.empty[s], (uint32_t)(((issued / SSTG) - 1) & 1))) {
            atomicExch(&g_staged_err, 1);
            *abort_flag = 1;
          }
        }
        if (*abort_flag) break;
        mk::fence_proxy_async_smem();
        staged_issue(sm, s, c, n4, ipix, dat, pol);
      }
    }
  } else {
    // ---- consumers: warp w takes samples [w*256, w*256 + 256) of every chunk
    const int t = warp * 32 + lane;
    const int j0 = t * 8;
    int64_t k = 0;
    for (int64_t c = blockIdx.x; c < nchunk; c += G, k++) {
      const int s = (int)(k % SSTG);
      const bool ok = mk::mbar_wait(&sm.full[s], (uint32_t)((k / SSTG) & 1));
      const int ab = __shfl_sync(0xffffffffu, *abort_flag, 0);  // one warp-uniform reading
      if (__any_sync(0xffffffffu, !ok) || ab) {
        if (lane == 0) {
          atomicExch(&g_staged_err, 1);
          *abort_flag = 1;
        }
        break;
      }
      const int64_t rem = n4 - c * SCH;
      const int cnt = (int)(rem < SCH ? rem : SCH);
      int32_t p[8];
      T v[8];
      int mv = cnt - j0;
      mv = mv < 0 ? 0 : (mv > 8 ? 8 : mv);
      if (mv == 8) {
        smem_load8(sm.pix[s], sm.val[s], t, p, v);
      } else {
#pragma unroll
        for (int j = 0; j < 8; j++) {
          p[j] = j < mv ? sm.pix[s][j0 + j] : INT32_MIN;
          v[j] = j < mv ? sm.val[s][j0 + j] : T(0);
        }
      }
      warp_runs<T>(map, p, v, mv, lane, npix);
      __syncwarp();
      if (lane == 0) mk::mbar_arrive(&sm.empty[s]);
    }
    if (blockIdx.x == 0 && warp == 0 && lane < (int)(n - n4)) {
      const int64_t i = n4 + lane;
      const int32_t key = ipix[i];
      if ((uint32_t)key < (uint64_t)npix) atomicAdd(map + key, dat[i]);
    }
  }
  // every loop above ends in bounded time; after an abort, no copy of this
  // CTA may still be landing in shared memory when it exits
  __syncthreads();
  if (warp == SCW && lane == 0 && *abort_flag) {
    const int64_t from = issued > SSTG ? issued - SSTG : 0;
    for (int64_t j = from; j < issued; j++) mk::mbar_wait(&sm.full[j % SSTG], (uint32_t)((j / SSTG) & 1));
  }
}

template <typename T>
int tod2map_staged_t(void *map, const void *dat, const int32_t *ipix, int64_t n, int64_t npix,
                     cudaStream_t st) {
  const size_t smem = sizeof(StagedSmem<T>);
  static bool attr_set[64] = {false};
  int dev = 0;
  MK_CUDA(cudaGetDevice(&dev));
  if (dev >= 0 && dev < 64 && !attr_set[dev]) {
    MK_CUDA(cudaFuncSetAttribute(k_tod2map_staged<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set[dev] = true;
  }
  const int64_t nchunk = ((n & ~(int64_t)3) + SCH - 1) / SCH;
  const int per_sm = mk::resident_ctas((const void *)k_tod2map_staged<T>, STHREADS, smem);
  int64_t g = (int64_t)mk::sm_count() * per_sm;
  if (g > nchunk) g = nchunk;
  if (g < 1) g = 1;
  k_tod2map_staged<T><<<(unsigned)g, STHREADS, smem, st>>>((T *)map, (const T *)dat, ipix, n, npix);
  return mk::launch_status("mk_tod2map_staged");
}

template <typename T>
int tod2map_fixed_t(void *map, const void *dat, const int32_t *ipix, int64_t n, int64_t npix,
                    int hbits, void *scratch, cudaStream_t st) {
  FixHdr *h = (FixHdr *)scratch;
  unsigned long long *acc = (unsigned long long *)((char *)scratch + sizeof(FixHdr));
  const bool vec = ((uintptr_t)dat % 16 == 0) && ((uintptr_t)ipix % 16 == 0);
  if (vec) {
    k_absmax8<T><<<mk_grid_fit(k_absmax8<T>, (n + 7) / 8, 256), 256, 0, st>>>((const T *)dat, n, h);
    k_scatter_fixed8<T><<<mk_grid_fit(k_scatter_fixed8<T>, (n + 7) / 8, 256), 256, 0, st>>>(
        acc, (T *)map, (const T *)dat, ipix, n, npix, hbits, h);
  } else {
    k_absmax<T><<<mk_grid_fit(k_absmax<T>, n, 256), 256, 0, st>>>((const T *)dat, n, h);
    constexpr int U = 4;
    k_scatter_fixed<T, U><<<mk_grid_fit(k_scatter_fixed<T, U>, (n + U - 1) / U, 256), 256, 0, st>>>(
        acc, (T *)map, (const T *)dat, ipix, n, npix, hbits, h);
  }
  k_fixed_finalize<T><<<mk_grid_fit(k_fixed_finalize<T>, npix, 256), 256, 0, st>>>((T *)map, acc, npix, h, n);
  k_fixed_reset<T><<<1, 1, 0, st>>>(h);
  return mk::launch_status("mk_tod2map_fixed");
}

}  // namespace

struct mk_pixplan {
  int32_t *perm = nullptr;   // sample indices sorted by pixel (stable)
  int32_t *off = nullptr;    // npix+1 offsets into perm
  int64_t n = 0, npix = 0;
};

extern "C" int mk_map2tod(void *dat, const void *map, const int32_t *ipix, int64_t ndet,
                          int64_t ndata, int64_t npix, int dtype, int do_add, void *stream) {
  MK_CHECK_ARG(ndet >= 0 && ndata >= 0 && npix >= 0, "mk_map2tod: negative size");
  MK_CHECK_ARG(MK_DTYPE_OK(dtype), "mk_map2tod: bad dtype %d", dtype);
  int64_t n = ndet * ndata;
  if (n == 0) return MK_OK;
  MK_CHECK_ARG(dat && map && ipix, "mk_map2tod: null pointer");
  cudaStream_t st = mk::as_stream(stream);
  return dtype == MK_F64 ? map2tod_t<double>(dat, map, ipix, n, npix, do_add, st)
                         : map2tod_t<float>(dat, map, ipix, n, npix, do_add, st);
}

extern "C" int mk_tod2map(void *map, const void *dat, const int32_t *ipix, int64_t ndet,
                          int64_t ndata, int64_t npix, int dtype, void *stream) {
  MK_CHECK_ARG(ndet >= 0 && ndata >= 0 && npix >= 0, "mk_tod2map: negative size");
  MK_CHECK_ARG(MK_DTYPE_OK(dtype), "mk_tod2map: bad dtype %d", dtype);
  int64_t n = ndet * ndata;
  if (n == 0) return MK_OK;
  MK_CHECK_ARG(dat && map && ipix, "mk_tod2map: null pointer");
  cudaStream_t st = mk::as_stream(stream);
  return dtype == MK_F64 ? tod2map_t<double, false>(map, dat, ipix, n, npix, nullptr, 1, st)
                         : tod2map_t<float, false>(map, dat, ipix, n, npix, nullptr, 1, st);
}

static bool is_device_ptr(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice;
}

extern "C" int mk_tod2map_staged(void *map, const void *dat, const int32_t *ipix, int64_t ndet,
                                 int64_t ndata, int64_t npix, int dtype, void *stream) {
  MK_CHECK_ARG(ndet >= 0 && ndata >= 0 && npix >= 0, "mk_tod2map_staged: negative size");
  MK_CHECK_ARG(MK_DTYPE_OK(dtype), "mk_tod2map_staged: bad dtype %d", dtype);
  int64_t n = ndet * ndata;
  if (n == 0) return MK_OK;
  MK_CHECK_ARG(dat && map && ipix, "mk_tod2map_staged: null pointer");
  MK_CHECK_ARG((uintptr_t)dat % 16 == 0 && (uintptr_t)ipix % 16 == 0,
               "mk_tod2map_staged: dat and ipix must be 16-byte aligned");
  MK_CHECK_ARG(is_device_ptr(dat) && is_device_ptr(ipix) && is_device_ptr(map),
               "mk_tod2map_staged: map, dat and ipix must be device memory");
  cudaStream_t st = mk::as_stream(stream);
  return dtype == MK_F64 ? tod2map_staged_t<double>(map, dat, ipix, n, npix, st)
                         : tod2map_staged_t<float>(map, dat, ipix, n, npix, st);
}

extern "C" int mk_tod2map_status(int *code, void *stream) {
  MK_CHECK_ARG(code, "mk_tod2map_status: null pointer");
  cudaStream_t st = mk::as_stream(stream);
  *code = 0;
  MK_CUDA(cudaMemcpyFromSymbolAsync(code, g_staged_err, sizeof(int), 0, cudaMemcpyDeviceToHost, st));
  const int zero = 0;
  MK_CUDA(cudaMemcpyToSymbolAsync(g_staged_err, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, st));
  MK_CUDA(cudaStreamSynchronize(st));
  return MK_OK;
}

extern "C" int mk_tod2map_rows(void *map, const void *w, const int32_t *ipix, int64_t ndet,
                               int64_t ndata, int64_t npix, int dtype, void *stream) {
  MK_CHECK_ARG(ndet >= 0 && ndata >= 0 && npix >= 0, "mk_tod2map_rows: negative size");
  MK_CHECK_ARG(MK_DTYPE_OK(dtype), "mk_tod2map_rows: bad dtype %d", dtype);
  int64_t n = ndet * ndata;
  if (n == 0) return MK_OK;
  MK_CHECK_ARG(map && ipix, "mk_tod2map_rows: null pointer");
  cudaStream_t st = mk::as_stream(stream);
  return dtype == MK_F64 ? tod2map_t<double, true>(map, nullptr, ipix, n, npix, w, ndata, st)
                         : tod2map_t<float, true>(map, nullptr, ipix, n, npix, w, ndata, st);
}

extern "C" int mk_check_pix(const int32_t *ipix, int64_t n, int64_t npix, int64_t *nbad,
                            void *stream) {
  MK_CHECK_ARG(nbad, "mk_check_pix: null result pointer");
  *nbad = 0;
  if (n <= 0) return MK_OK;
  MK_CHECK_ARG(ipix, "mk_check_pix: null ipix");
  cudaStream_t st = mk::as_stream(stream);
  unsigned long long *d = nullptr;
  MK_CUDA(cudaMallocAsync((void **)&d, sizeof(*d), st));
  MK_CUDA(cudaMemsetAsync(d, 0, sizeof(*d), st));
  k_count_bad<<<mk_grid_fit(k_count_bad, n, 256), 256, 0, st>>>(ipix, n, npix, d);
  int rc = mk::launch_status("mk_check_pix");
  unsigned long long h = 0;
  cudaError_t e1 = cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, st);
  cudaError_t e2 = cudaFreeAsync(d, st);
  cudaError_t e3 = cudaStreamSynchronize(st);
  if (rc != MK_OK) return rc;
  MK_CUDA(e1);
  MK_CUDA(e2);
  MK_CUDA(e3);
  *nbad = (int64_t)h;
  return MK_OK;
}

extern "C" int mk_pixplan_create(mk_pixplan **plan, const int32_t *ipix, int64_t n, int64_t npix,
                                 void *stream) {
  MK_CHECK_ARG(plan, "mk_pixplan_create: null plan pointer");
  *plan = nullptr;
  MK_CHECK_ARG(n >= 0 && n < (int64_t)INT32_MAX, "mk_pixplan_create: n=%lld must be < 2^31",
               (long long)n);
  MK_CHECK_ARG(npix > 0 && npix < (int64_t)INT32_MAX, "mk_pixplan_create: bad npix");
  MK_CHECK_ARG(n == 0 || ipix, "mk_pixplan_create: null ipix");
  int64_t nbad = 0;
  int rc = mk_check_pix(ipix, n, npix, &nbad, stream);
  if (rc) return rc;
  if (nbad) {
    mk::set_error("mk_pixplan_create: %lld pixel indices outside [0, %lld)", (long long)nbad,
                  (long long)npix);
    return MK_ERR_RANGE;
  }
  cudaStream_t st = mk::as_stream(stream);
  mk_pixplan *pl = new (std::nothrow) mk_pixplan;
  if (!pl) return MK_ERR_NOMEM;
  pl->n = n;
  pl->npix = npix;
  int32_t *keys_out = nullptr, *idx_in = nullptr;
  void *tmp = nullptr;
  size_t tmp_bytes = 0;
  int end_bit = 1;
  while (end_bit < 31 && (int64_t(1) << end_bit) < npix) end_bit++;
  cudaError_t e = cudaSuccess;
  auto fail = [&](const char *what, cudaError_t err) {
    mk::set_error("mk_pixplan_create: %s: %s", what, cudaGetErrorString(err));
    cudaFree(keys_out);
    cudaFree(idx_in);
    cudaFree(tmp);
    cudaFree(pl->perm);
    cudaFree(pl->off);
    delete pl;
    return MK_ERR_CUDA;
  };
  size_t nb = (size_t)(n > 0 ? n : 1) * sizeof(int32_t);
  if ((e = cudaMalloc(&pl->perm, nb)) != cudaSuccess) return fail("cudaMalloc", e);
  if ((e = cudaMalloc(&pl->off, (size_t)(npix + 1) * sizeof(int32_t))) != cudaSuccess)
    return fail("cudaMalloc", e);
  if ((e = cudaMalloc(&keys_out, nb)) != cudaSuccess) return fail("cudaMalloc", e);
  if ((e = cudaMalloc(&idx_in, nb)) != cudaSuccess) return fail("cudaMalloc", e);
  if (n > 0) {
    k_iota<<<mk_grid_fit(k_iota, n, 256), 256, 0, st>>>(idx_in, n);
    if ((e = cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, ipix, keys_out, idx_in, pl->perm,
                                             (int)n, 0, end_bit, st)) != cudaSuccess)
      return fail("sort sizing", e);
    if ((e = cudaMalloc(&tmp, tmp_bytes)) != cudaSuccess) return fail("cudaMalloc", e);
    if ((e = cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, ipix, keys_out, idx_in, pl->perm,
                                             (int)n, 0, end_bit, st)) != cudaSuccess)
      return fail("sort", e);
  }
  k_pix_offsets<<<mk_grid_fit(k_pix_offsets, npix + 1, 256), 256, 0, st>>>(keys_out, n, pl->off, npix);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail("offsets", e);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail("sync", e);
  cudaFree(keys_out);
  cudaFree(idx_in);
  cudaFree(tmp);
  *plan = pl;
  return MK_OK;
}

extern "C" int mk_tod2map_sorted(void *map, const void *dat, const mk_pixplan *plan, int dtype,
                                 void *stream) {
  MK_CHECK_ARG(plan && map, "mk_tod2map_sorted: null pointer");
  MK_CHECK_ARG(MK_DTYPE_OK(dtype), "mk_tod2map_sorted: bad dtype %d", dtype);
  if (plan->n == 0) return MK_OK;
  MK_CHECK_ARG(dat, "mk_tod2map_sorted: null dat");
  cudaStream_t st = mk::as_stream(stream);
  if (dtype == MK_F64)
    k_tod2map_sorted<double><<<mk_grid_fit(k_tod2map_sorted<double>, plan->npix * 32, 256), 256, 0, st>>>((double *)map, (const double *)dat, plan->perm,
                                                 plan->off, plan->npix);
  else
    k_tod2map_sorted<float><<<mk_grid_fit(k_tod2map_sorted<float>, plan->npix * 32, 256), 256, 0, st>>>((float *)map, (const float *)dat, plan->perm,
                                                plan->off, plan->npix);
  return mk::launch_status("mk_tod2map_sorted");
}

extern "C" int mk_pixplan_destroy(mk_pixplan *plan) {
  if (!plan) return MK_OK;
  cudaFree(plan->perm);
  cudaFree(plan->off);
  delete plan;
  return MK_OK;
}

extern "C" size_t mk_tod2map_fixed_scratch_bytes(int64_t npix) {
  return sizeof(FixHdr) + (size_t)(npix > 0 ? npix : 0) * sizeof(unsigned long long);
}

extern "C" int mk_tod2map_fixed(void *map, const void *dat, const int32_t *ipix, int64_t ndet,
                                int64_t ndata, int64_t npix, int64_t hmax, int dtype, void *scratch,
                                void *stream) {
  MK_CHECK_ARG(ndet >= 0 && ndata >= 0 && npix >= 0, "mk_tod2map_fixed: negative size");
  MK_CHECK_ARG(MK_DTYPE_OK(dtype), "mk_tod2map_fixed: bad dtype %d", dtype);
  MK_CHECK_ARG(hmax >= 1, "mk_tod2map_fixed: hmax must be >= 1 (max hits of any pixel)");
  int64_t n = ndet * ndata;
  if (n == 0) return MK_OK;
  MK_CHECK_ARG(map && dat && ipix && scratch, "mk_tod2map_fixed: null pointer");
  MK_CHECK_ARG(((uintptr_t)scratch % 256) == 0, "mk_tod2map_fixed: scratch must be 256-byte aligned");
  int hbits = 0;
  while (hbits < 62 && (int64_t(1) << hbits) < hmax) hbits++;
  MK_CHECK_ARG(hbits <= 40, "mk_tod2map_fixed: hmax=%lld too large for 64-bit accumulation",
               (long long)hmax);
  cudaStream_t st = mk::as_stream(stream);
  return dtype == MK_F64 ? tod2map_fixed_t<double>(map, dat, ipix, n, npix, hbits, scratch, st)
                         : tod2map_fixed_t<float>(map, dat, ipix, n, npix, hbits, scratch, st);
}

// ---- the same scatter with library-owned scratch, for callers that cannot
// allocate device memory ----------------------------------------------------
// The accumulator lives in a file-scope device array that every GPU loading
// this library holds until the process exits: a 256-byte header plus one
// int64 per pixel for up to MK_NOALLOC_MAX_NPIX pixels (32 MiB).  It is
// zero when the module loads, and every complete call leaves it zero again.
namespace {
constexpr int64_t NOALLOC_MAX_NPIX = MK_NOALLOC_MAX_NPIX;
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(FixHdr) +
                                                                 NOALLOC_MAX_NPIX * sizeof(unsigned long long)];
std::mutex g_noalloc_mu;
void *g_noalloc_ptr[64] = {};

// Device address of g_noalloc_scratch on the current device.  The name is a
// host-side stand-in for the array, not a device address, so it is resolved
// once per device with cudaGetSymbolAddress (this device must be current).
int noalloc_scratch(void **out) {
  int dev = 0;
  MK_CUDA(cudaGetDevice(&dev));
  MK_CHECK_ARG(dev >= 0 && dev < 64, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      mk::set_error("mk_tod2map_fixed_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
      return MK_ERR_CUDA;
    }
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return MK_OK;
}
}  // namespace

extern "C" int mk_tod2map_fixed_noalloc(void *map, const void *dat, const int32_t *ipix,
                                        int64_t ndet, int64_t ndata, int64_t npix, int64_t hmax,
                                        int dtype, void *stream) {
  MK_CHECK_ARG(npix >= 0, "mk_tod2map_fixed_noalloc: negative npix=%lld", (long long)npix);
  MK_CHECK_ARG(npix <= NOALLOC_MAX_NPIX,
               "mk_tod2map_fixed_noalloc: npix=%lld exceeds the built-in scratch limit of %lld pixels "
               "(use mk_tod2map_fixed with caller scratch for larger maps)",
               (long long)npix, (long long)NOALLOC_MAX_NPIX);
  void *scratch = nullptr;
  int rc = noalloc_scratch(&scratch);
  if (rc) return rc;
  return mk_tod2map_fixed(map, dat, ipix, ndet, ndata, npix, hmax, dtype, scratch, stream);
}
