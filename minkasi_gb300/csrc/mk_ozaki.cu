// FP64 detector rotation R = A . X on the bf16 tensor cores, by exact
// integer slicing (the splitting scheme of Ozaki, Ogita, Oishi and Rump,
// "Error-free transformations of matrix multiplication by using fast
// routines of matrix multiplication and its applications", Numer. Algorithms
// 59, 2012):
//   * each row i of A is scaled by 2^-sa_i and each sample column j of X by
//     2^-sx_j (powers of two: exact), so every scaled entry is below 1;
//   * the scaled entries are truncated to 56-bit fixed point and cut into
//     S = 8 signed slices of B = 7 bits: A = 2^sa sum_p A_p 2^(-7p),
//     X = 2^sx sum_q X_q 2^(-7q), with |A_p|, |X_q| <= 127 integers, exact in
//     bf16 (whose significand holds 8 bits);
//   * A_p X_q is then an integer matrix whose entries stay below
//     K * 127^2 = 4.1e6 for K = 256 detectors, so a bf16 tensor-core GEMM
//     with FP32 accumulation computes it exactly, in any order.  Products
//     with the same p + q = t are stacked along K into one GEMM while the sum
//     stays below 2^24 (up to 4 products at K = 256): 12 GEMMs for the 36
//     products with t <= S + 1 (the dropped ones are below 2^-63 relative);
//   * the 12 FP32 results are exact integers, combined per output in int64
//     and converted to FP64 once: R = 2^(sa_i + sx_j) (hi 2^-35 + lo 2^-63).
// The error is about 2^-53 relative to the row and column scales, the same
// order as DGEMM's, at the bf16 tensor rate instead of GB300's FP64 rate.
// Columns are processed in blocks of OZ_BLOCK samples to bound the scratch.
#include <cublas_v2.h>
#include <cuda_bf16.h>

#include <vector>

#include "mk_common.cuh"
#include "mk_ozaki.cuh"

namespace mk {
namespace {

constexpr int OZ_S = 8;     // slices per operand
constexpr int OZ_B = 7;     // bits per slice
constexpr int OZ_FRAC = OZ_S * OZ_B;  // fixed-point bits of a scaled entry (56)
constexpr int OZ_NOSCALE = -100000;   // a row / column holding a non-finite value

struct SubGroup {
  int t, q0, len;  // products A_{t-q} X_q for q = q0 .. q0 + len - 1
};

// the stacked GEMMs: for t = 2 .. S + 1, the t - 1 products A_{t-q} X_q
// (q = 1 .. t - 1) in runs of at most `lmax`
std::vector<SubGroup> subgroups(int lmax) {
  std::vector<SubGroup> g;
  for (int t = 2; t <= OZ_S + 1; t++)
    for (int q0 = 1; q0 <= t - 1; q0 += lmax) {
      int len = t - 1 - q0 + 1;
      if (len > lmax) len = lmax;
      g.push_back({t, q0, len});
    }
  return g;
}

// products per GEMM so that K * len * 127^2 < 2^24
int max_stack(int64_t nrow) {
  const int64_t per = nrow * 127 * 127;
  int64_t l = ((int64_t)1 << 24) / per;
  if (l > OZ_S) l = OZ_S;
  return (int)l;
}

// exponent e with |x| < 2^e for the largest |x| given as bits; OZ_NOSCALE if
// that value is not finite; 0 for an all-zero row or column
__device__ __forceinline__ int scale_of(unsigned long long maxbits) {
  const int ef = (int)((maxbits >> 52) & 0x7FF);
  if (ef == 0x7FF) return OZ_NOSCALE;
  if (maxbits == 0) return 0;
  return ef == 0 ? -1021 : ef - 1022;
}

// 56-bit fixed point of |x| * 2^-sc (truncated) and the sign
__device__ __forceinline__ unsigned long long fixed56(double x, int sc, bool *neg) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  *neg = (b >> 63) != 0;
  const int ef = (int)((b >> 52) & 0x7FF);
  unsigned long long m = b & 0x000FFFFFFFFFFFFFull;
  if (ef) m |= 0x0010000000000000ull;
  // |x| = m 2^(E), E = (ef ? ef : 1) - 1075; F = m 2^(E + 56 - sc)
  const int sh = (ef ? ef : 1) - 1075 + OZ_FRAC - sc;
  if (sh >= 0) return sh > 3 ? 0ull : m << sh;  // |x| < 2^sc keeps sh <= 3
  return sh > -64 ? m >> (-sh) : 0ull;
}

__device__ __forceinline__ __nv_bfloat16 slice_of(unsigned long long F, bool neg, int p) {
  const int v = (int)((F >> (OZ_FRAC - OZ_B * p)) & ((1u << OZ_B) - 1));
  return __int2bfloat16_rn(neg ? -v : v);
}

// sx[j] for the columns j0 .. j0 + nb - 1 of X (nrow x ncol, ld ldx)
__global__ void k_oz_colscale(const double *__restrict__ X, int64_t ldx, int64_t nrow, int64_t j0, int64_t nb,
                              int *__restrict__ sx) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nb) return;
  unsigned long long m = 0;
  for (int64_t k = 0; k < nrow; k++) {
    const unsigned long long a =
        (unsigned long long)__double_as_longlong(X[k * ldx + j0 + j]) & 0x7FFFFFFFFFFFFFFFull;
    m = a > m ? a : m;
  }
  sx[j] = scale_of(m);
}

// Xs[(q - 1) nrow + k][j] = slice q of X[k][j0 + j] (row-major, ld nb)
__global__ void k_oz_slice_x(const double *__restrict__ X, int64_t ldx, int64_t nrow, int64_t j0, int64_t nb,
                             const int *__restrict__ sx, __nv_bfloat16 *__restrict__ Xs) {
  const int64_t n = nrow * nb;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = e / nb, j = e - k * nb;
    const int sc = sx[j];
    bool neg = false;
    const unsigned long long F = sc == OZ_NOSCALE ? 0ull : fixed56(X[k * ldx + j0 + j], sc, &neg);
#pragma unroll
    for (int q = 1; q <= OZ_S; q++) Xs[((int64_t)(q - 1) * nrow + k) * nb + j] = slice_of(F, neg, q);
  }
}

__global__ void k_oz_rowscale(const double *__restrict__ A, int64_t nrow, int *__restrict__ sa) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrow) return;
  unsigned long long m = 0;
  for (int64_t k = 0; k < nrow; k++) {
    const unsigned long long a = (unsigned long long)__double_as_longlong(A[i * nrow + k]) & 0x7FFFFFFFFFFFFFFFull;
    m = a > m ? a : m;
  }
  sa[i] = scale_of(m);
}

// the A stack of one subgroup: row-major (nrow x len nrow), column block c
// holds slice t - (q0 + c) of A
__global__ void k_oz_stack_a(const double *__restrict__ A, int64_t nrow, const int *__restrict__ sa, int t, int q0,
                             int len, __nv_bfloat16 *__restrict__ As) {
  const int64_t kk = (int64_t)len * nrow, n = nrow * kk;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / kk, c = e - i * kk;
    const int q = q0 + (int)(c / nrow), k = (int)(c - (int64_t)(q - q0) * nrow);
    const int sc = sa[i];
    bool neg = false;
    const unsigned long long F = sc == OZ_NOSCALE ? 0ull : fixed56(A[i * nrow + k], sc, &neg);
    As[e] = slice_of(F, neg, t - q);
  }
}

// R[i][j0 + j] = 2^(sa_i + sx_j) sum_g G_g[i][j] 2^(-7 t_g), exactly in int64:
// t <= 5 go to hi (weights 2^(7 (5 - t))), t >= 6 to lo (2^(7 (9 - t))), so
// R = 2^(sa + sx) (hi 2^-35 + lo 2^-63).  Each G is an integer below 2^24.
struct GroupT {  // slice-index sum t of each stacked GEMM (kernel parameter: no copy)
  int n;
  int t[64];
};

__global__ void k_oz_combine(const float *__restrict__ G, const GroupT gt, int64_t nrow,
                             int64_t nb, const int *__restrict__ sa, const int *__restrict__ sx, double *__restrict__ R,
                             int64_t ldr, int64_t j0) {
  const int64_t n = nrow * nb, gs = nrow * nb;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / nb, j = e - i * nb;
    long long hi = 0, lo = 0;
    for (int g = 0; g < gt.n; g++) {
      const long long v = (long long)G[g * gs + e];
      const int t = gt.t[g];
      if (t <= 5)
        hi += v * (1ll << (OZ_B * (5 - t)));
      else
        lo += v * (1ll << (OZ_B * (9 - t)));
    }
    const int a = sa[i], c = sx[j];
    double r;
    if (a == OZ_NOSCALE || c == OZ_NOSCALE)
      r = __longlong_as_double(0x7FF8000000000000ll);  // NaN, as the FP64 product of a non-finite entry
    else
      r = ldexp(fma((double)hi, 0x1p-35, (double)lo * 0x1p-63), a + c);
    R[i * ldr + j0 + j] = r;
  }
}

size_t al256(size_t x) { return (x + 255) / 256 * 256; }

struct Layout {
  size_t sa, as, sx, xs, g, total;
  std::vector<SubGroup> groups;
  std::vector<size_t> as_off;
};

Layout layout(int64_t nrow) {
  Layout L;
  L.groups = subgroups(max_stack(nrow));
  size_t o = 0;
  L.sa = o;
  o += al256((size_t)nrow * sizeof(int));
  L.as = o;
  for (const auto &g : L.groups) {
    L.as_off.push_back(o);
    o += al256((size_t)nrow * g.len * nrow * sizeof(__nv_bfloat16));
  }
  L.sx = o;
  o += al256((size_t)OZ_BLOCK * sizeof(int));
  L.xs = o;
  o += al256((size_t)OZ_S * nrow * OZ_BLOCK * sizeof(__nv_bfloat16));
  L.g = o;
  o += al256((size_t)L.groups.size() * nrow * OZ_BLOCK * sizeof(float));
  L.total = o;
  return L;
}

}  // namespace

bool ozaki_supported(int64_t nrow) { return nrow >= 1 && max_stack(nrow) >= 1; }

size_t ozaki_ws_bytes(int64_t nrow) { return ozaki_supported(nrow) ? layout(nrow).total : 0; }

int ozaki_rotate_f64(cublasHandle_t h, const double *A, const double *X, int64_t ldx, double *R, int64_t ldr,
                     int64_t nrow, int64_t ncol, void *ws, size_t ws_bytes, cudaStream_t st) {
  MK_CHECK_ARG(ozaki_supported(nrow), "sliced FP64 rotation: ndet %lld too large for exact FP32 sums",
               (long long)nrow);
  const Layout L = layout(nrow);
  MK_CHECK_ARG(ws && ws_bytes >= L.total && ((uintptr_t)ws % 256) == 0,
               "sliced FP64 rotation: workspace too small (%zu < %zu)", ws_bytes, L.total);
  if (ncol <= 0) return MK_OK;
  char *w = (char *)ws;
  int *sa = (int *)(w + L.sa), *sx = (int *)(w + L.sx);
  __nv_bfloat16 *Xs = (__nv_bfloat16 *)(w + L.xs);
  float *G = (float *)(w + L.g);
  const int ng = (int)L.groups.size();
  GroupT gt{};
  gt.n = ng;
  for (int g = 0; g < ng && g < 64; g++) gt.t[g] = L.groups[g].t;
  k_oz_rowscale<<<(unsigned)((nrow + 127) / 128), 128, 0, st>>>(A, nrow, sa);
  for (int g = 0; g < ng; g++) {
    const SubGroup &s = L.groups[g];
    const int64_t n = nrow * s.len * nrow;
    k_oz_stack_a<<<mk_grid(n, 256, 8), 256, 0, st>>>(A, nrow, sa, s.t, s.q0, s.len,
                                                     (__nv_bfloat16 *)(w + L.as_off[g]));
  }
  int rc = launch_status("sliced FP64 rotation: A slices");
  if (rc) return rc;
  cublasSetStream(h, st);
  cublasSetMathMode(h, CUBLAS_DEFAULT_MATH);
  cublasSetEmulationStrategy(h, CUBLAS_EMULATION_STRATEGY_DEFAULT);
  const float one = 1.f, zero = 0.f;
  for (int64_t j0 = 0; j0 < ncol; j0 += OZ_BLOCK) {
    const int64_t nb = ncol - j0 < OZ_BLOCK ? ncol - j0 : OZ_BLOCK;
    k_oz_colscale<<<(unsigned)((nb + 255) / 256), 256, 0, st>>>(X, ldx, nrow, j0, nb, sx);
    k_oz_slice_x<<<mk_grid(nrow * nb, 256, 8), 256, 0, st>>>(X, ldx, nrow, j0, nb, sx, Xs);
    if ((rc = launch_status("sliced FP64 rotation: X slices"))) return rc;
    for (int g = 0; g < ng; g++) {
      const SubGroup &s = L.groups[g];
      // column-major: G_g (nb x nrow) = Xs[q0 ..] (nb x len nrow) . As_g (len nrow x nrow)
      const int64_t kk = (int64_t)s.len * nrow;
      const __nv_bfloat16 *xq = Xs + (int64_t)(s.q0 - 1) * nrow * nb;
      cublasStatus_t cs = cublasGemmEx_64(h, CUBLAS_OP_N, CUBLAS_OP_N, nb, nrow, kk, &one, xq, CUDA_R_16BF, nb,
                                          w + L.as_off[g], CUDA_R_16BF, kk, &zero, G + (int64_t)g * nrow * nb,
                                          CUDA_R_32F, nb, CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT);
      if (cs != CUBLAS_STATUS_SUCCESS) {
        set_error("sliced FP64 rotation: bf16 GEMM failed (status %d)", (int)cs);
        return MK_ERR_CUBLAS;
      }
    }
    k_oz_combine<<<mk_grid(nrow * nb, 256, 8), 256, 0, st>>>(G, gt, nrow, nb, sa, sx, R, ldr, j0);
    if ((rc = launch_status("sliced FP64 rotation: combine"))) return rc;
  }
  return MK_OK;
}

}  // namespace mk
