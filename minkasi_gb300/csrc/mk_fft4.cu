// FP32 DCT-I by a four-step FFT in shared memory (see mk_fft4.cuh).
#include <cufft.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <utility>
#include <vector>

#include "mk_async.cuh"
#include "mk_common.cuh"
#include "mk_fft4.cuh"

namespace mk {
namespace {

constexpr int FB = 8;  // transforms per CTA (consecutive j1 in pass A, k2 in pass B)
constexpr int NT = 256;
constexpr int WR3 = 0, WR5 = 3, WR7 = 8, WR9 = 15, WR11 = 24, WRN = 35;  // offsets into the radix constants

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// -i z
__device__ __forceinline__ float2 mul_mi(float2 z) { return make_float2(z.y, -z.x); }

// forward DFT of R points in registers: v_q <- sum_r v_r W_R^{rq}
template <int R>
struct Dft;

template <>
struct Dft<2> {
  __device__ static void run(float2 *v, const float2 *) {
    const float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};

template <>
struct Dft<4> {
  __device__ static void run(float2 *v, const float2 *) {
    const float2 s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
    const float2 s13 = cadd(v[1], v[3]), d13 = csub(v[1], v[3]);
    v[0] = cadd(s02, s13);
    v[2] = csub(s02, s13);
    v[1] = cadd(d02, mul_mi(d13));
    v[3] = csub(d02, mul_mi(d13));
  }
};

template <>
struct Dft<8> {
  __device__ static void run(float2 *v, const float2 *) {
    float2 e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
    Dft<4>::run(e, nullptr);
    Dft<4>::run(o, nullptr);
    const float h = 0.70710678118654752f;
    // o_k *= W_8^k
    o[1] = make_float2(h * (o[1].x + o[1].y), h * (o[1].y - o[1].x));
    o[2] = mul_mi(o[2]);
    o[3] = make_float2(h * (o[3].y - o[3].x), -h * (o[3].x + o[3].y));
#pragma unroll
    for (int k = 0; k < 4; k++) {
      v[k] = cadd(e[k], o[k]);
      v[k + 4] = csub(e[k], o[k]);
    }
  }
};

// odd R: pair r with R - r; wr[t] = W_R^t = (cos 2pi t/R, -sin 2pi t/R)
template <int R, int OFF>
struct DftOdd {
  __device__ static void run(float2 *v, const float2 *wr) {
    constexpr int H = (R - 1) / 2;
    float2 s[H + 1], d[H + 1];
    float2 x0 = v[0];
#pragma unroll
    for (int r = 1; r <= H; r++) {
      s[r] = cadd(v[r], v[R - r]);
      d[r] = csub(v[r], v[R - r]);
      x0 = cadd(x0, s[r]);
    }
    float2 out[R];
    out[0] = x0;
#pragma unroll
    for (int q = 1; q <= H; q++) {
      float2 A = v[0], B = make_float2(0.f, 0.f);
#pragma unroll
      for (int r = 1; r <= H; r++) {
        const float2 w = wr[OFF + (r * q) % R];
        const float c = w.x, sn = -w.y;
        A.x = fmaf(s[r].x, c, A.x);
        A.y = fmaf(s[r].y, c, A.y);
        B.x = fmaf(d[r].x, sn, B.x);
        B.y = fmaf(d[r].y, sn, B.y);
      }
      out[q] = make_float2(A.x + B.y, A.y - B.x);
      out[R - q] = make_float2(A.x - B.y, A.y + B.x);
    }
#pragma unroll
    for (int q = 0; q < R; q++) v[q] = out[q];
  }
};
template <>
struct Dft<3> : DftOdd<3, WR3> {};
template <>
struct Dft<5> : DftOdd<5, WR5> {};
template <>
struct Dft<7> : DftOdd<7, WR7> {};
template <>
struct Dft<9> : DftOdd<9, WR9> {};
template <>
struct Dft<11> : DftOdd<11, WR11> {};

// 4-byte asynchronous global -> shared copy; !valid zero-fills
// (src must still be a mapped address)
__device__ __forceinline__ void cp4(void *dst, const void *src, bool valid) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(valid ? 4 : 0)
               : "memory");
}

struct WrTable {
  float2 w[WRN];
};

// Stage indexing shared by both passes: butterfly q of a stage with span Ns
// is group g = q / Ns, offset k = q % Ns.  The division is done as
// trunc((q + 1/2) / Ns) in FP32: q < 1536 and Ns <= 1536, so (q + 1/2) / Ns
// lies at least 1/(2 Ns) from an integer, far above the rounding error of
// the product (checked exhaustively for all q, Ns < 2048).

// ---- pass A ------------------------------------------------------------
// The 8 transforms of the CTA (8 consecutive j1) are interleaved over the
// threads for the stages (row b = bf % 8): the first stage reads its inputs
// straight from the detector rows (8 lanes, 8 consecutive samples), forming
// the even extension; the stages run in shared memory with CTA barriers.
// Then warp b twiddles row b by W_L^{j1 k2} and stores it to T.
// what pass A's first stage reads: the rows' even extension (DCT), the same
// times the Bluestein chirp (zero past 2m), or a complex sequence (U)
enum { AM_DCT = 0, AM_BLUE = 1, AM_CPLX = 2 };

struct PassA {
  const float *x1, *x2;
  const float2 *U;  // AM_CPLX: this pair's sequence
  const float2 *chirp;
  bool has2;
  int L1, j1_0, nb, m, Lx, M;
  const int *iperm;
};

// input at position j: the even extension e_j (AM_DCT, j < 2m); for
// Bluestein, z_{|i|} c_{|i|} at the position j = i mod M of i in [-m + 1, m]
// and zero in between; or the sequence U
template <int AM>
__device__ __forceinline__ float2 a_input(const PassA &pa, int j) {
  if (AM == AM_CPLX) return pa.U[j];
  if (AM == AM_BLUE && j > pa.m && j <= pa.M - pa.m) return make_float2(0.f, 0.f);
  const int jj = j <= pa.m ? j : (AM == AM_BLUE ? pa.M : pa.Lx) - j;
  const float2 z = make_float2(__ldg(pa.x1 + jj), pa.has2 ? __ldg(pa.x2 + jj) : 0.f);
  return AM == AM_BLUE ? cmul(z, __ldg(pa.chirp + jj)) : z;
}

template <int R, bool FIRST, int AM>
__device__ __forceinline__ void astage(float2 *sbuf, int pitch, int Ls, int Ns, float invNs, const float2 *stw,
                                       const float2 *wr, const PassA &pa) {
  const int nq = Ls / R;
  for (int bf = threadIdx.x; bf < FB * nq; bf += NT) {
    const int b = bf % FB, q = bf / FB;
    if (b >= pa.nb) continue;
    const int g = __float2int_rz(((float)q + 0.5f) * invNs);
    const int k = q - g * Ns;
    float2 v[R];
    float2 *a = sbuf + b * pitch + g * Ns * R + k;
    if (FIRST) {  // Ns == 1
      const int jg = __ldg(pa.iperm + q * R);
#pragma unroll
      for (int r = 0; r < R; r++) v[r] = a_input<AM>(pa, pa.j1_0 + b + pa.L1 * (jg + (Ls / R) * r));
    } else {
#pragma unroll
      for (int r = 0; r < R; r++) v[r] = a[r * Ns];
      if (Ns > 1) {
#pragma unroll
        for (int r = 1; r < R; r++) v[r] = cmul(v[r], __ldg(stw + (r - 1) * Ns + k));
      }
    }
    Dft<R>::run(v, wr);
#pragma unroll
    for (int r = 0; r < R; r++) a[r * Ns] = v[r];
  }
}

template <bool FIRST, int AM>
__device__ __forceinline__ void astage_r(int R, float2 *sbuf, int pitch, int Ls, int Ns, float invNs,
                                         const float2 *stw, const float2 *wr, const PassA &pa) {
  switch (R) {
    case 2: astage<2, FIRST, AM>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pa); break;
    case 3: astage<3, FIRST, AM>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pa); break;
    case 4: astage<4, FIRST, AM>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pa); break;
    case 5: astage<5, FIRST, AM>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pa); break;
    case 7: astage<7, FIRST, AM>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pa); break;
    case 8: astage<8, FIRST, AM>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pa); break;
    case 9: astage<9, FIRST, AM>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pa); break;
    default: astage<11, FIRST, AM>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pa); break;
  }
}

// row pitch (float2) of a tile of 8 interleaved transforms: odd, so the 8
// rows fall in distinct shared-memory banks
__host__ __device__ __forceinline__ int pitch_odd(int Ls) { return Ls | 1; }

// pass A: rows (2 pair, 2 pair + 1) of x (or the pair's U) -> T[pair]
// (L1 x L2, twiddled)
template <int AM>
__global__ void __launch_bounds__(NT) k_fft4_a(const float *__restrict__ x, int64_t ldx, const float2 *__restrict__ U,
                                               int64_t nrow, float2 *__restrict__ T, const Fft4Dev p,
                                               const WrTable wt) {
  extern __shared__ float2 sbuf[];
  const int L1 = p.L1, L2 = p.L2, pitch = pitch_odd(L2), tid = threadIdx.x;
  const int64_t pair = blockIdx.y, r0 = 2 * pair;
  PassA pa;
  pa.has2 = r0 + 1 < nrow;
  pa.x1 = AM == AM_CPLX ? nullptr : x + r0 * ldx;
  pa.x2 = AM == AM_CPLX ? nullptr : pa.has2 ? pa.x1 + ldx : pa.x1;
  pa.U = AM == AM_CPLX ? U + pair * p.L : nullptr;
  pa.chirp = p.chirp;
  pa.L1 = L1;
  pa.j1_0 = blockIdx.x * FB;
  pa.nb = min(FB, L1 - pa.j1_0);
  pa.m = (int)p.m;
  pa.Lx = (int)p.Lx;
  pa.M = (int)p.L;
  pa.iperm = p.iperm2;
  const int S = p.nr2;
  if (S == 0) {  // L2 == 1: the column is its own transform
    if (tid < pa.nb) sbuf[tid * pitch] = a_input<AM>(pa, pa.j1_0 + tid);
  } else {
    astage_r<true, AM>(p.r2[0], sbuf, pitch, L2, 1, 1.0f, p.stw2, wt.w, pa);
    for (int s = 1; s < S; s++) {
      __syncthreads();
      astage_r<false, AM>(p.r2[s], sbuf, pitch, L2, p.ns2[s], p.inv2[s], p.stw2 + p.to2[s], wt.w, pa);
    }
  }
  __syncthreads();
  // warp b twiddles row b by W_L^{j1 k2} and stores it
  const int warp = tid >> 5, lane = tid & 31;
  if (warp >= pa.nb) return;
  const float2 *row = sbuf + warp * pitch;
  const int j1 = pa.j1_0 + warp;
  const float2 tl = __ldg(p.tlane + 32 * j1 + lane);
  const float2 *tb = p.tblk + j1 * p.nb32;
  float2 *Tp = T + pair * p.L + j1 * L2;
  for (int i = 0; i < p.nb32; i++) {
    const int k2 = 32 * i + lane;
    if (k2 < L2) Tp[k2] = cmul(row[k2], cmul(__ldg(tb + i), tl));
  }
}

// ---- pass B ------------------------------------------------------------
// The CTA's 8 transforms (8 consecutive k2) are interleaved over the threads:
// butterfly bf of a stage belongs to row b = bf % 8, so the 8 lanes of a row
// group read or write 8 consecutive columns of T / of the output.  The first
// stage reads its inputs straight from T (natural order: position g R0 + r of
// the digit-reversed layout holds index iperm[g R0] + (L1 / R0) r), and the
// last stage writes its outputs straight to the DCT rows with the epilogue.
// what pass B's last stage writes: DCT rows (k <= m, epilogue), the
// Bluestein product U = conj(F B^) (all k), or the Bluestein result
// c_k conj(F_k) as DCT rows
enum { BM_DCT = 0, BM_MUL = 1, BM_BLUE = 2 };

struct PassB {
  const float2 *Tp;  // this pair's T (L1 x L2)
  float2 *U;         // BM_MUL: this pair's output sequence
  const float2 *bhat, *chirp;
  int L2, k2_0, nb, m, epi;
  bool has2;
  float *o1, *o2;
  const float *sw;  // prefetched weights, [k1][b][row]
  const int *iperm;
};

template <int R, bool FIRST, bool LAST, int BM>
__device__ __forceinline__ void bstage(float2 *sbuf, int pitch, int Ls, int Ns, float invNs, const float2 *stw,
                                       const float2 *wr, const PassB &pb) {
  const int nq = Ls / R;
  for (int bf = threadIdx.x; bf < FB * nq; bf += NT) {
    const int b = bf % FB, q = bf / FB;
    if (b >= pb.nb) continue;
    const int g = __float2int_rz(((float)q + 0.5f) * invNs);
    const int k = q - g * Ns;
    float2 v[R];
    if (FIRST) {  // Ns == 1: g == q, k == 0
      const int jg = __ldg(pb.iperm + q * R);
#pragma unroll
      for (int r = 0; r < R; r++) v[r] = pb.Tp[(jg + (Ls / R) * r) * pb.L2 + pb.k2_0 + b];
    } else {
      const float2 *a = sbuf + b * pitch + g * Ns * R + k;
#pragma unroll
      for (int r = 0; r < R; r++) v[r] = a[r * Ns];
      if (Ns > 1) {
#pragma unroll
        for (int r = 1; r < R; r++) v[r] = cmul(v[r], __ldg(stw + (r - 1) * Ns + k));
      }
    }
    Dft<R>::run(v, wr);
    if (LAST) {
#pragma unroll
      for (int r = 0; r < R; r++) {
        const int k1 = g * Ns * R + k + r * Ns;
        const int kk = pb.k2_0 + b + pb.L2 * k1;
        if (BM == BM_MUL) {
          const float2 f = cmul(v[r], __ldg(pb.bhat + kk));
          pb.U[kk] = make_float2(f.x, -f.y);
          continue;
        }
        if (kk > pb.m) continue;
        if (BM == BM_BLUE) v[r] = cmul(make_float2(v[r].x, -v[r].y), __ldg(pb.chirp + kk));
        float a = v[r].x, c = v[r].y;
        if (pb.epi == FFT4_FILTER) {
          a *= pb.sw[2 * (k1 * FB + b)];
          c *= pb.sw[2 * (k1 * FB + b) + 1];
        } else if (pb.epi == FFT4_HALVE && (kk == 0 || kk == pb.m)) {
          a *= 0.5f;
          c *= 0.5f;
        }
        pb.o1[kk] = a;
        if (pb.has2) pb.o2[kk] = c;
      }
    } else {
      float2 *a = sbuf + b * pitch + g * Ns * R + k;
#pragma unroll
      for (int r = 0; r < R; r++) a[r * Ns] = v[r];
    }
  }
}

template <bool FIRST, bool LAST, int BM>
__device__ __forceinline__ void bstage_r(int R, float2 *sbuf, int pitch, int Ls, int Ns, float invNs,
                                         const float2 *stw, const float2 *wr, const PassB &pb) {
  switch (R) {
    case 2: bstage<2, FIRST, LAST, BM>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pb); break;
    case 3: bstage<3, FIRST, LAST, BM>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pb); break;
    case 4: bstage<4, FIRST, LAST, BM>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pb); break;
    case 5: bstage<5, FIRST, LAST, BM>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pb); break;
    case 7: bstage<7, FIRST, LAST, BM>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pb); break;
    case 8: bstage<8, FIRST, LAST, BM>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pb); break;
    case 9: bstage<9, FIRST, LAST, BM>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pb); break;
    default: bstage<11, FIRST, LAST, BM>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pb); break;
  }
}

// pass B: T[pair] -> DCT rows 2 pair, 2 pair + 1 of out (k <= m) with the
// epilogue, or (BM_MUL) -> the pair's U
template <int BM>
__global__ void __launch_bounds__(NT) k_fft4_b(const float2 *__restrict__ T, int64_t nrow, float *__restrict__ out,
                                               int64_t ldo, float2 *__restrict__ U, const float *__restrict__ w,
                                               int64_t ldw, int epi, const Fft4Dev p, const WrTable wt) {
  extern __shared__ float2 sbuf[];
  const int L1 = p.L1, L2 = p.L2, pitch = pitch_odd(L1), tid = threadIdx.x;
  const int64_t pair = blockIdx.y, r0 = 2 * pair;
  PassB pb;
  pb.has2 = r0 + 1 < nrow;
  pb.k2_0 = blockIdx.x * FB;
  pb.nb = min(FB, L2 - pb.k2_0);
  pb.Tp = T + pair * p.L;
  pb.U = BM == BM_MUL ? U + pair * p.L : nullptr;
  pb.bhat = p.bhat;
  pb.chirp = p.chirp;
  pb.L2 = L2;
  pb.m = (int)p.m;
  pb.epi = epi;
  pb.o1 = BM == BM_MUL ? nullptr : out + r0 * ldo;
  pb.o2 = BM == BM_MUL ? nullptr : pb.o1 + ldo;
  pb.iperm = p.iperm1;
  // the weights of this tile's outputs, [k1][b][row], prefetched during the
  // first stages
  float *sw = reinterpret_cast<float *>(sbuf + FB * pitch);
  pb.sw = sw;
  if (BM != BM_MUL && epi == FFT4_FILTER) {
    const float *w1 = w + r0 * ldw;
    const float *w2 = pb.has2 ? w1 + ldw : w1;
#pragma unroll 4
    for (int idx = tid; idx < FB * L1; idx += NT) {
      const int b = idx % FB, k1 = idx / FB;
      const int k = pb.k2_0 + b + L2 * k1;
      const bool ok = b < pb.nb && k <= pb.m;
      cp4(sw + 2 * idx, ok ? w1 + k : w1, ok);
      cp4(sw + 2 * idx + 1, ok ? w2 + k : w1, ok && pb.has2);
    }
  }
  const int S = p.nr1;
  if (S == 1) {
    cp_async_wait_all();
    __syncthreads();
    bstage_r<true, true, BM>(p.r1[0], sbuf, pitch, L1, 1, 1.0f, p.stw1, wt.w, pb);
    return;
  }
  bstage_r<true, false, BM>(p.r1[0], sbuf, pitch, L1, 1, 1.0f, p.stw1, wt.w, pb);
  __syncthreads();
  for (int s = 1; s < S - 1; s++) {
    bstage_r<false, false, BM>(p.r1[s], sbuf, pitch, L1, p.ns1[s], p.inv1[s], p.stw1 + p.to1[s], wt.w, pb);
    __syncthreads();
  }
  cp_async_wait_all();
  __syncthreads();
  bstage_r<false, true, BM>(p.r1[S - 1], sbuf, pitch, L1, p.ns1[S - 1], p.inv1[S - 1], p.stw1 + p.to1[S - 1],
                            wt.w, pb);
}

void factor(int64_t L, std::vector<int> &f) {
  for (int pr : {2, 3, 5, 7, 11})
    while (L % pr == 0) {
      f.push_back(pr);
      L /= pr;
    }
  if (L != 1) f.clear();
}

// radices of a transform of length Ls (a product of 2, 3, 5, 7, 11): odd
// ones first (the stride-1 first stage is then free of bank conflicts), 3 x 3
// as 9, powers of 2 as 8, 4, 2
bool radices(int Ls, int *r, int *nr) {
  std::vector<int> f;
  factor(Ls, f);
  if (f.empty() && Ls != 1) return false;
  int c[12] = {0};
  for (int x : f) c[x]++;
  std::vector<int> out;
  for (int i = 0; i < c[11]; i++) out.push_back(11);
  for (; c[3] >= 2; c[3] -= 2) out.push_back(9);
  for (int i = 0; i < c[7]; i++) out.push_back(7);
  for (int i = 0; i < c[5]; i++) out.push_back(5);
  if (c[3]) out.push_back(3);
  for (; c[2] >= 3; c[2] -= 3) out.push_back(8);
  if (c[2] == 2) out.push_back(4);
  if (c[2] == 1) out.push_back(2);
  if ((int)out.size() > FFT4_MAXR) return false;
  for (size_t i = 0; i < out.size(); i++) r[i] = out[i];
  *nr = (int)out.size();
  return true;
}

size_t al(size_t x) { return (x + 255) / 256 * 256; }

struct TableLayout {
  size_t stw1, stw2, iperm1, iperm2, tlane, tblk, chirp, bhat, total;
};

TableLayout layout(const Fft4Dev &d) {
  TableLayout t;
  size_t o = 0;
  t.stw1 = o;
  o += al((size_t)d.L1 * sizeof(float2));
  t.stw2 = o;
  o += al((size_t)d.L2 * sizeof(float2));
  t.iperm1 = o;
  o += al((size_t)d.L1 * sizeof(int));
  t.iperm2 = o;
  o += al((size_t)d.L2 * sizeof(int));
  t.tlane = o;
  o += al((size_t)d.L1 * 32 * sizeof(float2));
  t.tblk = o;
  o += al((size_t)d.L1 * d.nb32 * sizeof(float2));
  t.chirp = o;
  o += d.blue ? al((size_t)(d.m + 1) * sizeof(float2)) : 0;
  t.bhat = o;
  o += d.blue ? al((size_t)d.L * sizeof(float2)) : 0;
  t.total = o;
  return t;
}

float2 unit(double num, double den) {
  // exp(-2 pi i num / den) in double, rounded
  const double a = 2.0 * M_PI * num / den;
  return make_float2((float)std::cos(a), (float)-std::sin(a));
}

void digit_rev(int Ls, const int *r, int nr, int *P) {
  std::vector<int> d(nr > 0 ? nr : 1);
  for (int j = 0; j < Ls; j++) {
    int q = j;
    for (int i = nr - 1; i >= 0; i--) {
      d[i] = q % r[i];
      q /= r[i];
    }
    int pos = 0, span = 1;
    for (int i = 0; i < nr; i++) {
      pos += d[i] * span;
      span *= r[i];
    }
    P[j] = pos;
  }
}

WrTable radix_constants() {
  WrTable t;
  const int rs[5] = {3, 5, 7, 9, 11}, off[5] = {WR3, WR5, WR7, WR9, WR11};
  for (int i = 0; i < 5; i++)
    for (int k = 0; k < rs[i]; k++) t.w[off[i] + k] = unit(k, rs[i]);
  return t;
}

bool g_attr[64] = {false};

}  // namespace

// Which L1 x L2 split new plans take: 0 = the divisor pair closest to
// sqrt(L), r = the r-th next closest (the last one when there are fewer).
// Set by the autotuner around plan creation; a plan keeps its split.
static std::atomic<int> g_split_rank{0};
void fft4_set_split_rank(int r) { g_split_rank.store(r < 0 ? 0 : r); }
int fft4_split_rank() { return g_split_rank.load(); }

// L1 x L2 split of a transform of length L (by g_split_rank among the
// divisor pairs with both parts <= LMAX and L1 > 1, ordered by closeness to
// sqrt(L)), radices and stage constants
static bool split_len(int64_t L, Fft4Dev *t) {
  if (L < 2 || L > (int64_t)FFT4_LMAX * FFT4_LMAX) return false;
  std::vector<int> f;
  factor(L, f);
  if (f.empty()) return false;
  std::vector<int64_t> ds{1};
  for (int pr : f) {
    const size_t k = ds.size();
    for (size_t i = 0; i < k; i++) {
      const int64_t v = ds[i] * pr;
      bool seen = false;
      for (int64_t u : ds) seen |= (u == v);
      if (!seen) ds.push_back(v);
    }
  }
  std::vector<std::pair<double, int64_t>> cand;
  for (int64_t a : ds) {
    const int64_t b = L / a;
    if (a > FFT4_LMAX || b > FFT4_LMAX || a == 1) continue;  // pass B needs at least one stage
    cand.push_back({std::fabs(std::log((double)a) - std::log((double)b)), a});
  }
  if (cand.empty()) return false;
  std::sort(cand.begin(), cand.end());
  const size_t rank = (size_t)g_split_rank.load();
  const int64_t best = cand[rank < cand.size() ? rank : cand.size() - 1].second;
  t->L = L;
  t->L1 = (int)best;
  t->L2 = (int)(L / best);
  if (!radices(t->L1, t->r1, &t->nr1) || !radices(t->L2, t->r2, &t->nr2)) return false;
  t->nb32 = (t->L2 + 31) / 32;
  for (int pass = 0; pass < 2; pass++) {
    const int nr = pass ? t->nr2 : t->nr1;
    const int *r = pass ? t->r2 : t->r1;
    int *ns = pass ? t->ns2 : t->ns1, *to = pass ? t->to2 : t->to1;
    float *inv = pass ? t->inv2 : t->inv1;
    int span = 1, off = 0;
    for (int s = 0; s < nr; s++) {
      ns[s] = span;
      to[s] = off;
      inv[s] = 1.0f / (float)span;
      off += (r[s] - 1) * span;
      span *= r[s];
    }
  }
  return true;
}

bool fft4_shape(int64_t n, Fft4Dev *d, bool bluestein) {
  if (n < 2 || n > (int64_t)FFT4_LMAX * FFT4_LMAX / 2) return false;
  Fft4Dev t{};
  t.n = n;
  t.m = n - 1;
  t.Lx = 2 * t.m;
  if (split_len(t.Lx, &t)) {
    t.blue = false;
    *d = t;
    return true;
  }
  if (!bluestein) return false;
  for (int64_t M = 3 * t.m; M <= (int64_t)FFT4_LMAX * FFT4_LMAX; M++) {
    if (split_len(M, &t)) {
      t.blue = true;
      *d = t;
      return true;
    }
  }
  return false;
}

size_t fft4_table_bytes(const Fft4Dev &d) { return layout(d).total; }

size_t fft4_t_bytes(const Fft4Dev &d, int64_t nrow) {
  return (d.blue ? 2 : 1) * (size_t)((nrow + 1) / 2) * (size_t)d.L * sizeof(float2);
}

// B^ = DFT_M(b) / M with b_t = conj(c_t) at t mod M for t in [-m, 2m - 1]
// (M >= 3m keeps those positions distinct), in double precision through a
// cuFFT Z2Z transform, rounded to float
static int bluestein_bhat(const Fft4Dev &d, float2 *out) {
  const int64_t M = d.L, Lx = d.Lx, m = d.m;
  std::vector<cufftDoubleComplex> b((size_t)M);
  for (auto &v : b) v.x = v.y = 0.0;
  for (int64_t t = 0; t < 2 * m; t++) {
    const double a = M_PI * (double)((t * t) % (2 * Lx)) / (double)Lx;  // conj(c_t) = exp(+i a)
    b[(size_t)t].x = std::cos(a);
    b[(size_t)t].y = std::sin(a);
    if (t > 0 && t <= m) b[(size_t)(M - t)] = b[(size_t)t];
  }
  cufftDoubleComplex *db = nullptr;
  MK_CUDA(cudaMalloc(&db, (size_t)M * sizeof(cufftDoubleComplex)));
  int rc = MK_OK;
  cufftHandle h = 0;
  if (cudaMemcpy(db, b.data(), (size_t)M * sizeof(cufftDoubleComplex), cudaMemcpyHostToDevice) != cudaSuccess ||
      cufftPlan1d(&h, (int)M, CUFFT_Z2Z, 1) != CUFFT_SUCCESS ||
      cufftExecZ2Z(h, db, db, CUFFT_FORWARD) != CUFFT_SUCCESS ||
      cudaMemcpy(b.data(), db, (size_t)M * sizeof(cufftDoubleComplex), cudaMemcpyDeviceToHost) != cudaSuccess) {
    set_error("fft4: Bluestein kernel transform (M = %lld) failed", (long long)M);
    rc = MK_ERR_CUFFT;
  }
  if (h) cufftDestroy(h);
  cudaFree(db);
  if (rc) return rc;
  for (int64_t k = 0; k < M; k++)
    out[k] = make_float2((float)(b[(size_t)k].x / (double)M), (float)(b[(size_t)k].y / (double)M));
  return MK_OK;
}

int fft4_init(Fft4Plan *p, int64_t n, void *dev_tables, bool bluestein) {
  MK_CHECK_ARG(fft4_shape(n, &p->d, bluestein), "fft4: row length %lld has no supported factorisation",
               (long long)n);
  Fft4Dev &d = p->d;
  const TableLayout t = layout(d);
  std::vector<char> h(t.total, 0);
  for (int pass = 0; pass < 2; pass++) {
    const int nr = pass ? d.nr2 : d.nr1;
    const int *r = pass ? d.r2 : d.r1, *ns = pass ? d.ns2 : d.ns1, *to = pass ? d.to2 : d.to1;
    float2 *stw = (float2 *)(h.data() + (pass ? t.stw2 : t.stw1));
    for (int s = 0; s < nr; s++)
      for (int rr = 1; rr < r[s]; rr++)
        for (int k = 0; k < ns[s]; k++) stw[to[s] + (rr - 1) * ns[s] + k] = unit((double)rr * k, (double)ns[s] * r[s]);
  }
  {
    std::vector<int> P1(d.L1), P2(d.L2);
    digit_rev(d.L1, d.r1, d.nr1, P1.data());
    digit_rev(d.L2, d.r2, d.nr2, P2.data());
    int *I1 = (int *)(h.data() + t.iperm1), *I2 = (int *)(h.data() + t.iperm2);
    for (int j = 0; j < d.L1; j++) I1[P1[j]] = j;
    for (int j = 0; j < d.L2; j++) I2[P2[j]] = j;
  }
  float2 *tlane = (float2 *)(h.data() + t.tlane), *tblk = (float2 *)(h.data() + t.tblk);
  for (int64_t j1 = 0; j1 < d.L1; j1++) {
    for (int l = 0; l < 32; l++) tlane[32 * j1 + l] = unit((double)(j1 * l % d.L), (double)d.L);
    for (int i = 0; i < d.nb32; i++) tblk[j1 * d.nb32 + i] = unit((double)(j1 * 32 * i % d.L), (double)d.L);
  }
  if (d.blue) {
    float2 *chirp = (float2 *)(h.data() + t.chirp);
    for (int64_t j = 0; j <= d.m; j++) chirp[j] = unit((double)((j * j) % (2 * d.Lx)), 2.0 * (double)d.Lx);
    const int rc = bluestein_bhat(d, (float2 *)(h.data() + t.bhat));
    if (rc) return rc;
  }
  MK_CUDA(cudaMemcpy(dev_tables, h.data(), t.total, cudaMemcpyHostToDevice));
  char *b = (char *)dev_tables;
  d.stw1 = (const float2 *)(b + t.stw1);
  d.stw2 = (const float2 *)(b + t.stw2);
  d.iperm1 = (const int *)(b + t.iperm1);
  d.iperm2 = (const int *)(b + t.iperm2);
  d.tlane = (const float2 *)(b + t.tlane);
  d.tblk = (const float2 *)(b + t.tblk);
  d.chirp = d.blue ? (const float2 *)(b + t.chirp) : nullptr;
  d.bhat = d.blue ? (const float2 *)(b + t.bhat) : nullptr;
  p->tables = dev_tables;
  return MK_OK;
}

int fft4_dct(const Fft4Plan &p, const float *x, int64_t ldx, int64_t nrow, float2 *T, float *out, int64_t ldo,
             int epi, const float *w, int64_t ldw, cudaStream_t st) {
  const Fft4Dev &d = p.d;
  const int64_t npairs = (nrow + 1) / 2;
  MK_CHECK_ARG(npairs >= 1 && npairs <= 65535, "fft4: %lld rows out of range", (long long)nrow);
  MK_CHECK_ARG(ldx >= d.n && ldo >= d.n, "fft4: leading dimensions below the row length");
  MK_CHECK_ARG(epi != FFT4_FILTER || (w && ldw >= d.n), "fft4: filter weights missing");
  int dev = 0;
  MK_CUDA(cudaGetDevice(&dev));
  if (dev >= 0 && dev < 64 && !g_attr[dev]) {
    const int mx = FB * (FFT4_LMAX + 1) * (int)sizeof(float2) + FB * FFT4_LMAX * 2 * (int)sizeof(float);
    MK_CUDA(cudaFuncSetAttribute(k_fft4_a<AM_DCT>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    MK_CUDA(cudaFuncSetAttribute(k_fft4_a<AM_BLUE>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    MK_CUDA(cudaFuncSetAttribute(k_fft4_a<AM_CPLX>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    MK_CUDA(cudaFuncSetAttribute(k_fft4_b<BM_DCT>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    MK_CUDA(cudaFuncSetAttribute(k_fft4_b<BM_MUL>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    MK_CUDA(cudaFuncSetAttribute(k_fft4_b<BM_BLUE>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    g_attr[dev] = true;
  }
  static const WrTable wt = radix_constants();
  const dim3 ga((d.L1 + FB - 1) / FB, (unsigned)npairs), gb((d.L2 + FB - 1) / FB, (unsigned)npairs);
  const size_t smem_a = (size_t)FB * pitch_odd(d.L2) * sizeof(float2);
  const size_t smem_b = (size_t)FB * pitch_odd(d.L1) * sizeof(float2);
  const size_t smem_w = epi == FFT4_FILTER ? (size_t)FB * d.L1 * 2 * sizeof(float) : 0;
  int rc;
  if (!d.blue) {
    k_fft4_a<AM_DCT><<<ga, NT, smem_a, st>>>(x, ldx, nullptr, nrow, T, d, wt);
    if ((rc = launch_status("fft4 pass A"))) return rc;
    k_fft4_b<BM_DCT><<<gb, NT, smem_b + smem_w, st>>>(T, nrow, out, ldo, nullptr, w, ldw, epi, d, wt);
    return launch_status("fft4 pass B");
  }
  float2 *U = T + npairs * d.L;
  k_fft4_a<AM_BLUE><<<ga, NT, smem_a, st>>>(x, ldx, nullptr, nrow, T, d, wt);
  if ((rc = launch_status("fft4 Bluestein pass A"))) return rc;
  k_fft4_b<BM_MUL><<<gb, NT, smem_b, st>>>(T, nrow, nullptr, 0, U, nullptr, 0, FFT4_PLAIN, d, wt);
  if ((rc = launch_status("fft4 Bluestein pass B"))) return rc;
  k_fft4_a<AM_CPLX><<<ga, NT, smem_a, st>>>(nullptr, 0, U, nrow, T, d, wt);
  if ((rc = launch_status("fft4 Bluestein pass A (second)"))) return rc;
  k_fft4_b<BM_BLUE><<<gb, NT, smem_b + smem_w, st>>>(T, nrow, out, ldo, nullptr, w, ldw, epi, d, wt);
  return launch_status("fft4 Bluestein pass B (second)");
}

}  // namespace mk
