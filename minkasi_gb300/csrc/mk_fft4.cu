// FP32 DCT-I by a four-step FFT in shared memory (see mk_fft4.cuh).
#include <cufft.h>

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cmath>
#include <string>
#include <utility>
#include <vector>

#include "mk_async.cuh"
#include "mk_common.cuh"
#include "mk_fft4.cuh"

namespace mk {
namespace {

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

// 16 = 4 x 4 (decimation in time): four 4-point DFTs of the stride-4
// subsequences, the twiddles W_16^{n2 k1}, four 4-point DFTs across them
__device__ __forceinline__ float2 cmulc(float2 a, float c, float s) {  // a (c + i s)
  return make_float2(a.x * c - a.y * s, a.x * s + a.y * c);
}
template <>
struct Dft<16> {
  __device__ static void run(float2 *v, const float2 *) {
    const float c1 = 0.92387953251128674f, s1 = 0.38268343236508977f, h = 0.70710678118654752f;
    float2 y[4][4];
#pragma unroll
    for (int n2 = 0; n2 < 4; n2++) {
#pragma unroll
      for (int n1 = 0; n1 < 4; n1++) y[n2][n1] = v[4 * n1 + n2];
      Dft<4>::run(y[n2], nullptr);
    }
    // W_16^j = cos(pi j / 8) - i sin(pi j / 8)
    y[1][1] = cmulc(y[1][1], c1, -s1);
    y[1][2] = cmulc(y[1][2], h, -h);
    y[1][3] = cmulc(y[1][3], s1, -c1);
    y[2][1] = cmulc(y[2][1], h, -h);
    y[2][2] = mul_mi(y[2][2]);
    y[2][3] = cmulc(y[2][3], -h, -h);
    y[3][1] = cmulc(y[3][1], s1, -c1);
    y[3][2] = cmulc(y[3][2], -h, -h);
    y[3][3] = cmulc(y[3][3], -c1, s1);
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++) {
      float2 t[4] = {y[0][k1], y[1][k1], y[2][k1], y[3][k1]};
      Dft<4>::run(t, nullptr);
#pragma unroll
      for (int k2 = 0; k2 < 4; k2++) v[k1 + 4 * k2] = t[k2];
    }
  }
};

constexpr int inv_mod(int a, int m) {
  for (int x = 1; x < m; x++)
    if ((a * x) % m == 1) return x;
  return 1;
}

// R = R1 R2 with R1, R2 coprime, by the Good-Thomas index maps (no twiddles):
// input n = (n1 R2 + n2 R1) mod R, output k = (k1 R2 e1 + k2 R1 e2) mod R with
// e1 = R2^-1 mod R1, e2 = R1^-1 mod R2, and X_k = sum W_R1^{n1 k1} W_R2^{n2 k2} x_n
template <int R1, int R2>
struct DftPfa {
  __device__ static void run(float2 *v, const float2 *wr) {
    constexpr int R = R1 * R2, e1 = inv_mod(R2 % R1, R1), e2 = inv_mod(R1 % R2, R2);
    float2 a[R2][R1];
#pragma unroll
    for (int n2 = 0; n2 < R2; n2++) {
#pragma unroll
      for (int n1 = 0; n1 < R1; n1++) a[n2][n1] = v[(n1 * R2 + n2 * R1) % R];
      Dft<R1>::run(a[n2], wr);
    }
#pragma unroll
    for (int k1 = 0; k1 < R1; k1++) {
      float2 c[R2];
#pragma unroll
      for (int n2 = 0; n2 < R2; n2++) c[n2] = a[n2][k1];
      Dft<R2>::run(c, wr);
#pragma unroll
      for (int k2 = 0; k2 < R2; k2++) v[(k1 * R2 * e1 + k2 * R1 * e2) % R] = c[k2];
    }
  }
};
template <>
struct Dft<6> : DftPfa<2, 3> {};
template <>
struct Dft<10> : DftPfa<2, 5> {};
template <>
struct Dft<12> : DftPfa<4, 3> {};
template <>
struct Dft<14> : DftPfa<2, 7> {};
template <>
struct Dft<15> : DftPfa<3, 5> {};

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
// A CTA runs FB transforms (FB consecutive j1) with 256 threads.  The
// stages interleave them over the threads (row b = bf % FB), so the first
// stage reads its inputs straight from the detector rows (FB lanes read FB
// consecutive samples), forming the even extension, and the middle stages
// run in shared memory with CTA barriers.  The last stage maps the threads
// row by row instead (32 consecutive butterflies of one row per warp): it
// reads shared memory without conflicts (its span is the whole row), twiddles
// its outputs k2 (natural order) by W_L^{j1 k2} and stores them straight to
// T, one contiguous span per instruction.
// what pass A's first stage reads: the rows' even extension (DCT), the same
// times the Bluestein chirp (zero past 2m), or a complex sequence (U)
enum { AM_DCT = 0, AM_BLUE = 1, AM_CPLX = 2 };

// threads per CTA by transforms per CTA, and the CTAs per SM the register
// budget is sized for (two: shared memory holds two tiles of the longest
// passes each kind is used for)
#ifndef MK_FFT4_NT16
#define MK_FFT4_NT16 512
#endif
#ifndef MK_FFT4_NT8
#define MK_FFT4_NT8 512
#endif
#ifndef MK_FFT4_RMAX
#define MK_FFT4_RMAX 16  // largest radix held in registers
#endif
#ifndef MK_FFT4_MINB8
#define MK_FFT4_MINB8 2
#endif
template <int FB>
struct Cfg {
  static constexpr int NT = FB == 16 ? MK_FFT4_NT16 : MK_FFT4_NT8;
  static constexpr int MINB = FB == 16 ? 2 : MK_FFT4_MINB8;
};

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

template <int R, bool FIRST, int AM, int FB>
__device__ __forceinline__ void astage(float2 *sbuf, int pitch, int Ls, int Ns, float invNs, const float2 *stw,
                                       const float2 *wr, const PassA &pa) {
  const int nq = Ls / R;
  for (int bf = threadIdx.x; bf < FB * nq; bf += Cfg<FB>::NT) {
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

template <bool FIRST, int AM, int FB>
__device__ __forceinline__ void astage_r(int R, float2 *sbuf, int pitch, int Ls, int Ns, float invNs,
                                         const float2 *stw, const float2 *wr, const PassA &pa) {
  switch (R) {
    case 2: astage<2, FIRST, AM, FB>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pa); break;
    case 3: astage<3, FIRST, AM, FB>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pa); break;
    case 4: astage<4, FIRST, AM, FB>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pa); break;
    case 5: astage<5, FIRST, AM, FB>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pa); break;
    case 7: astage<7, FIRST, AM, FB>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pa); break;
    case 8: astage<8, FIRST, AM, FB>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pa); break;
    case 9: astage<9, FIRST, AM, FB>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pa); break;
    case 6: astage<6, FIRST, AM, FB>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pa); break;
    case 10: astage<10, FIRST, AM, FB>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pa); break;
#if MK_FFT4_RMAX >= 12
    case 12: astage<12, FIRST, AM, FB>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pa); break;
#endif
#if MK_FFT4_RMAX >= 14
    case 14: astage<14, FIRST, AM, FB>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pa); break;
#endif
#if MK_FFT4_RMAX >= 15
    case 15: astage<15, FIRST, AM, FB>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pa); break;
#endif
#if MK_FFT4_RMAX >= 16
    case 16: astage<16, FIRST, AM, FB>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pa); break;
#endif
    default: astage<11, FIRST, AM, FB>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pa); break;
  }
}

// the last stage of pass A (Ns R = L2, so every butterfly has g = 0): rows
// mapped warp by warp, outputs k2 = q + r Ns twiddled by W_L^{j1 k2} and
// stored to this pair's T (row j1 = j1_0 + b)
template <int R, int FB>
__device__ __forceinline__ void astage_last(const float2 *sbuf, int pitch, int Ns, const float2 *stw,
                                            const float2 *wr, const PassA &pa, const Fft4Dev &p,
                                            float2 *Tp) {
  for (int bf = threadIdx.x; bf < FB * Ns; bf += Cfg<FB>::NT) {
    const int b = bf / Ns, q = bf - b * Ns;
    if (b >= pa.nb) break;  // b grows with bf
    const float2 *a = sbuf + b * pitch + q;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = a[r * Ns];
#pragma unroll
    for (int r = 1; r < R; r++) v[r] = cmul(v[r], __ldg(stw + (r - 1) * Ns + q));
    Dft<R>::run(v, wr);
    const int j1 = pa.j1_0 + b;
    const float2 *tl = p.tlane + 32 * j1, *tb = p.tblk + j1 * p.nb32;
    float2 *row = Tp + (int64_t)j1 * p.L2;
#pragma unroll
    for (int r = 0; r < R; r++) {
      const int k2 = q + r * Ns;
      row[k2] = cmul(v[r], cmul(__ldg(tb + (k2 >> 5)), __ldg(tl + (k2 & 31))));
    }
  }
}

template <int FB>
__device__ __forceinline__ void astage_last_r(int R, const float2 *sbuf, int pitch, int Ns, const float2 *stw,
                                              const float2 *wr, const PassA &pa, const Fft4Dev &p, float2 *Tp) {
  switch (R) {
    case 2: astage_last<2, FB>(sbuf, pitch, Ns, stw, wr, pa, p, Tp); break;
    case 3: astage_last<3, FB>(sbuf, pitch, Ns, stw, wr, pa, p, Tp); break;
    case 4: astage_last<4, FB>(sbuf, pitch, Ns, stw, wr, pa, p, Tp); break;
    case 5: astage_last<5, FB>(sbuf, pitch, Ns, stw, wr, pa, p, Tp); break;
    case 7: astage_last<7, FB>(sbuf, pitch, Ns, stw, wr, pa, p, Tp); break;
    case 8: astage_last<8, FB>(sbuf, pitch, Ns, stw, wr, pa, p, Tp); break;
    case 9: astage_last<9, FB>(sbuf, pitch, Ns, stw, wr, pa, p, Tp); break;
    case 6: astage_last<6, FB>(sbuf, pitch, Ns, stw, wr, pa, p, Tp); break;
    case 10: astage_last<10, FB>(sbuf, pitch, Ns, stw, wr, pa, p, Tp); break;
#if MK_FFT4_RMAX >= 12
    case 12: astage_last<12, FB>(sbuf, pitch, Ns, stw, wr, pa, p, Tp); break;
#endif
#if MK_FFT4_RMAX >= 14
    case 14: astage_last<14, FB>(sbuf, pitch, Ns, stw, wr, pa, p, Tp); break;
#endif
#if MK_FFT4_RMAX >= 15
    case 15: astage_last<15, FB>(sbuf, pitch, Ns, stw, wr, pa, p, Tp); break;
#endif
#if MK_FFT4_RMAX >= 16
    case 16: astage_last<16, FB>(sbuf, pitch, Ns, stw, wr, pa, p, Tp); break;
#endif
    default: astage_last<11, FB>(sbuf, pitch, Ns, stw, wr, pa, p, Tp); break;
  }
}

// row pitch (float2) of a tile of FB interleaved transforms: odd, so the
// rows fall in distinct shared-memory banks
__host__ __device__ __forceinline__ int pitch_odd(int Ls) { return Ls | 1; }

// pass A: rows (2 pair, 2 pair + 1) of x (or the pair's U) -> T[pair]
// (L1 x L2, twiddled)
template <int AM, int FB>
__global__ void __launch_bounds__(Cfg<FB>::NT, Cfg<FB>::MINB) k_fft4_a(const float *__restrict__ x, int64_t ldx,
                                                    const float2 *__restrict__ U, int64_t nrow,
                                                    float2 *__restrict__ T, const Fft4Dev p, const WrTable wt) {
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
  float2 *Tp = T + pair * p.L;
  const int S = p.nr2;
  if (S >= 2) {
    astage_r<true, AM, FB>(p.r2[0], sbuf, pitch, L2, 1, 1.0f, p.stw2, wt.w, pa);
    for (int s = 1; s < S - 1; s++) {
      __syncthreads();
      astage_r<false, AM, FB>(p.r2[s], sbuf, pitch, L2, p.ns2[s], p.inv2[s], p.stw2 + p.to2[s], wt.w, pa);
    }
    __syncthreads();
    astage_last_r<FB>(p.r2[S - 1], sbuf, pitch, p.ns2[S - 1], p.stw2 + p.to2[S - 1], wt.w, pa, p, Tp);
    return;
  }
  // one stage at most (L2 <= 16): into shared memory, then each warp
  // twiddles rows b by W_L^{j1 k2} and stores them
  if (S == 0) {  // L2 == 1: the column is its own transform
    if (tid < pa.nb) sbuf[tid * pitch] = a_input<AM>(pa, pa.j1_0 + tid);
  } else {
    astage_r<true, AM, FB>(p.r2[0], sbuf, pitch, L2, 1, 1.0f, p.stw2, wt.w, pa);
  }
  __syncthreads();
  const int lane = tid & 31;
  for (int b = tid >> 5; b < pa.nb; b += Cfg<FB>::NT / 32) {
    const float2 *row = sbuf + b * pitch;
    const int j1 = pa.j1_0 + b;
    const float2 tl = __ldg(p.tlane + 32 * j1 + lane);
    const float2 *tb = p.tblk + j1 * p.nb32;
    for (int i = 0; i < p.nb32; i++) {
      const int k2 = 32 * i + lane;
      if (k2 < L2) Tp[(int64_t)j1 * L2 + k2] = cmul(row[k2], cmul(__ldg(tb + i), tl));
    }
  }
}

// ---- pass B ------------------------------------------------------------
// The CTA's FB transforms (FB consecutive k2) are interleaved over its
// 256 threads: butterfly bf of a stage belongs to row b = bf % FB, so the
// FB lanes of a row group read or write FB consecutive columns of T / of the
// output.  The first stage reads its inputs straight from T (natural order:
// position g R0 + r of the digit-reversed layout holds index
// iperm[g R0] + (L1 / R0) r), and the last stage writes its outputs straight
// to the DCT rows with the epilogue.
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
  const float *sw;        // prefetched weights, [k1][b][row], or null
  const float *w1, *w2;   // else the weight rows, read in the last stage
  const int *iperm;
};

template <int R, bool FIRST, bool LAST, int BM, int FB>
__device__ __forceinline__ void bstage(float2 *sbuf, int pitch, int Ls, int Ns, float invNs, const float2 *stw,
                                       const float2 *wr, const PassB &pb) {
  const int nq = Ls / R;
  for (int bf = threadIdx.x; bf < FB * nq; bf += Cfg<FB>::NT) {
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
          if (pb.sw) {
            a *= pb.sw[2 * (k1 * FB + b)];
            c *= pb.sw[2 * (k1 * FB + b) + 1];
          } else {
            a *= __ldg(pb.w1 + kk);
            if (pb.has2) c *= __ldg(pb.w2 + kk);
          }
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

template <bool FIRST, bool LAST, int BM, int FB>
__device__ __forceinline__ void bstage_r(int R, float2 *sbuf, int pitch, int Ls, int Ns, float invNs,
                                         const float2 *stw, const float2 *wr, const PassB &pb) {
  switch (R) {
    case 2: bstage<2, FIRST, LAST, BM, FB>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pb); break;
    case 3: bstage<3, FIRST, LAST, BM, FB>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pb); break;
    case 4: bstage<4, FIRST, LAST, BM, FB>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pb); break;
    case 5: bstage<5, FIRST, LAST, BM, FB>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pb); break;
    case 7: bstage<7, FIRST, LAST, BM, FB>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pb); break;
    case 8: bstage<8, FIRST, LAST, BM, FB>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pb); break;
    case 9: bstage<9, FIRST, LAST, BM, FB>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pb); break;
    case 6: bstage<6, FIRST, LAST, BM, FB>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pb); break;
    case 10: bstage<10, FIRST, LAST, BM, FB>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pb); break;
#if MK_FFT4_RMAX >= 12
    case 12: bstage<12, FIRST, LAST, BM, FB>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pb); break;
#endif
#if MK_FFT4_RMAX >= 14
    case 14: bstage<14, FIRST, LAST, BM, FB>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pb); break;
#endif
#if MK_FFT4_RMAX >= 15
    case 15: bstage<15, FIRST, LAST, BM, FB>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pb); break;
#endif
#if MK_FFT4_RMAX >= 16
    case 16: bstage<16, FIRST, LAST, BM, FB>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pb); break;
#endif
    default: bstage<11, FIRST, LAST, BM, FB>(sbuf, pitch, Ls, Ns, invNs, stw, wr, pb); break;
  }
}

// pass B: T[pair] -> DCT rows 2 pair, 2 pair + 1 of out (k <= m) with the
// epilogue, or (BM_MUL) -> the pair's U
template <int BM, int FB>
__global__ void __launch_bounds__(Cfg<FB>::NT, Cfg<FB>::MINB) k_fft4_b(const float2 *__restrict__ T, int64_t nrow,
                                                    float *__restrict__ out, int64_t ldo, float2 *__restrict__ U,
                                                    const float *__restrict__ w, int64_t ldw, int epi,
                                                    int wpre, const Fft4Dev p, const WrTable wt) {
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
  pb.sw = nullptr;
  pb.w1 = pb.w2 = nullptr;
  if (BM != BM_MUL && epi == FFT4_FILTER) {
    const float *w1 = w + r0 * ldw;
    const float *w2 = pb.has2 ? w1 + ldw : w1;
    pb.w1 = w1;
    pb.w2 = w2;
    if (wpre) {
      // the weights of this tile's outputs, [k1][b][row], prefetched during
      // the first stages (when two CTAs still fit an SM with them)
      float *sw = reinterpret_cast<float *>(sbuf + FB * pitch);
      pb.sw = sw;
#pragma unroll 4
      for (int idx = tid; idx < FB * L1; idx += Cfg<FB>::NT) {
        const int b = idx % FB, k1 = idx / FB;
        const int k = pb.k2_0 + b + L2 * k1;
        const bool ok = b < pb.nb && k <= pb.m;
        cp4(sw + 2 * idx, ok ? w1 + k : w1, ok);
        cp4(sw + 2 * idx + 1, ok ? w2 + k : w1, ok && pb.has2);
      }
    }
  }
  const int S = p.nr1;
  if (S == 1) {
    cp_async_wait_all();
    __syncthreads();
    bstage_r<true, true, BM, FB>(p.r1[0], sbuf, pitch, L1, 1, 1.0f, p.stw1, wt.w, pb);
    return;
  }
  bstage_r<true, false, BM, FB>(p.r1[0], sbuf, pitch, L1, 1, 1.0f, p.stw1, wt.w, pb);
  __syncthreads();
  for (int s = 1; s < S - 1; s++) {
    bstage_r<false, false, BM, FB>(p.r1[s], sbuf, pitch, L1, p.ns1[s], p.inv1[s], p.stw1 + p.to1[s], wt.w, pb);
    __syncthreads();
  }
  cp_async_wait_all();
  __syncthreads();
  bstage_r<false, true, BM, FB>(p.r1[S - 1], sbuf, pitch, L1, p.ns1[S - 1], p.inv1[S - 1],
                                p.stw1 + p.to1[S - 1], wt.w, pb);
}

// ---- Bluestein's middle pass ----------------------------------------------
// Between pass A (a -> T) and the last pass, Bluestein needs
// U = conj(DFT_M(a) B^) and then DFT_M(U).  With M = L1 L2, U is indexed
// i = i2 + L2 i1 (i2 = k2 of the first transform, i1 = k1), and
//   DFT(U)[o1 + L1 o2] = sum_i2 W_L2^{i2 o2} W_M^{i2 o1} sum_i1 W_L1^{i1 o1} U[i2 + L2 i1],
// so for each column k2 the last step of the first transform (length L1
// over j1 -> k1), the product with B^ and the first step of the second
// transform (length L1 over i1 -> o1) run in one CTA without leaving shared
// memory.  The first transform runs by decimation in frequency (natural
// input read from T, digit-reversed output, twiddles after each butterfly),
// which leaves exactly the digit-reversed input order the second transform's
// decimation-in-time stages take, so no permutation is needed: its stage 0
// and the second transform's stage 0 share one butterfly pass with the
// product in between.  The last stage stores V[k2][o1] = W_M^{k2 o1} (.)
// row by row (o1 contiguous), and pass B over the transposed shape (length
// L2 over i2 -> o2, rows o1) finishes with the chirp and the epilogue.
struct PassC {
  const float2 *Tp;  // this pair's T (L1 x L2)
  float2 *Vp;        // this pair's V (L2 x L1)
  const float2 *bhat;
  int L1, L2, k2_0, nb;
};

// the first decimation-in-frequency stage (span Ns = L1 / R): natural-order
// inputs k + r Ns from T's column, butterfly, twiddle after it
template <int R, int FB>
__device__ __forceinline__ void cstage_first(float2 *sbuf, int pitch, int Ns, const float2 *stw, const float2 *wr,
                                             const PassC &pc) {
  for (int bf = threadIdx.x; bf < FB * Ns; bf += Cfg<FB>::NT) {
    const int b = bf % FB, q = bf / FB;
    if (b >= pc.nb) continue;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = pc.Tp[(int64_t)(q + r * Ns) * pc.L2 + pc.k2_0 + b];
    Dft<R>::run(v, wr);
#pragma unroll
    for (int r = 1; r < R; r++) v[r] = cmul(v[r], __ldg(stw + (r - 1) * Ns + q));
    float2 *a = sbuf + b * pitch + q;
#pragma unroll
    for (int r = 0; r < R; r++) a[r * Ns] = v[r];
  }
}

// a decimation-in-frequency stage in shared memory (twiddles after the
// butterfly), same butterfly indexing as the decimation-in-time stages
template <int R, int FB>
__device__ __forceinline__ void cstage_dif(float2 *sbuf, int pitch, int Ls, int Ns, float invNs, const float2 *stw,
                                           const float2 *wr, int nb) {
  const int nq = Ls / R;
  for (int bf = threadIdx.x; bf < FB * nq; bf += Cfg<FB>::NT) {
    const int b = bf % FB, q = bf / FB;
    if (b >= nb) continue;
    const int g = __float2int_rz(((float)q + 0.5f) * invNs);
    const int k = q - g * Ns;
    float2 *a = sbuf + b * pitch + g * Ns * R + k;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = a[r * Ns];
    Dft<R>::run(v, wr);
#pragma unroll
    for (int r = 1; r < R; r++) v[r] = cmul(v[r], __ldg(stw + (r - 1) * Ns + k));
#pragma unroll
    for (int r = 0; r < R; r++) a[r * Ns] = v[r];
  }
}

// stage 0 of both transforms: the last DIF butterflies give F at k1 =
// iperm[q R] + (L1 / R) r; U = conj(F B^) there; then the first DIT
// butterflies of the second transform on the same R values
template <int R, int FB>
__device__ __forceinline__ void cstage_mid(float2 *sbuf, int pitch, int L1, const int *iperm, const float2 *wr,
                                           const PassC &pc) {
  const int nq = L1 / R;
  for (int bf = threadIdx.x; bf < FB * nq; bf += Cfg<FB>::NT) {
    const int b = bf % FB, q = bf / FB;
    if (b >= pc.nb) continue;
    float2 *a = sbuf + b * pitch + q * R;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = a[r];
    Dft<R>::run(v, wr);
    const int k1 = __ldg(iperm + q * R);
#pragma unroll
    for (int r = 0; r < R; r++) {
      const float2 f = cmul(v[r], __ldg(pc.bhat + pc.k2_0 + b + (int64_t)pc.L2 * (k1 + (L1 / R) * r)));
      v[r] = make_float2(f.x, -f.y);
    }
    Dft<R>::run(v, wr);
#pragma unroll
    for (int r = 0; r < R; r++) a[r] = v[r];
  }
}

// a decimation-in-time stage in shared memory (twiddles before the butterfly)
template <int R, int FB>
__device__ __forceinline__ void cstage_dit(float2 *sbuf, int pitch, int Ls, int Ns, float invNs, const float2 *stw,
                                           const float2 *wr, int nb) {
  const int nq = Ls / R;
  for (int bf = threadIdx.x; bf < FB * nq; bf += Cfg<FB>::NT) {
    const int b = bf % FB, q = bf / FB;
    if (b >= nb) continue;
    const int g = __float2int_rz(((float)q + 0.5f) * invNs);
    const int k = q - g * Ns;
    float2 *a = sbuf + b * pitch + g * Ns * R + k;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = a[r * Ns];
#pragma unroll
    for (int r = 1; r < R; r++) v[r] = cmul(v[r], __ldg(stw + (r - 1) * Ns + k));
    Dft<R>::run(v, wr);
#pragma unroll
    for (int r = 0; r < R; r++) a[r * Ns] = v[r];
  }
}

// the last DIT stage (Ns R = L1): rows warp by warp, outputs o1 = q + r Ns
// twiddled by W_M^{k2 o1} and stored to V row k2
template <int R, int FB>
__device__ __forceinline__ void cstage_last(const float2 *sbuf, int pitch, int Ns, const float2 *stw,
                                            const float2 *wr, const PassC &pc, const Fft4Dev &p) {
  for (int bf = threadIdx.x; bf < FB * Ns; bf += Cfg<FB>::NT) {
    const int b = bf / Ns, q = bf - b * Ns;
    if (b >= pc.nb) break;
    const float2 *a = sbuf + b * pitch + q;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = a[r * Ns];
#pragma unroll
    for (int r = 1; r < R; r++) v[r] = cmul(v[r], __ldg(stw + (r - 1) * Ns + q));
    Dft<R>::run(v, wr);
    const int k2 = pc.k2_0 + b;
    const float2 *tl = p.tlane2 + 32 * k2, *tb = p.tblk2 + k2 * p.nb32b;
    float2 *row = pc.Vp + (int64_t)k2 * pc.L1;
#pragma unroll
    for (int r = 0; r < R; r++) {
      const int o1 = q + r * Ns;
      row[o1] = cmul(v[r], cmul(__ldg(tb + (o1 >> 5)), __ldg(tl + (o1 & 31))));
    }
  }
}

#if MK_FFT4_RMAX >= 12
#define MK_RCASE12(CALL) case 12: { constexpr int RR = 12; CALL; } break;
#else
#define MK_RCASE12(CALL)
#endif
#if MK_FFT4_RMAX >= 14
#define MK_RCASE14(CALL) case 14: { constexpr int RR = 14; CALL; } break;
#else
#define MK_RCASE14(CALL)
#endif
#if MK_FFT4_RMAX >= 15
#define MK_RCASE15(CALL) case 15: { constexpr int RR = 15; CALL; } break;
#else
#define MK_RCASE15(CALL)
#endif
#if MK_FFT4_RMAX >= 16
#define MK_RCASE16(CALL) case 16: { constexpr int RR = 16; CALL; } break;
#else
#define MK_RCASE16(CALL)
#endif
#define MK_RADIX_SWITCH(R, CALL)                     \
  switch (R) {                                       \
    case 2: { constexpr int RR = 2; CALL; } break;   \
    case 3: { constexpr int RR = 3; CALL; } break;   \
    case 4: { constexpr int RR = 4; CALL; } break;   \
    case 5: { constexpr int RR = 5; CALL; } break;   \
    case 6: { constexpr int RR = 6; CALL; } break;   \
    case 7: { constexpr int RR = 7; CALL; } break;   \
    case 8: { constexpr int RR = 8; CALL; } break;   \
    case 9: { constexpr int RR = 9; CALL; } break;   \
    case 10: { constexpr int RR = 10; CALL; } break; \
    MK_RCASE12(CALL)                                 \
    MK_RCASE14(CALL)                                 \
    MK_RCASE15(CALL)                                 \
    MK_RCASE16(CALL)                                 \
    default: { constexpr int RR = 11; CALL; } break; \
  }

// T[pair] (L1 x L2, from pass A on the chirped rows) -> V[pair] (L2 x L1);
// needs nr1 >= 2
template <int FB>
__global__ void __launch_bounds__(Cfg<FB>::NT, Cfg<FB>::MINB) k_fft4_conv(const float2 *__restrict__ T, float2 *__restrict__ V,
                                                     const Fft4Dev p, const WrTable wt) {
  extern __shared__ float2 sbuf[];
  const int L1 = p.L1, pitch = pitch_odd(L1), S = p.nr1;
  const int64_t pair = blockIdx.y;
  PassC pc;
  pc.Tp = T + pair * p.L;
  pc.Vp = V + pair * p.L;
  pc.bhat = p.bhat;
  pc.L1 = L1;
  pc.L2 = p.L2;
  pc.k2_0 = blockIdx.x * FB;
  pc.nb = min(FB, p.L2 - pc.k2_0);
  MK_RADIX_SWITCH(p.r1[S - 1], (cstage_first<RR, FB>(sbuf, pitch, p.ns1[S - 1], p.stw1 + p.to1[S - 1], wt.w, pc)));
  __syncthreads();
  for (int s = S - 2; s >= 1; s--) {
    MK_RADIX_SWITCH(p.r1[s], (cstage_dif<RR, FB>(sbuf, pitch, L1, p.ns1[s], p.inv1[s], p.stw1 + p.to1[s], wt.w,
                                                 pc.nb)));
    __syncthreads();
  }
  MK_RADIX_SWITCH(p.r1[0], (cstage_mid<RR, FB>(sbuf, pitch, L1, p.iperm1, wt.w, pc)));
  __syncthreads();
  for (int s = 1; s < S - 1; s++) {
    MK_RADIX_SWITCH(p.r1[s], (cstage_dit<RR, FB>(sbuf, pitch, L1, p.ns1[s], p.inv1[s], p.stw1 + p.to1[s], wt.w,
                                                 pc.nb)));
    __syncthreads();
  }
  MK_RADIX_SWITCH(p.r1[S - 1], (cstage_last<RR, FB>(sbuf, pitch, p.ns1[S - 1], p.stw1 + p.to1[S - 1], wt.w, pc, p)));
}
#undef MK_RADIX_SWITCH
#undef MK_RCASE12
#undef MK_RCASE14
#undef MK_RCASE15
#undef MK_RCASE16

void factor(int64_t L, std::vector<int> &f) {
  for (int pr : {2, 3, 5, 7, 11})
    while (L % pr == 0) {
      f.push_back(pr);
      L /= pr;
    }
  if (L != 1) f.clear();
}

// radices of a transform of length Ls (a product of 2, 3, 5, 7, 11): the
// fewest stages over the radices 2 .. 16 held in registers (ties broken by
// an estimate of the arithmetic), odd ones first (the stride-1 first stage
// is then free of bank conflicts), each group in decreasing order.
// MINKASI_GB300_FFT4_RADIX=basic keeps the prime radices with 3 x 3 as 9
// and powers of 2 as 8, 4, 2.
static const int kRadix[] = {16, 15, 14, 12, 11, 10, 9, 8, 7, 6, 5, 4, 3, 2};
static const int kRadixCost[] = {4, 5, 5, 4, 6, 4, 4, 3, 4, 3, 3, 2, 2, 1};

static void radix_exps(int R, int *e) {
  const int pr[5] = {2, 3, 5, 7, 11};
  for (int i = 0; i < 5; i++) {
    e[i] = 0;
    while (R % pr[i] == 0) {
      R /= pr[i];
      e[i]++;
    }
  }
}

// best (stages, cost) radix list for the exponent vector e, memoised
struct RadixPlan {
  int stages = 1 << 20, cost = 0;
  std::vector<int> r;
};
static const RadixPlan &best_plan(const int *e, std::vector<RadixPlan> &memo, std::vector<bool> &done) {
  const int key = (((e[0] * 8 + e[1]) * 6 + e[2]) * 5 + e[3]) * 5 + e[4];
  if (done[key]) return memo[key];
  RadixPlan best;
  if (!e[0] && !e[1] && !e[2] && !e[3] && !e[4]) {
    best.stages = 0;
  } else {
    for (size_t i = 0; i < sizeof(kRadix) / sizeof(int); i++) {
      if (kRadix[i] > MK_FFT4_RMAX) continue;
      int f[5];
      radix_exps(kRadix[i], f);
      bool fits = true;
      for (int k = 0; k < 5; k++) fits &= f[k] <= e[k];
      if (!fits) continue;
      int rest[5];
      for (int k = 0; k < 5; k++) rest[k] = e[k] - f[k];
      const RadixPlan &sub = best_plan(rest, memo, done);
      const int st = sub.stages + 1, co = sub.cost + kRadixCost[i];
      if (st < best.stages || (st == best.stages && co < best.cost)) {
        best.stages = st;
        best.cost = co;
        best.r = sub.r;
        best.r.push_back(kRadix[i]);
      }
    }
  }
  memo[key] = best;
  done[key] = true;
  return memo[key];
}

bool radices(int Ls, int *r, int *nr) {
  std::vector<int> f;
  factor(Ls, f);
  if (f.empty() && Ls != 1) return false;
  int c[12] = {0};
  for (int x : f) c[x]++;
  std::vector<int> out;
  const char *mode = getenv("MINKASI_GB300_FFT4_RADIX");
  if (mode && std::string(mode) == "basic") {
    for (int i = 0; i < c[11]; i++) out.push_back(11);
    for (; c[3] >= 2; c[3] -= 2) out.push_back(9);
    for (int i = 0; i < c[7]; i++) out.push_back(7);
    for (int i = 0; i < c[5]; i++) out.push_back(5);
    if (c[3]) out.push_back(3);
    for (; c[2] >= 3; c[2] -= 3) out.push_back(8);
    if (c[2] == 2) out.push_back(4);
    if (c[2] == 1) out.push_back(2);
  } else {
    int e[5] = {c[2], c[3], c[5], c[7], c[11]};
    if (e[0] > 10 || e[1] > 7 || e[2] > 5 || e[3] > 4 || e[4] > 4) return false;
    std::vector<RadixPlan> memo(11 * 8 * 6 * 5 * 5);
    std::vector<bool> done(memo.size(), false);
    out = best_plan(e, memo, done).r;
    std::stable_sort(out.begin(), out.end(), [](int a, int b) {
      if ((a & 1) != (b & 1)) return (a & 1) > (b & 1);
      return a > b;
    });
  }
  if ((int)out.size() > FFT4_MAXR) return false;
  for (size_t i = 0; i < out.size(); i++) r[i] = out[i];
  *nr = (int)out.size();
  return true;
}

size_t al(size_t x) { return (x + 255) / 256 * 256; }

struct TableLayout {
  size_t stw1, stw2, iperm1, iperm2, tlane, tblk, chirp, bhat, tlane2, tblk2, total;
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
  t.tlane2 = o;
  o += d.blue ? al((size_t)d.L2 * 32 * sizeof(float2)) : 0;
  t.tblk2 = o;
  o += d.blue ? al((size_t)d.L2 * ((d.L1 + 31) / 32) * sizeof(float2)) : 0;
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

// transforms per CTA for a pass of length Ls: 16 (wider coalesced rows)
// while two such CTAs fit in an SM's shared memory, else 8.
// MINKASI_GB300_FFT4_FB=8 or 16 forces one of them.
static int fb_for(int Ls) {
  const char *e = getenv("MINKASI_GB300_FFT4_FB");
  if (e && (e[0] == '8' && e[1] == 0)) return 8;
  if (e && (e[0] == '1' && e[1] == '6' && e[2] == 0)) return 16;
  return 16 * (size_t)(Ls | 1) * sizeof(float2) <= 113 * 1024 ? 16 : 8;
}

bool fft4_shape(int64_t n, Fft4Dev *d, bool bluestein) {
  if (n < 2 || n > (int64_t)FFT4_LMAX * FFT4_LMAX / 2) return false;
  Fft4Dev t{};
  t.n = n;
  t.m = n - 1;
  t.Lx = 2 * t.m;
  bool ok = false;
  if (split_len(t.Lx, &t)) {
    t.blue = false;
    ok = true;
  } else if (bluestein) {
    for (int64_t M = 3 * t.m; M <= (int64_t)FFT4_LMAX * FFT4_LMAX && !ok; M++) {
      if (split_len(M, &t)) {
        t.blue = true;
        ok = true;
      }
    }
  }
  if (!ok) return false;
  t.fba = fb_for(t.L2);
  t.fbb = fb_for(t.L1);
  *d = t;
  return true;
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
    d.nb32b = (d.L1 + 31) / 32;
    float2 *tl2 = (float2 *)(h.data() + t.tlane2), *tb2 = (float2 *)(h.data() + t.tblk2);
    for (int64_t k2 = 0; k2 < d.L2; k2++) {
      for (int l = 0; l < 32; l++) tl2[32 * k2 + l] = unit((double)(k2 * l % d.L), (double)d.L);
      for (int i = 0; i < d.nb32b; i++) tb2[k2 * d.nb32b + i] = unit((double)(k2 * 32 * i % d.L), (double)d.L);
    }
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
  d.tlane2 = d.blue ? (const float2 *)(b + t.tlane2) : nullptr;
  d.tblk2 = d.blue ? (const float2 *)(b + t.tblk2) : nullptr;
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
    const int mx = 16 * (FFT4_LMAX + 1) * (int)sizeof(float2);
    const int mx8 = 8 * (FFT4_LMAX + 1) * (int)sizeof(float2) + 8 * FFT4_LMAX * 2 * (int)sizeof(float);
#define MK_FFT4_ATTR(k, v) MK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, v))
    MK_FFT4_ATTR((k_fft4_a<AM_DCT, 8>), mx8);
    MK_FFT4_ATTR((k_fft4_a<AM_BLUE, 8>), mx8);
    MK_FFT4_ATTR((k_fft4_a<AM_CPLX, 8>), mx8);
    MK_FFT4_ATTR((k_fft4_b<BM_DCT, 8>), mx8);
    MK_FFT4_ATTR((k_fft4_b<BM_MUL, 8>), mx8);
    MK_FFT4_ATTR((k_fft4_b<BM_BLUE, 8>), mx8);
    MK_FFT4_ATTR((k_fft4_a<AM_DCT, 16>), mx);
    MK_FFT4_ATTR((k_fft4_a<AM_BLUE, 16>), mx);
    MK_FFT4_ATTR((k_fft4_a<AM_CPLX, 16>), mx);
    MK_FFT4_ATTR((k_fft4_b<BM_DCT, 16>), mx);
    MK_FFT4_ATTR((k_fft4_b<BM_MUL, 16>), mx);
    MK_FFT4_ATTR((k_fft4_b<BM_BLUE, 16>), mx);
    MK_FFT4_ATTR((k_fft4_conv<8>), mx8);
    MK_FFT4_ATTR((k_fft4_conv<16>), mx);
#undef MK_FFT4_ATTR
    g_attr[dev] = true;
  }
  static const WrTable wt = radix_constants();
  const int fa = d.fba == 16 ? 16 : 8, fb = d.fbb == 16 ? 16 : 8;
  const dim3 ga((d.L1 + fa - 1) / fa, (unsigned)npairs), gb((d.L2 + fb - 1) / fb, (unsigned)npairs);
  const size_t smem_a = (size_t)fa * pitch_odd(d.L2) * sizeof(float2);
  const size_t smem_b = (size_t)fb * pitch_odd(d.L1) * sizeof(float2);
  // FILTER weights go through shared memory on 8-transform passes while two
  // CTAs still fit an SM; otherwise the last stage reads them directly
  const size_t smem_w8 = (size_t)8 * d.L1 * 2 * sizeof(float);
  const int wpre = epi == FFT4_FILTER && fb == 8 && smem_b + smem_w8 <= 113 * 1024;
  const size_t smem_w = wpre ? smem_w8 : 0;
  auto pass_a = [&](int am, const float *xx, int64_t ldxx, const float2 *uu) {
    if (fa == 16) {
      if (am == AM_DCT) k_fft4_a<AM_DCT, 16><<<ga, Cfg<16>::NT, smem_a, st>>>(xx, ldxx, uu, nrow, T, d, wt);
      else if (am == AM_BLUE) k_fft4_a<AM_BLUE, 16><<<ga, Cfg<16>::NT, smem_a, st>>>(xx, ldxx, uu, nrow, T, d, wt);
      else k_fft4_a<AM_CPLX, 16><<<ga, Cfg<16>::NT, smem_a, st>>>(xx, ldxx, uu, nrow, T, d, wt);
    } else {
      if (am == AM_DCT) k_fft4_a<AM_DCT, 8><<<ga, Cfg<8>::NT, smem_a, st>>>(xx, ldxx, uu, nrow, T, d, wt);
      else if (am == AM_BLUE) k_fft4_a<AM_BLUE, 8><<<ga, Cfg<8>::NT, smem_a, st>>>(xx, ldxx, uu, nrow, T, d, wt);
      else k_fft4_a<AM_CPLX, 8><<<ga, Cfg<8>::NT, smem_a, st>>>(xx, ldxx, uu, nrow, T, d, wt);
    }
  };
  auto pass_b = [&](int bm, float2 *uu, int e, size_t sm, int wp) {
    if (fb == 16) {
      if (bm == BM_DCT) k_fft4_b<BM_DCT, 16><<<gb, Cfg<16>::NT, sm, st>>>(T, nrow, out, ldo, uu, w, ldw, e, wp, d, wt);
      else if (bm == BM_MUL) k_fft4_b<BM_MUL, 16><<<gb, Cfg<16>::NT, sm, st>>>(T, nrow, out, ldo, uu, w, ldw, e, wp, d, wt);
      else k_fft4_b<BM_BLUE, 16><<<gb, Cfg<16>::NT, sm, st>>>(T, nrow, out, ldo, uu, w, ldw, e, wp, d, wt);
    } else {
      if (bm == BM_DCT) k_fft4_b<BM_DCT, 8><<<gb, Cfg<8>::NT, sm, st>>>(T, nrow, out, ldo, uu, w, ldw, e, wp, d, wt);
      else if (bm == BM_MUL) k_fft4_b<BM_MUL, 8><<<gb, Cfg<8>::NT, sm, st>>>(T, nrow, out, ldo, uu, w, ldw, e, wp, d, wt);
      else k_fft4_b<BM_BLUE, 8><<<gb, Cfg<8>::NT, sm, st>>>(T, nrow, out, ldo, uu, w, ldw, e, wp, d, wt);
    }
  };
  int rc;
  if (!d.blue) {
    pass_a(AM_DCT, x, ldx, nullptr);
    if ((rc = launch_status("fft4 pass A"))) return rc;
    pass_b(BM_DCT, nullptr, epi, smem_b + smem_w, wpre);
    return launch_status("fft4 pass B");
  }
  float2 *U = T + npairs * d.L;
  pass_a(AM_BLUE, x, ldx, nullptr);
  if ((rc = launch_status("fft4 Bluestein pass A"))) return rc;
  // MINKASI_GB300_FFT4_BLUE3=0 keeps the four-pass form (U written out)
  const char *e4 = getenv("MINKASI_GB300_FFT4_BLUE3");
  const bool four_pass = e4 && e4[0] == '0' && e4[1] == 0;
  if (d.nr1 >= 2 && !four_pass) {
    // the middle pass T -> V (= U's space), then pass B on the transposed
    // shape: length L2 over the rows of V, outputs o1 + L1 o2
    const size_t smem_c = (size_t)fb * pitch_odd(d.L1) * sizeof(float2);
    if (fb == 16) k_fft4_conv<16><<<gb, Cfg<16>::NT, smem_c, st>>>(T, U, d, wt);
    else k_fft4_conv<8><<<gb, Cfg<8>::NT, smem_c, st>>>(T, U, d, wt);
    if ((rc = launch_status("fft4 Bluestein middle pass"))) return rc;
    Fft4Dev tr = d;
    std::swap(tr.L1, tr.L2);
    std::swap(tr.nr1, tr.nr2);
    std::swap(tr.r1, tr.r2);
    std::swap(tr.ns1, tr.ns2);
    std::swap(tr.to1, tr.to2);
    std::swap(tr.inv1, tr.inv2);
    std::swap(tr.stw1, tr.stw2);
    std::swap(tr.iperm1, tr.iperm2);
    const dim3 gt((tr.L2 + fa - 1) / fa, (unsigned)npairs);
    const size_t smem_t = (size_t)fa * pitch_odd(tr.L1) * sizeof(float2);
    const size_t smem_tw8 = (size_t)8 * tr.L1 * 2 * sizeof(float);
    const int wpre_t = epi == FFT4_FILTER && fa == 8 && smem_t + smem_tw8 <= 113 * 1024;
    const size_t smem_tw = wpre_t ? smem_tw8 : 0;
    if (fa == 16)
      k_fft4_b<BM_BLUE, 16><<<gt, Cfg<16>::NT, smem_t, st>>>(U, nrow, out, ldo, nullptr, w, ldw, epi, 0, tr, wt);
    else
      k_fft4_b<BM_BLUE, 8><<<gt, Cfg<8>::NT, smem_t + smem_tw, st>>>(U, nrow, out, ldo, nullptr, w, ldw, epi, wpre_t,
                                                                    tr, wt);
    return launch_status("fft4 Bluestein last pass");
  }
  pass_b(BM_MUL, U, FFT4_PLAIN, smem_b, 0);
  if ((rc = launch_status("fft4 Bluestein pass B"))) return rc;
  pass_a(AM_CPLX, nullptr, 0, U);
  if ((rc = launch_status("fft4 Bluestein pass A (second)"))) return rc;
  pass_b(BM_BLUE, nullptr, epi, smem_b + smem_w, wpre);
  return launch_status("fft4 Bluestein pass B (second)");
}

}  // namespace mk
