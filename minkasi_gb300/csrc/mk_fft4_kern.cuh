// Device side of the four-step FFT DCT-I (see mk_fft4.cuh), written once
// for both precisions: the including file defines
//   MK_FFT4_NS   the namespace (one per precision)
//   MK_FFT4_C    the complex type (float2 or double2)
//   MK_FFT4_RT   the real type (float or double)
//   MK_FFT4_FBHI / MK_FFT4_FBLO        transforms per CTA, wide and narrow tile
//   MK_FFT4_NTHI / MK_FFT4_NTLO        threads per CTA for each
//   MK_FFT4_MINBLO                     CTAs per SM the narrow tile's registers are sized for
//   (MK_FFT4_MINBHI, default 2: the same for the wide tile)
// and includes this file once.  dct_launch is the host entry of the
// precision.
#include <cufft.h>

#include <cmath>
#include <cstdlib>
#include <utility>

#include "mk_async.cuh"
#include "mk_common.cuh"
#include "mk_fft4.cuh"

namespace mk {
namespace MK_FFT4_NS {

using C = MK_FFT4_C;
using RT = MK_FFT4_RT;
constexpr int FB_HI = MK_FFT4_FBHI, FB_LO = MK_FFT4_FBLO;
#ifndef MK_FFT4_MINBHI
#define MK_FFT4_MINBHI 2
#endif
constexpr int NT_HI = MK_FFT4_NTHI, NT_LO = MK_FFT4_NTLO, MINB_LO = MK_FFT4_MINBLO, MINB_HI = MK_FFT4_MINBHI;
constexpr int WR3 = 0, WR5 = 3, WR7 = 8, WR9 = 15, WR11 = 24, WRN = 35;  // offsets into the radix constants

__host__ __device__ __forceinline__ C mkc(RT x, RT y) {
  C c;
  c.x = x;
  c.y = y;
  return c;
}



__device__ __forceinline__ C cmul(C a, C b) {
  return mkc(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ C cadd(C a, C b) { return mkc(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ C csub(C a, C b) { return mkc(a.x - b.x, a.y - b.y); }
// -i z
__device__ __forceinline__ C mul_mi(C z) { return mkc(z.y, -z.x); }

// forward DFT of R points in registers: v_q <- sum_r v_r W_R^{rq}
template <int R>
struct Dft;

template <>
struct Dft<2> {
  __device__ static void run(C *v, const C *) {
    const C a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};

template <>
struct Dft<4> {
  __device__ static void run(C *v, const C *) {
    const C s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
    const C s13 = cadd(v[1], v[3]), d13 = csub(v[1], v[3]);
    v[0] = cadd(s02, s13);
    v[2] = csub(s02, s13);
    v[1] = cadd(d02, mul_mi(d13));
    v[3] = csub(d02, mul_mi(d13));
  }
};

template <>
struct Dft<8> {
  __device__ static void run(C *v, const C *) {
    C e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
    Dft<4>::run(e, nullptr);
    Dft<4>::run(o, nullptr);
    const RT h = (RT)0.70710678118654752440;
    // o_k *= W_8^k
    o[1] = mkc(h * (o[1].x + o[1].y), h * (o[1].y - o[1].x));
    o[2] = mul_mi(o[2]);
    o[3] = mkc(h * (o[3].y - o[3].x), -h * (o[3].x + o[3].y));
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
  __device__ static void run(C *v, const C *wr) {
    constexpr int H = (R - 1) / 2;
    C s[H + 1], d[H + 1];
    C x0 = v[0];
#pragma unroll
    for (int r = 1; r <= H; r++) {
      s[r] = cadd(v[r], v[R - r]);
      d[r] = csub(v[r], v[R - r]);
      x0 = cadd(x0, s[r]);
    }
    C out[R];
    out[0] = x0;
#pragma unroll
    for (int q = 1; q <= H; q++) {
      C A = v[0], B = mkc((RT)0, (RT)0);
#pragma unroll
      for (int r = 1; r <= H; r++) {
        const C w = wr[OFF + (r * q) % R];
        const RT c = w.x, sn = -w.y;
        A.x = fma(s[r].x, c, A.x);
        A.y = fma(s[r].y, c, A.y);
        B.x = fma(d[r].x, sn, B.x);
        B.y = fma(d[r].y, sn, B.y);
      }
      out[q] = mkc(A.x + B.y, A.y - B.x);
      out[R - q] = mkc(A.x - B.y, A.y + B.x);
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
__device__ __forceinline__ C cmulc(C a, RT c, RT s) {  // a (c + i s)
  return mkc(a.x * c - a.y * s, a.x * s + a.y * c);
}
template <>
struct Dft<16> {
  __device__ static void run(C *v, const C *) {
    const RT c1 = (RT)0.92387953251128674785, s1 = (RT)0.38268343236508977173, h = (RT)0.70710678118654752440;
    C y[4][4];
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
      C t[4] = {y[0][k1], y[1][k1], y[2][k1], y[3][k1]};
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
  __device__ static void run(C *v, const C *wr) {
    constexpr int R = R1 * R2, e1 = inv_mod(R2 % R1, R1), e2 = inv_mod(R1 % R2, R2);
    C a[R2][R1];
#pragma unroll
    for (int n2 = 0; n2 < R2; n2++) {
#pragma unroll
      for (int n1 = 0; n1 < R1; n1++) a[n2][n1] = v[(n1 * R2 + n2 * R1) % R];
      Dft<R1>::run(a[n2], wr);
    }
#pragma unroll
    for (int k1 = 0; k1 < R1; k1++) {
      C c[R2];
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

// one-element (4 or 8 byte) asynchronous global -> shared copy; !valid
// zero-fills (src must still be a mapped address)
__device__ __forceinline__ void cp4(void *dst, const void *src, bool valid) {
  if (sizeof(RT) == 4)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(valid ? 4 : 0)
                 : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(valid ? 8 : 0)
                 : "memory");
}

struct WrTable {
  C w[WRN];
};

__device__ __forceinline__ const C *tab(const void *t) { return static_cast<const C *>(t); }

// Stage indexing shared by both passes: butterfly q of a stage with span Ns
// is group g = q / Ns, offset k = q % Ns.  The division is done as
// trunc((q + 1/2) / Ns) in FP32: q < 1536 and Ns <= 1536, so (q + 1/2) / Ns
// lies at least 1/(2 Ns) from an integer, far above the rounding error of
// the product (checked exhaustively for all q, Ns < 2048).

// ---- pass A ------------------------------------------------------------
// A CTA runs FB transforms (FB consecutive j1) with Cfg<FB>::NT threads.  The
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

// threads per CTA by transforms per CTA (FB_HI on passes short enough for
// two such CTAs per SM, FB_LO on longer ones), and the CTAs per SM the
// register budget is sized for
template <int FB>
struct Cfg {
  static constexpr int NT = FB == FB_HI ? NT_HI : NT_LO;
  static constexpr int MINB = FB == FB_HI ? MINB_HI : MINB_LO;
};

struct PassA {
  const RT *x1, *x2;
  const C *U;  // AM_CPLX: this pair's sequence
  const C *chirp;
  bool has2;
  int L1, j1_0, nb, m, Lx, M;
  const int *iperm;
};

// input at position j: the even extension e_j (AM_DCT, j < 2m); for
// Bluestein, z_{|i|} c_{|i|} at the position j = i mod M of i in [-m + 1, m]
// and zero in between; or the sequence U
template <int AM>
__device__ __forceinline__ C a_input(const PassA &pa, int j) {
  if (AM == AM_CPLX) return pa.U[j];
  if (AM == AM_BLUE && j > pa.m && j <= pa.M - pa.m) return mkc((RT)0, (RT)0);
  const int jj = j <= pa.m ? j : (AM == AM_BLUE ? pa.M : pa.Lx) - j;
  const C z = mkc(__ldg(pa.x1 + jj), pa.has2 ? __ldg(pa.x2 + jj) : (RT)0);
  return AM == AM_BLUE ? cmul(z, __ldg(pa.chirp + jj)) : z;
}

template <int R, bool FIRST, int AM, int FB>
__device__ __forceinline__ void astage(C *sbuf, int pitch, int Ls, int Ns, float invNs, const C *stw,
                                       const C *wr, const PassA &pa) {
  const int nq = Ls / R;
  for (int bf = threadIdx.x; bf < FB * nq; bf += Cfg<FB>::NT) {
    const int b = bf % FB, q = bf / FB;
    if (b >= pa.nb) continue;
    const int g = __float2int_rz(((float)q + 0.5f) * invNs);
    const int k = q - g * Ns;
    C v[R];
    C *a = sbuf + b * pitch + g * Ns * R + k;
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
__device__ __forceinline__ void astage_r(int R, C *sbuf, int pitch, int Ls, int Ns, float invNs,
                                         const C *stw, const C *wr, const PassA &pa) {
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
__device__ __forceinline__ void astage_last(const C *sbuf, int pitch, int Ns, const C *stw,
                                            const C *wr, const PassA &pa, const Fft4Dev &p,
                                            C *Tp) {
  for (int bf = threadIdx.x; bf < FB * Ns; bf += Cfg<FB>::NT) {
    const int b = bf / Ns, q = bf - b * Ns;
    if (b >= pa.nb) break;  // b grows with bf
    const C *a = sbuf + b * pitch + q;
    C v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = a[r * Ns];
#pragma unroll
    for (int r = 1; r < R; r++) v[r] = cmul(v[r], __ldg(stw + (r - 1) * Ns + q));
    Dft<R>::run(v, wr);
    const int j1 = pa.j1_0 + b;
    const C *tl = tab(p.tlane) + 32 * j1, *tb = tab(p.tblk) + j1 * p.nb32;
    C *row = Tp + (int64_t)j1 * p.L2;
#pragma unroll
    for (int r = 0; r < R; r++) {
      const int k2 = q + r * Ns;
      row[k2] = cmul(v[r], cmul(__ldg(tb + (k2 >> 5)), __ldg(tl + (k2 & 31))));
    }
  }
}

template <int FB>
__device__ __forceinline__ void astage_last_r(int R, const C *sbuf, int pitch, int Ns, const C *stw,
                                              const C *wr, const PassA &pa, const Fft4Dev &p, C *Tp) {
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

// row pitch (C) of a tile of FB interleaved transforms: odd, so the
// rows fall in distinct shared-memory banks
__host__ __device__ __forceinline__ int pitch_odd(int Ls) { return Ls | 1; }

// pass A: rows (2 pair, 2 pair + 1) of x (or the pair's U) -> T[pair]
// (L1 x L2, twiddled)
template <int AM, int FB>
__global__ void __launch_bounds__(Cfg<FB>::NT, Cfg<FB>::MINB) k_fft4_a(const RT *__restrict__ x, int64_t ldx,
                                                    const C *__restrict__ U, int64_t nrow,
                                                    C *__restrict__ T, const Fft4Dev p, const WrTable wt) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *const sbuf = reinterpret_cast<C *>(smem_raw);
  const int L1 = p.L1, L2 = p.L2, pitch = pitch_odd(L2), tid = threadIdx.x;
  const int64_t pair = blockIdx.y, r0 = 2 * pair;
  PassA pa;
  pa.has2 = r0 + 1 < nrow;
  pa.x1 = AM == AM_CPLX ? nullptr : x + r0 * ldx;
  pa.x2 = AM == AM_CPLX ? nullptr : pa.has2 ? pa.x1 + ldx : pa.x1;
  pa.U = AM == AM_CPLX ? U + pair * p.L : nullptr;
  pa.chirp = tab(p.chirp);
  pa.L1 = L1;
  pa.j1_0 = blockIdx.x * FB;
  pa.nb = min(FB, L1 - pa.j1_0);
  pa.m = (int)p.m;
  pa.Lx = (int)p.Lx;
  pa.M = (int)p.L;
  pa.iperm = p.iperm2;
  C *Tp = T + pair * p.L;
  const int S = p.nr2;
  if (S >= 2) {
    astage_r<true, AM, FB>(p.r2[0], sbuf, pitch, L2, 1, 1.0f, tab(p.stw2), wt.w, pa);
    for (int s = 1; s < S - 1; s++) {
      __syncthreads();
      astage_r<false, AM, FB>(p.r2[s], sbuf, pitch, L2, p.ns2[s], p.inv2[s], tab(p.stw2) + p.to2[s], wt.w, pa);
    }
    __syncthreads();
    astage_last_r<FB>(p.r2[S - 1], sbuf, pitch, p.ns2[S - 1], tab(p.stw2) + p.to2[S - 1], wt.w, pa, p, Tp);
    return;
  }
  // one stage at most (L2 <= 16): into shared memory, then each warp
  // twiddles rows b by W_L^{j1 k2} and stores them
  if (S == 0) {  // L2 == 1: the column is its own transform
    if (tid < pa.nb) sbuf[tid * pitch] = a_input<AM>(pa, pa.j1_0 + tid);
  } else {
    astage_r<true, AM, FB>(p.r2[0], sbuf, pitch, L2, 1, 1.0f, tab(p.stw2), wt.w, pa);
  }
  __syncthreads();
  const int lane = tid & 31;
  for (int b = tid >> 5; b < pa.nb; b += Cfg<FB>::NT / 32) {
    const C *row = sbuf + b * pitch;
    const int j1 = pa.j1_0 + b;
    const C tl = __ldg(tab(p.tlane) + 32 * j1 + lane);
    const C *tb = tab(p.tblk) + j1 * p.nb32;
    for (int i = 0; i < p.nb32; i++) {
      const int k2 = 32 * i + lane;
      if (k2 < L2) Tp[(int64_t)j1 * L2 + k2] = cmul(row[k2], cmul(__ldg(tb + i), tl));
    }
  }
}

// ---- pass B ------------------------------------------------------------
// The CTA's FB transforms (FB consecutive k2) are interleaved over its
// Cfg<FB>::NT threads: butterfly bf of a stage belongs to row b = bf % FB, so the
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
  const C *Tp;  // this pair's T (L1 x L2)
  C *U;         // BM_MUL: this pair's output sequence
  const C *bhat, *chirp;
  int L2, k2_0, nb, m, epi;
  bool has2;
  RT *o1, *o2;
  const RT *sw;        // prefetched weights, [k1][b][row], or null
  const RT *w1, *w2;      // else the weight rows, read in the last stage
  const int *iperm;
};

template <int R, bool FIRST, bool LAST, int BM, int FB>
__device__ __forceinline__ void bstage(C *sbuf, int pitch, int Ls, int Ns, float invNs, const C *stw,
                                       const C *wr, const PassB &pb) {
  const int nq = Ls / R;
  for (int bf = threadIdx.x; bf < FB * nq; bf += Cfg<FB>::NT) {
    const int b = bf % FB, q = bf / FB;
    if (b >= pb.nb) continue;
    const int g = __float2int_rz(((float)q + 0.5f) * invNs);
    const int k = q - g * Ns;
    C v[R];
    if (FIRST) {  // Ns == 1: g == q, k == 0
      const int jg = __ldg(pb.iperm + q * R);
#pragma unroll
      for (int r = 0; r < R; r++) v[r] = pb.Tp[(jg + (Ls / R) * r) * pb.L2 + pb.k2_0 + b];
    } else {
      const C *a = sbuf + b * pitch + g * Ns * R + k;
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
          const C f = cmul(v[r], __ldg(pb.bhat + kk));
          pb.U[kk] = mkc(f.x, -f.y);
          continue;
        }
        if (kk > pb.m) continue;
        if (BM == BM_BLUE) v[r] = cmul(mkc(v[r].x, -v[r].y), __ldg(pb.chirp + kk));
        RT a = v[r].x, c = v[r].y;
        if (pb.epi == FFT4_FILTER) {
          if (pb.sw) {
            a *= pb.sw[2 * (k1 * FB + b)];
            c *= pb.sw[2 * (k1 * FB + b) + 1];
          } else {
            a *= __ldg(pb.w1 + kk);
            if (pb.has2) c *= __ldg(pb.w2 + kk);
          }
        } else if (pb.epi == FFT4_HALVE && (kk == 0 || kk == pb.m)) {
          a *= (RT)0.5;
          c *= (RT)0.5;
        }
        pb.o1[kk] = a;
        if (pb.has2) pb.o2[kk] = c;
      }
    } else {
      C *a = sbuf + b * pitch + g * Ns * R + k;
#pragma unroll
      for (int r = 0; r < R; r++) a[r * Ns] = v[r];
    }
  }
}

template <bool FIRST, bool LAST, int BM, int FB>
__device__ __forceinline__ void bstage_r(int R, C *sbuf, int pitch, int Ls, int Ns, float invNs,
                                         const C *stw, const C *wr, const PassB &pb) {
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
__global__ void __launch_bounds__(Cfg<FB>::NT, Cfg<FB>::MINB) k_fft4_b(const C *__restrict__ T, int64_t nrow,
                                                    RT *__restrict__ out, int64_t ldo, C *__restrict__ U,
                                                    const RT *__restrict__ w, int64_t ldw, int epi,
                                                    int wpre, const Fft4Dev p, const WrTable wt) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *const sbuf = reinterpret_cast<C *>(smem_raw);
  const int L1 = p.L1, L2 = p.L2, pitch = pitch_odd(L1), tid = threadIdx.x;
  const int64_t pair = blockIdx.y, r0 = 2 * pair;
  PassB pb;
  pb.has2 = r0 + 1 < nrow;
  pb.k2_0 = blockIdx.x * FB;
  pb.nb = min(FB, L2 - pb.k2_0);
  pb.Tp = T + pair * p.L;
  pb.U = BM == BM_MUL ? U + pair * p.L : nullptr;
  pb.bhat = tab(p.bhat);
  pb.chirp = tab(p.chirp);
  pb.L2 = L2;
  pb.m = (int)p.m;
  pb.epi = epi;
  pb.o1 = BM == BM_MUL ? nullptr : out + r0 * ldo;
  pb.o2 = BM == BM_MUL ? nullptr : pb.o1 + ldo;
  pb.iperm = p.iperm1;
  pb.sw = nullptr;
  pb.w1 = pb.w2 = nullptr;
  if (BM != BM_MUL && epi == FFT4_FILTER) {
    const RT *w1 = w + r0 * ldw;
    const RT *w2 = pb.has2 ? w1 + ldw : w1;
    pb.w1 = w1;
    pb.w2 = w2;
    if (wpre) {
      // the weights of this tile's outputs, [k1][b][row], prefetched during
      // the first stages (when two CTAs still fit an SM with them)
      RT *sw = reinterpret_cast<RT *>(sbuf + FB * pitch);
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
    bstage_r<true, true, BM, FB>(p.r1[0], sbuf, pitch, L1, 1, 1.0f, tab(p.stw1), wt.w, pb);
    return;
  }
  bstage_r<true, false, BM, FB>(p.r1[0], sbuf, pitch, L1, 1, 1.0f, tab(p.stw1), wt.w, pb);
  __syncthreads();
  for (int s = 1; s < S - 1; s++) {
    bstage_r<false, false, BM, FB>(p.r1[s], sbuf, pitch, L1, p.ns1[s], p.inv1[s], tab(p.stw1) + p.to1[s], wt.w, pb);
    __syncthreads();
  }
  cp_async_wait_all();
  __syncthreads();
  bstage_r<false, true, BM, FB>(p.r1[S - 1], sbuf, pitch, L1, p.ns1[S - 1], p.inv1[S - 1],
                                tab(p.stw1) + p.to1[S - 1], wt.w, pb);
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
  const C *Tp;  // this pair's T (L1 x L2)
  C *Vp;        // this pair's V (L2 x L1)
  const C *bhat;
  int L1, L2, k2_0, nb;
};

// the first decimation-in-frequency stage (span Ns = L1 / R): natural-order
// inputs k + r Ns from T's column, butterfly, twiddle after it
template <int R, int FB>
__device__ __forceinline__ void cstage_first(C *sbuf, int pitch, int Ns, const C *stw, const C *wr,
                                             const PassC &pc) {
  for (int bf = threadIdx.x; bf < FB * Ns; bf += Cfg<FB>::NT) {
    const int b = bf % FB, q = bf / FB;
    if (b >= pc.nb) continue;
    C v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = pc.Tp[(int64_t)(q + r * Ns) * pc.L2 + pc.k2_0 + b];
    Dft<R>::run(v, wr);
#pragma unroll
    for (int r = 1; r < R; r++) v[r] = cmul(v[r], __ldg(stw + (r - 1) * Ns + q));
    C *a = sbuf + b * pitch + q;
#pragma unroll
    for (int r = 0; r < R; r++) a[r * Ns] = v[r];
  }
}

// a decimation-in-frequency stage in shared memory (twiddles after the
// butterfly), same butterfly indexing as the decimation-in-time stages
template <int R, int FB>
__device__ __forceinline__ void cstage_dif(C *sbuf, int pitch, int Ls, int Ns, float invNs, const C *stw,
                                           const C *wr, int nb) {
  const int nq = Ls / R;
  for (int bf = threadIdx.x; bf < FB * nq; bf += Cfg<FB>::NT) {
    const int b = bf % FB, q = bf / FB;
    if (b >= nb) continue;
    const int g = __float2int_rz(((float)q + 0.5f) * invNs);
    const int k = q - g * Ns;
    C *a = sbuf + b * pitch + g * Ns * R + k;
    C v[R];
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
__device__ __forceinline__ void cstage_mid(C *sbuf, int pitch, int L1, const int *iperm, const C *wr,
                                           const PassC &pc) {
  const int nq = L1 / R;
  for (int bf = threadIdx.x; bf < FB * nq; bf += Cfg<FB>::NT) {
    const int b = bf % FB, q = bf / FB;
    if (b >= pc.nb) continue;
    C *a = sbuf + b * pitch + q * R;
    C v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = a[r];
    Dft<R>::run(v, wr);
    const int k1 = __ldg(iperm + q * R);
#pragma unroll
    for (int r = 0; r < R; r++) {
      const C f = cmul(v[r], __ldg(pc.bhat + pc.k2_0 + b + (int64_t)pc.L2 * (k1 + (L1 / R) * r)));
      v[r] = mkc(f.x, -f.y);
    }
    Dft<R>::run(v, wr);
#pragma unroll
    for (int r = 0; r < R; r++) a[r] = v[r];
  }
}

// a decimation-in-time stage in shared memory (twiddles before the butterfly)
template <int R, int FB>
__device__ __forceinline__ void cstage_dit(C *sbuf, int pitch, int Ls, int Ns, float invNs, const C *stw,
                                           const C *wr, int nb) {
  const int nq = Ls / R;
  for (int bf = threadIdx.x; bf < FB * nq; bf += Cfg<FB>::NT) {
    const int b = bf % FB, q = bf / FB;
    if (b >= nb) continue;
    const int g = __float2int_rz(((float)q + 0.5f) * invNs);
    const int k = q - g * Ns;
    C *a = sbuf + b * pitch + g * Ns * R + k;
    C v[R];
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
__device__ __forceinline__ void cstage_last(const C *sbuf, int pitch, int Ns, const C *stw,
                                            const C *wr, const PassC &pc, const Fft4Dev &p) {
  for (int bf = threadIdx.x; bf < FB * Ns; bf += Cfg<FB>::NT) {
    const int b = bf / Ns, q = bf - b * Ns;
    if (b >= pc.nb) break;
    const C *a = sbuf + b * pitch + q;
    C v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = a[r * Ns];
#pragma unroll
    for (int r = 1; r < R; r++) v[r] = cmul(v[r], __ldg(stw + (r - 1) * Ns + q));
    Dft<R>::run(v, wr);
    const int k2 = pc.k2_0 + b;
    const C *tl = tab(p.tlane2) + 32 * k2, *tb = tab(p.tblk2) + k2 * p.nb32b;
    C *row = pc.Vp + (int64_t)k2 * pc.L1;
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
__global__ void __launch_bounds__(Cfg<FB>::NT, Cfg<FB>::MINB) k_fft4_conv(const C *__restrict__ T, C *__restrict__ V,
                                                     const Fft4Dev p, const WrTable wt) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *const sbuf = reinterpret_cast<C *>(smem_raw);
  const int L1 = p.L1, pitch = pitch_odd(L1), S = p.nr1;
  const int64_t pair = blockIdx.y;
  PassC pc;
  pc.Tp = T + pair * p.L;
  pc.Vp = V + pair * p.L;
  pc.bhat = tab(p.bhat);
  pc.L1 = L1;
  pc.L2 = p.L2;
  pc.k2_0 = blockIdx.x * FB;
  pc.nb = min(FB, p.L2 - pc.k2_0);
  MK_RADIX_SWITCH(p.r1[S - 1], (cstage_first<RR, FB>(sbuf, pitch, p.ns1[S - 1], tab(p.stw1) + p.to1[S - 1], wt.w, pc)));
  __syncthreads();
  for (int s = S - 2; s >= 1; s--) {
    MK_RADIX_SWITCH(p.r1[s], (cstage_dif<RR, FB>(sbuf, pitch, L1, p.ns1[s], p.inv1[s], tab(p.stw1) + p.to1[s], wt.w,
                                                 pc.nb)));
    __syncthreads();
  }
  MK_RADIX_SWITCH(p.r1[0], (cstage_mid<RR, FB>(sbuf, pitch, L1, p.iperm1, wt.w, pc)));
  __syncthreads();
  for (int s = 1; s < S - 1; s++) {
    MK_RADIX_SWITCH(p.r1[s], (cstage_dit<RR, FB>(sbuf, pitch, L1, p.ns1[s], p.inv1[s], tab(p.stw1) + p.to1[s], wt.w,
                                                 pc.nb)));
    __syncthreads();
  }
  MK_RADIX_SWITCH(p.r1[S - 1], (cstage_last<RR, FB>(sbuf, pitch, p.ns1[S - 1], tab(p.stw1) + p.to1[S - 1], wt.w, pc, p)));
}
#undef MK_RADIX_SWITCH
#undef MK_RCASE12
#undef MK_RCASE14
#undef MK_RCASE15
#undef MK_RCASE16


// radix constants W_R^t for the odd radices, in double, rounded to RT
inline WrTable make_wr() {
  WrTable t;
  const int rs[5] = {3, 5, 7, 9, 11}, off[5] = {WR3, WR5, WR7, WR9, WR11};
  for (int i = 0; i < 5; i++)
    for (int k = 0; k < rs[i]; k++) {
      const double a = 2.0 * M_PI * (double)k / (double)rs[i];
      t.w[off[i] + k] = mkc((RT)std::cos(a), (RT)-std::sin(a));
    }
  return t;
}

bool g_attr[64] = {false};

// out rows = DCT-I of x rows with the epilogue (see mk_fft4.cuh)
int dct_launch(const Fft4Plan &p, const RT *x, int64_t ldx, int64_t nrow, C *T, RT *out, int64_t ldo, int epi,
               const RT *w, int64_t ldw, cudaStream_t st) {
  const Fft4Dev &d = p.d;
  const int64_t npairs = (nrow + 1) / 2;
  MK_CHECK_ARG(npairs >= 1 && npairs <= 65535, "fft4: %lld rows out of range", (long long)nrow);
  MK_CHECK_ARG(ldx >= d.n && ldo >= d.n, "fft4: leading dimensions below the row length");
  MK_CHECK_ARG(epi != FFT4_FILTER || (w && ldw >= d.n), "fft4: filter weights missing");
  MK_CHECK_ARG(d.f64 == (sizeof(RT) == 8), "fft4: plan precision does not match the call");
  int dev = 0;
  MK_CUDA(cudaGetDevice(&dev));
  if (dev >= 0 && dev < 64 && !g_attr[dev]) {
    const int mhi = FB_HI * (FFT4_LMAX + 1) * (int)sizeof(C);
    const int mlo = FB_LO * (FFT4_LMAX + 1) * (int)sizeof(C) + FB_LO * FFT4_LMAX * 2 * (int)sizeof(RT);
#define MK_FFT4_ATTR(k, v) MK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, v))
    MK_FFT4_ATTR((k_fft4_a<AM_DCT, FB_LO>), mlo);
    MK_FFT4_ATTR((k_fft4_a<AM_BLUE, FB_LO>), mlo);
    MK_FFT4_ATTR((k_fft4_a<AM_CPLX, FB_LO>), mlo);
    MK_FFT4_ATTR((k_fft4_b<BM_DCT, FB_LO>), mlo);
    MK_FFT4_ATTR((k_fft4_b<BM_MUL, FB_LO>), mlo);
    MK_FFT4_ATTR((k_fft4_b<BM_BLUE, FB_LO>), mlo);
    MK_FFT4_ATTR((k_fft4_a<AM_DCT, FB_HI>), mhi);
    MK_FFT4_ATTR((k_fft4_a<AM_BLUE, FB_HI>), mhi);
    MK_FFT4_ATTR((k_fft4_a<AM_CPLX, FB_HI>), mhi);
    MK_FFT4_ATTR((k_fft4_b<BM_DCT, FB_HI>), mhi);
    MK_FFT4_ATTR((k_fft4_b<BM_MUL, FB_HI>), mhi);
    MK_FFT4_ATTR((k_fft4_b<BM_BLUE, FB_HI>), mhi);
    MK_FFT4_ATTR((k_fft4_conv<FB_LO>), mlo);
    MK_FFT4_ATTR((k_fft4_conv<FB_HI>), mhi);
#undef MK_FFT4_ATTR
    g_attr[dev] = true;
  }
  static const WrTable wt = make_wr();
  const bool hia = d.fba == FB_HI, hib = d.fbb == FB_HI;
  const int fa = hia ? FB_HI : FB_LO, fb = hib ? FB_HI : FB_LO;
  const dim3 ga((d.L1 + fa - 1) / fa, (unsigned)npairs), gb((d.L2 + fb - 1) / fb, (unsigned)npairs);
  const size_t smem_a = (size_t)fa * pitch_odd(d.L2) * sizeof(C);
  const size_t smem_b = (size_t)fb * pitch_odd(d.L1) * sizeof(C);
  // FILTER weights go through shared memory on FB_LO passes while two CTAs
  // still fit an SM; otherwise the last stage reads them directly
  const size_t smem_wlo = (size_t)FB_LO * d.L1 * 2 * sizeof(RT);
  const int wpre = epi == FFT4_FILTER && !hib && smem_b + smem_wlo <= 113 * 1024;
  const size_t smem_w = wpre ? smem_wlo : 0;
  auto pass_a = [&](int am, const RT *xx, int64_t ldxx, const C *uu) {
    if (hia) {
      if (am == AM_DCT) k_fft4_a<AM_DCT, FB_HI><<<ga, Cfg<FB_HI>::NT, smem_a, st>>>(xx, ldxx, uu, nrow, T, d, wt);
      else if (am == AM_BLUE) k_fft4_a<AM_BLUE, FB_HI><<<ga, Cfg<FB_HI>::NT, smem_a, st>>>(xx, ldxx, uu, nrow, T, d, wt);
      else k_fft4_a<AM_CPLX, FB_HI><<<ga, Cfg<FB_HI>::NT, smem_a, st>>>(xx, ldxx, uu, nrow, T, d, wt);
    } else {
      if (am == AM_DCT) k_fft4_a<AM_DCT, FB_LO><<<ga, Cfg<FB_LO>::NT, smem_a, st>>>(xx, ldxx, uu, nrow, T, d, wt);
      else if (am == AM_BLUE) k_fft4_a<AM_BLUE, FB_LO><<<ga, Cfg<FB_LO>::NT, smem_a, st>>>(xx, ldxx, uu, nrow, T, d, wt);
      else k_fft4_a<AM_CPLX, FB_LO><<<ga, Cfg<FB_LO>::NT, smem_a, st>>>(xx, ldxx, uu, nrow, T, d, wt);
    }
  };
  auto pass_b = [&](int bm, C *uu, int e, size_t sm, int wp) {
    if (hib) {
      if (bm == BM_DCT)
        k_fft4_b<BM_DCT, FB_HI><<<gb, Cfg<FB_HI>::NT, sm, st>>>(T, nrow, out, ldo, uu, w, ldw, e, wp, d, wt);
      else if (bm == BM_MUL)
        k_fft4_b<BM_MUL, FB_HI><<<gb, Cfg<FB_HI>::NT, sm, st>>>(T, nrow, out, ldo, uu, w, ldw, e, wp, d, wt);
      else
        k_fft4_b<BM_BLUE, FB_HI><<<gb, Cfg<FB_HI>::NT, sm, st>>>(T, nrow, out, ldo, uu, w, ldw, e, wp, d, wt);
    } else {
      if (bm == BM_DCT)
        k_fft4_b<BM_DCT, FB_LO><<<gb, Cfg<FB_LO>::NT, sm, st>>>(T, nrow, out, ldo, uu, w, ldw, e, wp, d, wt);
      else if (bm == BM_MUL)
        k_fft4_b<BM_MUL, FB_LO><<<gb, Cfg<FB_LO>::NT, sm, st>>>(T, nrow, out, ldo, uu, w, ldw, e, wp, d, wt);
      else
        k_fft4_b<BM_BLUE, FB_LO><<<gb, Cfg<FB_LO>::NT, sm, st>>>(T, nrow, out, ldo, uu, w, ldw, e, wp, d, wt);
    }
  };
  int rc;
  if (!d.blue) {
    pass_a(AM_DCT, x, ldx, nullptr);
    if ((rc = launch_status("fft4 pass A"))) return rc;
    pass_b(BM_DCT, nullptr, epi, smem_b + smem_w, wpre);
    return launch_status("fft4 pass B");
  }
  C *U = T + npairs * d.L;
  pass_a(AM_BLUE, x, ldx, nullptr);
  if ((rc = launch_status("fft4 Bluestein pass A"))) return rc;
  if (d.nr1 >= 2 && !d.blue4) {
    // the middle pass T -> V (= U's space), then pass B on the transposed
    // shape: length L2 over the rows of V, outputs o1 + L1 o2
    const size_t smem_c = (size_t)fb * pitch_odd(d.L1) * sizeof(C);
    if (hib) k_fft4_conv<FB_HI><<<gb, Cfg<FB_HI>::NT, smem_c, st>>>(T, U, d, wt);
    else k_fft4_conv<FB_LO><<<gb, Cfg<FB_LO>::NT, smem_c, st>>>(T, U, d, wt);
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
    const size_t smem_t = (size_t)fa * pitch_odd(tr.L1) * sizeof(C);
    const size_t smem_twlo = (size_t)FB_LO * tr.L1 * 2 * sizeof(RT);
    const int wpre_t = epi == FFT4_FILTER && !hia && smem_t + smem_twlo <= 113 * 1024;
    const size_t smem_tw = wpre_t ? smem_twlo : 0;
    if (hia)
      k_fft4_b<BM_BLUE, FB_HI><<<gt, Cfg<FB_HI>::NT, smem_t, st>>>(U, nrow, out, ldo, nullptr, w, ldw, epi, 0, tr,
                                                                   wt);
    else
      k_fft4_b<BM_BLUE, FB_LO><<<gt, Cfg<FB_LO>::NT, smem_t + smem_tw, st>>>(U, nrow, out, ldo, nullptr, w, ldw, epi,
                                                                             wpre_t, tr, wt);
    return launch_status("fft4 Bluestein last pass");
  }
  pass_b(BM_MUL, U, FFT4_PLAIN, smem_b, 0);
  if ((rc = launch_status("fft4 Bluestein pass B"))) return rc;
  pass_a(AM_CPLX, nullptr, 0, U);
  if ((rc = launch_status("fft4 Bluestein pass A (second)"))) return rc;
  pass_b(BM_BLUE, nullptr, epi, smem_b + smem_w, wpre);
  return launch_status("fft4 Bluestein pass B (second)");
}

}  // namespace MK_FFT4_NS
}  // namespace mk
