// DCT-I of detector rows by a four-step FFT in shared memory (FP32 and FP64).
//
// DCT-I of a row x (length n = m + 1) is the DFT of its even extension
// e_j = x_{min(j, 2m - j)} (length L = 2m), which is real.  Two rows r, r+1
// therefore share one complex transform: F = DFT(e_r + i e_{r+1}) gives
// DCT(x_r)_k = Re F_k and DCT(x_{r+1})_k = Im F_k, k = 0..m.
//
// With L = L1 L2 (both <= FFT4_LMAX, factors in {2,3,5,7,11}), j = j1 + L1 j2
// and k = k2 + L2 k1:
//   pass A: for each j1, T[j1][k2] = W_L^{j1 k2} sum_j2 e_{j1 + L1 j2} W_L2^{j2 k2}
//   pass B: for each k2, F[k2 + L2 k1] = sum_j1 T[j1][k2] W_L1^{j1 k1}
// Each CTA runs 8 or 16 (FP64: 4 or 8) transforms of one pass in shared memory (mixed-radix
// decimation in time, butterflies in place), interleaved over its threads.
// The first stage of each pass reads its inputs straight from global memory
// (pass A forms the even extension there); pass A's last stage twiddles its
// outputs and stores them to T; pass B's last stage writes only k <= m
// straight to the rows with the epilogue (plain, times the inverse-spectrum
// weights, or with columns 0 and m halved).  Twiddles come from tables computed in
// double precision on the host.
//
// Lengths whose 2m has a prime factor above 11 (minkasi's truncate_tod leaves
// some) go through Bluestein's algorithm on the same passes.  With the chirp
// c_t = exp(-i pi t^2 / 2m) (even in t), W^{jk} = c_j c_k conj(c_{k-j}) for
// W = exp(-i pi / m), and the extension is periodic in j with period 2m, so
//   F_k = c_k sum_{j=-m+1}^{m} (e_j c_j) conj(c_{k-j}),   e_{-j} = e_j = z_{|j|}.
// Only k = 0..m are needed, so the lags k - j cover [-m, 2m - 1]: 3m values.
// F is then a circular convolution a (*) b of a smooth length M >= 3m, with
// a at positions j mod M (z_{|j|} c_{|j|}, zero elsewhere) and b_t = conj(c_t)
// at t mod M for t in [-m, 2m - 1] (one quarter shorter than the M >= 4m - 1
// of taking j, k over a whole period).  Pass A forms a from the rows; a
// middle pass finishes DFT(a) column by column, multiplies by
// B^ = DFT_M(b) / M, conjugates (U = conj(DFT(a) B^)) and runs the first
// step of DFT(U) on the same column in shared memory; pass B on the
// transposed shape finishes DFT(U) and writes c_k conj(DFT(U)_k) for k <= m
// with the usual epilogue (three passes; four when L1 takes one stage).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace mk {

constexpr int FFT4_LMAX = 1536;  // longest transform of one pass
// largest radix the kernels hold in registers, FP32 and FP64
#ifndef MK_FFT4_RMAX
#define MK_FFT4_RMAX 16
#endif
#ifndef MK_FFT4_RMAX64
#define MK_FFT4_RMAX64 16
#endif
constexpr int FFT4_MAXR = 16;    // most radix stages of one pass

// device view of a plan (kernel argument)
struct Fft4Dev {
  int64_t n, m, L;  // row length, m = n - 1, transform length (2m, or M for Bluestein)
  int64_t Lx;       // even-extension length 2m
  bool blue;        // Bluestein: L = M, chirp and bhat set
  bool f64;         // FP64 plan: tables of double2, FP64 kernels
  bool blue4;       // Bluestein in four passes (U written out) instead of three
  int L1, L2, nb32;  // nb32 = ceil(L2 / 32)
  int fba, fbb;      // transforms per CTA of pass A (length L2) and pass B (length L1): 8 or 16
  int nr1, nr2;
  int r1[FFT4_MAXR], r2[FFT4_MAXR];
  // per stage: span Ns of the earlier stages, 1 / Ns, offset of its twiddles
  int ns1[FFT4_MAXR], ns2[FFT4_MAXR], to1[FFT4_MAXR], to2[FFT4_MAXR];
  float inv1[FFT4_MAXR], inv2[FFT4_MAXR];
  // complex tables (float2 or double2 by precision)
  // stage twiddles W_{Ns R}^{r k} at [to + (r - 1) Ns + k]
  const void *stw1, *stw2;
  const int *iperm1, *iperm2;  // natural index at each digit-reversed (DIT input) position
  // four-step twiddle W_L^{j1 k2} = tblk[j1 nb32 + k2 / 32] * tlane[32 j1 + k2 % 32]
  const void *tlane, *tblk;
  const void *chirp;  // Bluestein: c_t, t <= m
  const void *bhat;   // Bluestein: DFT_M(b) / M
  // Bluestein's middle pass: W_M^{k2 o1} = tblk2[k2 nb32b + o1 / 32] * tlane2[32 k2 + o1 % 32]
  const void *tlane2, *tblk2;
  int nb32b;  // ceil(L1 / 32)
};

// epilogues of pass B
enum { FFT4_PLAIN = 0, FFT4_FILTER = 1, FFT4_HALVE = 2 };

struct Fft4Plan {
  Fft4Dev d{};
  void *tables = nullptr;  // device tables (plan-owned memory)
};

// The transform for rows of length n: L = 2(n-1) split into L1 x L2 with
// radix lists, or, when 2(n-1) has a prime factor above 11 and `bluestein`
// is set, the smallest splittable M >= 3(n-1); false when neither fits
// within FFT4_LMAX x FFT4_LMAX.
bool fft4_shape(int64_t n, Fft4Dev *d, bool bluestein = true, bool f64 = false);
// the rank of the L1 x L2 split new plans take (0: closest to sqrt(L))
void fft4_set_split_rank(int r);
int fft4_split_rank();
// bytes of the device tables for that shape
size_t fft4_table_bytes(const Fft4Dev &d);
// bytes of the scratch (T, and U for Bluestein) for nrow rows
size_t fft4_t_bytes(const Fft4Dev &d, int64_t nrow);
// computes the tables on the host (B^ with a double-precision cuFFT
// transform) and uploads them to `dev_tables`
int fft4_init(Fft4Plan *p, int64_t n, void *dev_tables, bool bluestein = true, bool f64 = false);
// out rows (ld ldo) = DCT-I of x rows (ld ldx) with the given epilogue;
// T is scratch of fft4_t_bytes; w (ld ldw) only for FFT4_FILTER.
int fft4_dct(const Fft4Plan &p, const float *x, int64_t ldx, int64_t nrow, float2 *T, float *out,
             int64_t ldo, int epi, const float *w, int64_t ldw, cudaStream_t st);
// the same for an FP64 plan (fft4_init with f64)
int fft4_dct_f64(const Fft4Plan &p, const double *x, int64_t ldx, int64_t nrow, double2 *T, double *out,
                 int64_t ldo, int epi, const double *w, int64_t ldw, cudaStream_t st);

}  // namespace mk
