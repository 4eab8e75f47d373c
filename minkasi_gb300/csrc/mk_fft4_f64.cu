// FP64 DCT-I by the four-step FFT: the kernels of mk_fft4_kern.cuh in
// double precision (8 or 4 transforms per CTA, 256 threads).
#define MK_FFT4_NS f4d
#define MK_FFT4_C double2
#define MK_FFT4_RT double
#define MK_FFT4_FBHI 8
#define MK_FFT4_FBLO 4
#define MK_FFT4_NTHI 256
#define MK_FFT4_NTLO 256
#define MK_FFT4_MINBLO 2
#include "mk_fft4.cuh"
#undef MK_FFT4_RMAX
#define MK_FFT4_RMAX MK_FFT4_RMAX64
#include "mk_fft4_kern.cuh"

namespace mk {

int fft4_dct_f64(const Fft4Plan &p, const double *x, int64_t ldx, int64_t nrow, double2 *T, double *out,
                 int64_t ldo, int epi, const double *w, int64_t ldw, cudaStream_t st) {
  return f4d::dct_launch(p, x, ldx, nrow, T, out, ldo, epi, w, ldw, st);
}

}  // namespace mk
