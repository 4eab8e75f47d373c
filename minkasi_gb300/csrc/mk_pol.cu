// Polarized projections (PolMap).  Stokes maps are pixel-major:
// map[p * npol + k], p = x * ny + y, as the reference's (nx, ny, npol) array.
// With c = cos(twogamma[i]), s = sin(twogamma[i]) and d = dat[i]:
//
//   map2tod  IQU        dat (+)= I + Q c + U s                minkasi/lib/minkasi.c:146-159
//            QU         dat (+)= Q c + U s                    minkasi.c:162-174
//   tod2map  IQU        (I, Q, U)      += (d, d c, d s)       minkasi.c:176-185
//            QU         (Q, U)         += (d c, d s)          minkasi.c:187-194
//            QU_PRECON  (QQ, UU, QU)   += (d c c, d s s, d s c)              minkasi.c:196-207
//            IQU_PRECON (I, Q, U, QQ, QU, UU) += (d, d c, d s, d c c, d s c, d s s)
//                                                              minkasi.c:231-245
//
// The reference evaluates cos/sin of every sample on every call.  Here the
// angle terms are either computed in the kernel from twogamma (the drop-in
// form, FP64) or read from a cos/sin pair computed once per TOD by
// mk_pol_sincos (the pointing is fixed across PCG iterations, so this trades
// 8 more bytes per sample for no FP64 transcendental work on GB300's narrow
// FP64 pipe).  tod2map sums runs of equal pixels over 4 consecutive samples
// per thread in registers and issues one atomic per Stokes component per run.
#include <math.h>

#include "mk_common.cuh"

namespace {

template <int MODE>
struct Pol;
// npol per mode; the integer values are the MK_POL_* codes
template <> struct Pol<MK_POL_QU> { static constexpr int N = 2; };
template <> struct Pol<MK_POL_IQU> { static constexpr int N = 3; };
template <> struct Pol<MK_POL_QU_PRECON> { static constexpr int N = 3; };
template <> struct Pol<MK_POL_IQU_PRECON> { static constexpr int N = 6; };

// per-sample Stokes weights, in the reference's operation order
template <int MODE, typename T>
__device__ __forceinline__ void pol_terms(T d, T c, T s, T (&o)[Pol<MODE>::N]) {
  if constexpr (MODE == MK_POL_QU) {
    o[0] = d * c; o[1] = d * s;
  } else if constexpr (MODE == MK_POL_IQU) {
    o[0] = d; o[1] = d * c; o[2] = d * s;
  } else if constexpr (MODE == MK_POL_QU_PRECON) {
    o[0] = (d * c) * c; o[1] = (d * s) * s; o[2] = (d * s) * c;
  } else {
    o[0] = d; o[1] = d * c; o[2] = d * s;
    o[3] = (d * c) * c; o[4] = (d * s) * c; o[5] = (d * s) * s;
  }
}

// angle terms of sample i: from the cached pair, or sincos of twogamma
template <typename T, bool TRIG>
__device__ __forceinline__ void angle(const T *__restrict__ cs, const T *__restrict__ sn,
                                      const double *__restrict__ tg, int64_t i, T &c, T &s) {
  if constexpr (TRIG) {
    double sd, cd;
    sincos(__ldcs(tg + i), &sd, &cd);
    c = (T)cd;
    s = (T)sd;
  } else {
    c = __ldcs(cs + i);
    s = __ldcs(sn + i);
  }
}

template <int MODE, typename T, bool TRIG, bool ADD>
__global__ void __launch_bounds__(256) k_polmap2tod(T *__restrict__ dat, const T *__restrict__ map,
                                                    const T *__restrict__ cs, const T *__restrict__ sn,
                                                    const double *__restrict__ tg,
                                                    const int32_t *__restrict__ ipix, int64_t n, int64_t npix) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int32_t p = __ldcs(ipix + i);
    T c, s;
    angle<T, TRIG>(cs, sn, tg, i, c, s);
    T v = T(0);
    if ((uint32_t)p < (uint64_t)npix) {
      if constexpr (MODE == MK_POL_IQU) {
        const T *m = map + 3 * (int64_t)p;
        v = __ldg(m) + __ldg(m + 1) * c + __ldg(m + 2) * s;
      } else {
        const T *m = map + 2 * (int64_t)p;
        v = __ldg(m) * c + __ldg(m + 1) * s;
      }
    }
    if (ADD) v = dat[i] + v;
    __stcs(dat + i, v);
  }
}

// ROWS: d = rowval[i / ndata] (1 if rowval is NULL): hit / weight maps
template <int MODE, typename T, bool TRIG, bool ROWS>
__global__ void __launch_bounds__(256) k_tod2polmap(T *__restrict__ map, const T *__restrict__ dat,
                                                    const T *__restrict__ cs, const T *__restrict__ sn,
                                                    const double *__restrict__ tg,
                                                    const int32_t *__restrict__ ipix, int64_t n, int64_t npix,
                                                    const T *__restrict__ rowval, int64_t ndata) {
  constexpr int NP = Pol<MODE>::N;
  constexpr int U = 4;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t nu = (n + U - 1) / U;
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < nu; g += stride) {
    int32_t key = -1;
    T acc[NP];
#pragma unroll
    for (int k = 0; k < NP; k++) acc[k] = T(0);
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int64_t i = g * U + u;
      if (i >= n) break;
      const int32_t p = __ldcs(ipix + i);
      T d;
      if (ROWS)
        d = rowval ? rowval[i / ndata] : T(1);
      else
        d = __ldcs(dat + i);
      T c, s;
      angle<T, TRIG>(cs, sn, tg, i, c, s);
      T o[NP];
      pol_terms<MODE, T>(d, c, s, o);
      if (p != key) {
        if ((uint32_t)key < (uint64_t)npix) {
#pragma unroll
          for (int k = 0; k < NP; k++) atomicAdd(map + (int64_t)key * NP + k, acc[k]);
        }
        key = p;
#pragma unroll
        for (int k = 0; k < NP; k++) acc[k] = o[k];
      } else {
#pragma unroll
        for (int k = 0; k < NP; k++) acc[k] += o[k];
      }
    }
    if ((uint32_t)key < (uint64_t)npix) {
#pragma unroll
      for (int k = 0; k < NP; k++) atomicAdd(map + (int64_t)key * NP + k, acc[k]);
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_pol_sincos(T *__restrict__ cs, T *__restrict__ sn,
                                                    const double *__restrict__ tg, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    double s, c;
    sincos(tg[i], &s, &c);
    cs[i] = (T)c;
    sn[i] = (T)s;
  }
}

// out = P . m per pixel for a PRECON map P and a map m (PolMap.__mul__,
// minkasi/maps/polmap.py:624-684):
//   QU_PRECON (QQ, UU, QU) . (Q, U)
//   IQU_PRECON (I, Q, U, QQ, QU, UU) as the symmetric [a0 a1 a2; a1 a3 a4; a2 a4 a5] . (I, Q, U)
template <typename T>
__global__ void __launch_bounds__(256) k_pol_precon_mul(T *__restrict__ out, const T *__restrict__ P,
                                                        const T *__restrict__ m, int64_t npix, int iqu) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += stride) {
    if (iqu) {
      const T *a = P + 6 * p;
      const T *x = m + 3 * p;
      const T x0 = x[0], x1 = x[1], x2 = x[2];
      out[3 * p] = a[0] * x0 + a[1] * x1 + a[2] * x2;
      out[3 * p + 1] = a[1] * x0 + a[3] * x1 + a[4] * x2;
      out[3 * p + 2] = a[2] * x0 + a[4] * x1 + a[5] * x2;
    } else {
      const T *a = P + 3 * p;
      const T *x = m + 2 * p;
      const T x0 = x[0], x1 = x[1];
      out[2 * p] = a[0] * x0 + a[2] * x1;
      out[2 * p + 1] = a[2] * x0 + a[1] * x1;
    }
  }
}

template <int MODE, typename T, bool TRIG>
int polmap2tod_t(void *dat, const void *map, const void *cs, const void *sn, const double *tg,
                 const int32_t *ipix, int64_t n, int64_t npix, int do_add, cudaStream_t st) {
  if (do_add) {
    auto k = k_polmap2tod<MODE, T, TRIG, true>;
    k<<<mk_grid_fit(k, n, 256), 256, 0, st>>>((T *)dat, (const T *)map, (const T *)cs, (const T *)sn, tg,
                                               ipix, n, npix);
  } else {
    auto k = k_polmap2tod<MODE, T, TRIG, false>;
    k<<<mk_grid_fit(k, n, 256), 256, 0, st>>>((T *)dat, (const T *)map, (const T *)cs, (const T *)sn, tg,
                                               ipix, n, npix);
  }
  return mk::launch_status("mk_polmap2tod");
}

template <int MODE, typename T, bool TRIG, bool ROWS>
int tod2polmap_t(void *map, const void *dat, const void *cs, const void *sn, const double *tg,
                 const int32_t *ipix, int64_t n, int64_t npix, const void *rowval, int64_t ndata,
                 cudaStream_t st) {
  auto k = k_tod2polmap<MODE, T, TRIG, ROWS>;
  k<<<mk_grid_fit(k, (n + 3) / 4, 256), 256, 0, st>>>((T *)map, (const T *)dat, (const T *)cs, (const T *)sn,
                                                       tg, ipix, n, npix, (const T *)rowval, ndata);
  return mk::launch_status("mk_tod2polmap");
}

template <typename T, bool TRIG, bool ROWS>
int tod2polmap_mode(int mode, void *map, const void *dat, const void *cs, const void *sn, const double *tg,
                    const int32_t *ipix, int64_t n, int64_t npix, const void *rowval, int64_t ndata,
                    cudaStream_t st) {
  switch (mode) {
    case MK_POL_QU:
      return tod2polmap_t<MK_POL_QU, T, TRIG, ROWS>(map, dat, cs, sn, tg, ipix, n, npix, rowval, ndata, st);
    case MK_POL_IQU:
      return tod2polmap_t<MK_POL_IQU, T, TRIG, ROWS>(map, dat, cs, sn, tg, ipix, n, npix, rowval, ndata, st);
    case MK_POL_QU_PRECON:
      return tod2polmap_t<MK_POL_QU_PRECON, T, TRIG, ROWS>(map, dat, cs, sn, tg, ipix, n, npix, rowval, ndata,
                                                           st);
    default:
      return tod2polmap_t<MK_POL_IQU_PRECON, T, TRIG, ROWS>(map, dat, cs, sn, tg, ipix, n, npix, rowval, ndata,
                                                            st);
  }
}

bool pol_mode_ok(int mode) {
  return mode == MK_POL_QU || mode == MK_POL_IQU || mode == MK_POL_QU_PRECON || mode == MK_POL_IQU_PRECON;
}

}  // namespace

extern "C" int mk_pol_npol(int mode) {
  switch (mode) {
    case MK_POL_QU: return 2;
    case MK_POL_IQU: return 3;
    case MK_POL_QU_PRECON: return 3;
    case MK_POL_IQU_PRECON: return 6;
    default: return 0;
  }
}

extern "C" int mk_pol_sincos(void *cs, void *sn, const double *twogamma, int64_t n, int dtype, void *stream) {
  MK_CHECK_ARG(n >= 0, "mk_pol_sincos: negative size");
  MK_CHECK_ARG(MK_DTYPE_OK(dtype), "mk_pol_sincos: bad dtype %d", dtype);
  if (n == 0) return MK_OK;
  MK_CHECK_ARG(cs && sn && twogamma, "mk_pol_sincos: null pointer");
  cudaStream_t st = mk::as_stream(stream);
  if (dtype == MK_F64)
    k_pol_sincos<double><<<mk_grid_fit(k_pol_sincos<double>, n, 256), 256, 0, st>>>((double *)cs, (double *)sn,
                                                                                   twogamma, n);
  else
    k_pol_sincos<float><<<mk_grid_fit(k_pol_sincos<float>, n, 256), 256, 0, st>>>((float *)cs, (float *)sn,
                                                                                 twogamma, n);
  return mk::launch_status("mk_pol_sincos");
}

extern "C" int mk_polmap2tod(void *dat, const void *map, const void *cos2g, const void *sin2g,
                             const double *twogamma, const int32_t *ipix, int64_t ndet, int64_t ndata,
                             int64_t npix, int mode, int dtype, int do_add, void *stream) {
  MK_CHECK_ARG(ndet >= 0 && ndata >= 0 && npix >= 0, "mk_polmap2tod: negative size");
  MK_CHECK_ARG(mode == MK_POL_QU || mode == MK_POL_IQU,
               "mk_polmap2tod: mode %d not implemented (QU and IQU only, as the reference)", mode);
  MK_CHECK_ARG(MK_DTYPE_OK(dtype), "mk_polmap2tod: bad dtype %d", dtype);
  const int64_t n = ndet * ndata;
  if (n == 0) return MK_OK;
  MK_CHECK_ARG(dat && map && ipix, "mk_polmap2tod: null pointer");
  const bool trig = (cos2g == nullptr);
  MK_CHECK_ARG(trig ? (twogamma != nullptr) : (sin2g != nullptr),
               "mk_polmap2tod: give cos2g and sin2g, or twogamma");
  MK_CHECK_ARG(!trig || dtype == MK_F64, "mk_polmap2tod: the twogamma form is FP64 only");
  cudaStream_t st = mk::as_stream(stream);
  if (trig)
    return mode == MK_POL_IQU
               ? polmap2tod_t<MK_POL_IQU, double, true>(dat, map, nullptr, nullptr, twogamma, ipix, n, npix, do_add, st)
               : polmap2tod_t<MK_POL_QU, double, true>(dat, map, nullptr, nullptr, twogamma, ipix, n, npix, do_add, st);
  if (dtype == MK_F64)
    return mode == MK_POL_IQU
               ? polmap2tod_t<MK_POL_IQU, double, false>(dat, map, cos2g, sin2g, nullptr, ipix, n, npix, do_add, st)
               : polmap2tod_t<MK_POL_QU, double, false>(dat, map, cos2g, sin2g, nullptr, ipix, n, npix, do_add, st);
  return mode == MK_POL_IQU
             ? polmap2tod_t<MK_POL_IQU, float, false>(dat, map, cos2g, sin2g, nullptr, ipix, n, npix, do_add, st)
             : polmap2tod_t<MK_POL_QU, float, false>(dat, map, cos2g, sin2g, nullptr, ipix, n, npix, do_add, st);
}

extern "C" int mk_tod2polmap(void *map, const void *dat, const void *cos2g, const void *sin2g,
                             const double *twogamma, const int32_t *ipix, int64_t ndet, int64_t ndata,
                             int64_t npix, int mode, int dtype, const void *rowval, void *stream) {
  MK_CHECK_ARG(ndet >= 0 && ndata >= 0 && npix >= 0, "mk_tod2polmap: negative size");
  MK_CHECK_ARG(pol_mode_ok(mode), "mk_tod2polmap: unknown mode %d", mode);
  MK_CHECK_ARG(MK_DTYPE_OK(dtype), "mk_tod2polmap: bad dtype %d", dtype);
  const int64_t n = ndet * ndata;
  if (n == 0) return MK_OK;
  MK_CHECK_ARG(map && ipix, "mk_tod2polmap: null pointer");
  const bool rows = (dat == nullptr);
  const bool trig = (cos2g == nullptr);
  MK_CHECK_ARG(trig ? (twogamma != nullptr) : (sin2g != nullptr),
               "mk_tod2polmap: give cos2g and sin2g, or twogamma");
  MK_CHECK_ARG(!trig || dtype == MK_F64, "mk_tod2polmap: the twogamma form is FP64 only");
  cudaStream_t st = mk::as_stream(stream);
  if (trig)
    return rows ? tod2polmap_mode<double, true, true>(mode, map, dat, nullptr, nullptr, twogamma, ipix, n, npix,
                                                      rowval, ndata, st)
                : tod2polmap_mode<double, true, false>(mode, map, dat, nullptr, nullptr, twogamma, ipix, n, npix,
                                                       rowval, ndata, st);
  if (dtype == MK_F64)
    return rows ? tod2polmap_mode<double, false, true>(mode, map, dat, cos2g, sin2g, nullptr, ipix, n, npix,
                                                       rowval, ndata, st)
                : tod2polmap_mode<double, false, false>(mode, map, dat, cos2g, sin2g, nullptr, ipix, n, npix,
                                                        rowval, ndata, st);
  return rows ? tod2polmap_mode<float, false, true>(mode, map, dat, cos2g, sin2g, nullptr, ipix, n, npix, rowval,
                                                    ndata, st)
              : tod2polmap_mode<float, false, false>(mode, map, dat, cos2g, sin2g, nullptr, ipix, n, npix, rowval,
                                                     ndata, st);
}

extern "C" int mk_pol_precon_mul(void *out, const void *precon, const void *map, int64_t npix, int mode,
                                 int dtype, void *stream) {
  MK_CHECK_ARG(npix >= 0, "mk_pol_precon_mul: negative size");
  MK_CHECK_ARG(mode == MK_POL_QU_PRECON || mode == MK_POL_IQU_PRECON,
               "mk_pol_precon_mul: mode must be QU_PRECON or IQU_PRECON");
  MK_CHECK_ARG(MK_DTYPE_OK(dtype), "mk_pol_precon_mul: bad dtype %d", dtype);
  if (npix == 0) return MK_OK;
  MK_CHECK_ARG(out && precon && map, "mk_pol_precon_mul: null pointer");
  cudaStream_t st = mk::as_stream(stream);
  const int iqu = mode == MK_POL_IQU_PRECON;
  if (dtype == MK_F64)
    k_pol_precon_mul<double><<<mk_grid_fit(k_pol_precon_mul<double>, npix, 256), 256, 0, st>>>(
        (double *)out, (const double *)precon, (const double *)map, npix, iqu);
  else
    k_pol_precon_mul<float><<<mk_grid_fit(k_pol_precon_mul<float>, npix, 256), 256, 0, st>>>(
        (float *)out, (const float *)precon, (const float *)map, npix, iqu);
  return mk::launch_status("mk_pol_precon_mul");
}
