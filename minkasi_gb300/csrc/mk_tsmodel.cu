// Projections of the per-TOD model members of a Mapset (besides sky maps):
//
//   cuts     vec[i] (+)= dat[imap[i]] / dat[imap[i]] (+)= vec[i]
//            tod2cuts / cuts2tod, minkasi/lib/minkasi.c:260-284 (CutsCompact,
//            minkasi/tods/cuts.py:351-417)
//   stripes  dat[d, t] (+)= pars[d, s(t)] / pars[d, s] (+)= sum_{t in s} dat[d, t]
//            map2tod_destriped / tod2map_destriped, minkasi/mapmaking/map2tod.py:156-190,
//            tod2map.py:242-269 (tsStripes, minkasi/mapmaking/timestream.py:486-531)
//   binned   dat[d, t] (+)= pars[d, b(t)] / pars[d, b] += sum_{b(t) = b} dat[d, t],
//            b(t) = int64((vec[t] - lo) * (nbin / (hi - lo)))
//            map2tod_binned_det / tod2map_binned_det, map2tod.py:195-253,
//            tod2map.py:272-340 (tsBinnedAz, timestream.py:533-560)
//
// All are HBM streams over the TOD with a small parameter array that stays in
// L1/L2.  The stripe sums use a fixed reduction tree (reproducible bits); the
// binned sums accumulate a per-CTA histogram in shared memory and add it to
// the parameters with one atomic per touched bin.
#include "mk_common.cuh"

namespace {

// ---- cuts --------------------------------------------------------------
template <typename T, bool ADD>
__global__ void __launch_bounds__(256) k_cuts_gather(T *__restrict__ vec, const T *__restrict__ dat,
                                                     const int64_t *__restrict__ imap, int64_t ncut,
                                                     int64_t ndat) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ncut; i += stride) {
    const int64_t j = imap[i];
    const T v = ((uint64_t)j < (uint64_t)ndat) ? dat[j] : T(0);
    vec[i] = ADD ? vec[i] + v : v;
  }
}

template <typename T, bool ADD>
__global__ void __launch_bounds__(256) k_cuts_scatter(T *__restrict__ dat, const T *__restrict__ vec,
                                                      const int64_t *__restrict__ imap, int64_t ncut,
                                                      int64_t ndat) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ncut; i += stride) {
    const int64_t j = imap[i];
    if ((uint64_t)j >= (uint64_t)ndat) continue;
    if (ADD)
      atomicAdd(dat + j, vec[i]);  // cut segments may overlap before merge_cuts
    else
      dat[j] = vec[i];
  }
}

// ---- stripes: one CTA per (segment, detector) ----------------------------
__device__ __forceinline__ void seg_bounds(const int64_t *__restrict__ lims, int64_t s, int64_t ndata,
                                           int64_t &a, int64_t &b) {
  a = lims[s];
  b = lims[s + 1];
  a = a < 0 ? 0 : (a > ndata ? ndata : a);
  b = b < a ? a : (b > ndata ? ndata : b);
}

template <typename T, bool ADD>
__global__ void __launch_bounds__(128) k_stripes_map2tod(T *__restrict__ dat, const T *__restrict__ pars,
                                                         const int64_t *__restrict__ lims, int64_t ndata,
                                                         int64_t nseg) {
  const int64_t s = blockIdx.x, d = blockIdx.y;
  int64_t a, b;
  seg_bounds(lims, s, ndata, a, b);
  const T p = pars[d * nseg + s];
  T *row = dat + d * ndata;
  for (int64_t t = a + threadIdx.x; t < b; t += blockDim.x) row[t] = ADD ? row[t] + p : p;
}

template <typename T>
__global__ void __launch_bounds__(128) k_stripes_tod2map(T *__restrict__ pars, const T *__restrict__ dat,
                                                         const int64_t *__restrict__ lims, int64_t ndata,
                                                         int64_t nseg, int do_add) {
  __shared__ T red[4];
  const int64_t s = blockIdx.x, d = blockIdx.y;
  int64_t a, b;
  seg_bounds(lims, s, ndata, a, b);
  const T *row = dat + d * ndata;
  T acc = T(0);
  for (int64_t t = a + threadIdx.x; t < b; t += blockDim.x) acc += row[t];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    const T sum = (red[0] + red[1]) + (red[2] + red[3]);
    T *p = pars + d * nseg + s;
    *p = do_add ? *p + sum : sum;
  }
}

// ---- binned: bin of sample t, exactly numpy's int64((vec - lo) * fac) ----
__device__ __forceinline__ int64_t bin_of(double x, double lo, double fac) {
  const double u = __dmul_rn(__dsub_rn(x, lo), fac);
  if (!(u > -9.2e18 && u < 9.2e18)) return -1;
  return __double2ll_rz(u);
}

template <typename T, bool ADD>
__global__ void __launch_bounds__(256) k_binned_map2tod(T *__restrict__ dat, const T *__restrict__ pars,
                                                        const double *__restrict__ vec, int64_t ndet,
                                                        int64_t ndata, int64_t nbin, double lo, double fac,
                                                        int vec_per_det) {
  const int64_t n = ndet * ndata;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int64_t d = i / ndata, t = i - d * ndata;
    const int64_t b = bin_of(vec[vec_per_det ? i : t], lo, fac);
    const T v = ((uint64_t)b < (uint64_t)nbin) ? pars[d * nbin + b] : T(0);
    dat[i] = ADD ? dat[i] + v : v;
  }
}

// grid (chunks, ndet); shared histogram of nbin entries when it fits
constexpr int BIN_CHUNK = 4096;

template <typename T, bool SMEM>
__global__ void __launch_bounds__(256) k_binned_tod2map(T *__restrict__ pars, const T *__restrict__ dat,
                                                        const double *__restrict__ vec, int64_t ndata,
                                                        int64_t nbin, double lo, double fac, int vec_per_det) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T *hist = reinterpret_cast<T *>(smraw);
  const int64_t d = blockIdx.y;
  const int64_t t0 = (int64_t)blockIdx.x * BIN_CHUNK;
  const int64_t t1 = t0 + BIN_CHUNK < ndata ? t0 + BIN_CHUNK : ndata;
  if (SMEM) {
    for (int64_t k = threadIdx.x; k < nbin; k += blockDim.x) hist[k] = T(0);
    __syncthreads();
  }
  const T *row = dat + d * ndata;
  const double *vrow = vec + (vec_per_det ? d * ndata : 0);
  T *prow = pars + d * nbin;
  for (int64_t t = t0 + threadIdx.x; t < t1; t += blockDim.x) {
    const int64_t b = bin_of(vrow[t], lo, fac);
    if ((uint64_t)b >= (uint64_t)nbin) continue;
    if (SMEM)
      atomicAdd(hist + b, row[t]);
    else
      atomicAdd(prow + b, row[t]);
  }
  if (SMEM) {
    __syncthreads();
    for (int64_t k = threadIdx.x; k < nbin; k += blockDim.x)
      if (hist[k] != T(0)) atomicAdd(prow + k, hist[k]);
  }
}

template <typename T>
int cuts_t(bool gather, void *out, const void *in, const int64_t *imap, int64_t ncut, int64_t ndat, int do_add,
           cudaStream_t st) {
  const unsigned g = mk_grid(ncut, 256, 8);
  if (gather) {
    if (do_add)
      k_cuts_gather<T, true><<<g, 256, 0, st>>>((T *)out, (const T *)in, imap, ncut, ndat);
    else
      k_cuts_gather<T, false><<<g, 256, 0, st>>>((T *)out, (const T *)in, imap, ncut, ndat);
  } else {
    if (do_add)
      k_cuts_scatter<T, true><<<g, 256, 0, st>>>((T *)out, (const T *)in, imap, ncut, ndat);
    else
      k_cuts_scatter<T, false><<<g, 256, 0, st>>>((T *)out, (const T *)in, imap, ncut, ndat);
  }
  return mk::launch_status(gather ? "mk_cuts_gather" : "mk_cuts_scatter");
}

template <typename T>
int binned_map2tod_t(void *dat, const void *pars, const double *vec, int64_t ndet, int64_t ndata, int64_t nbin,
                     double lo, double fac, int vec_per_det, int do_add, cudaStream_t st) {
  const unsigned g = mk_grid(ndet * ndata, 256, 8);
  if (do_add)
    k_binned_map2tod<T, true><<<g, 256, 0, st>>>((T *)dat, (const T *)pars, vec, ndet, ndata, nbin, lo, fac,
                                                  vec_per_det);
  else
    k_binned_map2tod<T, false><<<g, 256, 0, st>>>((T *)dat, (const T *)pars, vec, ndet, ndata, nbin, lo, fac,
                                                   vec_per_det);
  return mk::launch_status("mk_binned_map2tod");
}

template <typename T>
int binned_tod2map_t(void *pars, const void *dat, const double *vec, int64_t ndet, int64_t ndata, int64_t nbin,
                     double lo, double fac, int vec_per_det, cudaStream_t st) {
  const size_t smem = (size_t)nbin * sizeof(T);
  dim3 g((unsigned)((ndata + BIN_CHUNK - 1) / BIN_CHUNK), (unsigned)ndet);
  if (smem <= 48 * 1024)
    k_binned_tod2map<T, true><<<g, 256, smem, st>>>((T *)pars, (const T *)dat, vec, ndata, nbin, lo, fac,
                                                     vec_per_det);
  else
    k_binned_tod2map<T, false><<<g, 256, 0, st>>>((T *)pars, (const T *)dat, vec, ndata, nbin, lo, fac,
                                                   vec_per_det);
  return mk::launch_status("mk_binned_tod2map");
}

}  // namespace

extern "C" int mk_cuts_gather(void *vec, const void *dat, const int64_t *imap, int64_t ncut, int64_t ndat,
                              int dtype, int do_add, void *stream) {
  MK_CHECK_ARG(ncut >= 0 && ndat >= 0, "mk_cuts_gather: negative size");
  MK_CHECK_ARG(MK_DTYPE_OK(dtype), "mk_cuts_gather: bad dtype %d", dtype);
  if (ncut == 0) return MK_OK;
  MK_CHECK_ARG(vec && dat && imap, "mk_cuts_gather: null pointer");
  cudaStream_t st = mk::as_stream(stream);
  return dtype == MK_F64 ? cuts_t<double>(true, vec, dat, imap, ncut, ndat, do_add, st)
                         : cuts_t<float>(true, vec, dat, imap, ncut, ndat, do_add, st);
}

extern "C" int mk_cuts_scatter(void *dat, const void *vec, const int64_t *imap, int64_t ncut, int64_t ndat,
                               int dtype, int do_add, void *stream) {
  MK_CHECK_ARG(ncut >= 0 && ndat >= 0, "mk_cuts_scatter: negative size");
  MK_CHECK_ARG(MK_DTYPE_OK(dtype), "mk_cuts_scatter: bad dtype %d", dtype);
  if (ncut == 0) return MK_OK;
  MK_CHECK_ARG(vec && dat && imap, "mk_cuts_scatter: null pointer");
  cudaStream_t st = mk::as_stream(stream);
  return dtype == MK_F64 ? cuts_t<double>(false, dat, vec, imap, ncut, ndat, do_add, st)
                         : cuts_t<float>(false, dat, vec, imap, ncut, ndat, do_add, st);
}

extern "C" int mk_stripes_map2tod(void *dat, const void *pars, const int64_t *lims, int64_t ndet, int64_t ndata,
                                  int64_t nseg, int dtype, int do_add, void *stream) {
  MK_CHECK_ARG(ndet >= 0 && ndata >= 0 && nseg >= 0, "mk_stripes_map2tod: negative size");
  MK_CHECK_ARG(ndet <= 65535 && nseg <= 2147483647LL, "mk_stripes_map2tod: too many detectors or segments");
  MK_CHECK_ARG(MK_DTYPE_OK(dtype), "mk_stripes_map2tod: bad dtype %d", dtype);
  if (ndet == 0 || nseg == 0) return MK_OK;
  MK_CHECK_ARG(dat && pars && lims, "mk_stripes_map2tod: null pointer");
  cudaStream_t st = mk::as_stream(stream);
  dim3 g((unsigned)nseg, (unsigned)ndet);
  if (dtype == MK_F64) {
    if (do_add)
      k_stripes_map2tod<double, true><<<g, 128, 0, st>>>((double *)dat, (const double *)pars, lims, ndata, nseg);
    else
      k_stripes_map2tod<double, false><<<g, 128, 0, st>>>((double *)dat, (const double *)pars, lims, ndata, nseg);
  } else {
    if (do_add)
      k_stripes_map2tod<float, true><<<g, 128, 0, st>>>((float *)dat, (const float *)pars, lims, ndata, nseg);
    else
      k_stripes_map2tod<float, false><<<g, 128, 0, st>>>((float *)dat, (const float *)pars, lims, ndata, nseg);
  }
  return mk::launch_status("mk_stripes_map2tod");
}

extern "C" int mk_stripes_tod2map(void *pars, const void *dat, const int64_t *lims, int64_t ndet, int64_t ndata,
                                  int64_t nseg, int dtype, int do_add, void *stream) {
  MK_CHECK_ARG(ndet >= 0 && ndata >= 0 && nseg >= 0, "mk_stripes_tod2map: negative size");
  MK_CHECK_ARG(ndet <= 65535 && nseg <= 2147483647LL, "mk_stripes_tod2map: too many detectors or segments");
  MK_CHECK_ARG(MK_DTYPE_OK(dtype), "mk_stripes_tod2map: bad dtype %d", dtype);
  if (ndet == 0 || nseg == 0) return MK_OK;
  MK_CHECK_ARG(dat && pars && lims, "mk_stripes_tod2map: null pointer");
  cudaStream_t st = mk::as_stream(stream);
  dim3 g((unsigned)nseg, (unsigned)ndet);
  if (dtype == MK_F64)
    k_stripes_tod2map<double><<<g, 128, 0, st>>>((double *)pars, (const double *)dat, lims, ndata, nseg, do_add);
  else
    k_stripes_tod2map<float><<<g, 128, 0, st>>>((float *)pars, (const float *)dat, lims, ndata, nseg, do_add);
  return mk::launch_status("mk_stripes_tod2map");
}

extern "C" int mk_binned_map2tod(void *dat, const void *pars, const double *vec, int64_t ndet, int64_t ndata,
                                 int64_t nbin, double lo, double hi, int vec_per_det, int dtype, int do_add,
                                 void *stream) {
  MK_CHECK_ARG(ndet >= 0 && ndata >= 0 && nbin > 0, "mk_binned_map2tod: bad size");
  MK_CHECK_ARG(hi != lo, "mk_binned_map2tod: empty binning range");
  MK_CHECK_ARG(MK_DTYPE_OK(dtype), "mk_binned_map2tod: bad dtype %d", dtype);
  if (ndet * ndata == 0) return MK_OK;
  MK_CHECK_ARG(dat && pars && vec, "mk_binned_map2tod: null pointer");
  const double fac = (double)nbin / (hi - lo);  // numpy: nbin / (lims[1] - lims[0])
  cudaStream_t st = mk::as_stream(stream);
  return dtype == MK_F64
             ? binned_map2tod_t<double>(dat, pars, vec, ndet, ndata, nbin, lo, fac, vec_per_det, do_add, st)
             : binned_map2tod_t<float>(dat, pars, vec, ndet, ndata, nbin, lo, fac, vec_per_det, do_add, st);
}

extern "C" int mk_binned_tod2map(void *pars, const void *dat, const double *vec, int64_t ndet, int64_t ndata,
                                 int64_t nbin, double lo, double hi, int vec_per_det, int dtype, int do_add,
                                 void *stream) {
  MK_CHECK_ARG(ndet >= 0 && ndata >= 0 && nbin > 0, "mk_binned_tod2map: bad size");
  MK_CHECK_ARG(ndet <= 65535, "mk_binned_tod2map: too many detectors");
  MK_CHECK_ARG(hi != lo, "mk_binned_tod2map: empty binning range");
  MK_CHECK_ARG(MK_DTYPE_OK(dtype), "mk_binned_tod2map: bad dtype %d", dtype);
  if (ndet == 0) return MK_OK;
  MK_CHECK_ARG(pars, "mk_binned_tod2map: null pointer");
  cudaStream_t st = mk::as_stream(stream);
  const size_t es = dtype == MK_F64 ? 8 : 4;
  if (!do_add) MK_CUDA(cudaMemsetAsync(pars, 0, (size_t)(ndet * nbin) * es, st));
  if (ndata == 0) return MK_OK;
  MK_CHECK_ARG(dat && vec, "mk_binned_tod2map: null pointer");
  const double fac = (double)nbin / (hi - lo);
  return dtype == MK_F64 ? binned_tod2map_t<double>(pars, dat, vec, ndet, ndata, nbin, lo, fac, vec_per_det, st)
                         : binned_tod2map_t<float>(pars, dat, vec, ndet, ndata, nbin, lo, fac, vec_per_det, st);
}
