// Map-space vector algebra and the PCG recurrence of run_pcg_wprior
// (minkasi/mapmaking/pcg.py:101-178), with every scalar kept on the device.
//
// Reductions accumulate in FP64 whatever the map dtype, over a grid whose
// size depends only on n, then the last CTA to finish sums the per-CTA
// partials in a fixed order: results are bitwise reproducible run to run.
// Products and sums use explicit _rn intrinsics so the compiler does not fuse
// them into FMAs; x + alpha*p then rounds exactly as numpy's
// `x + a*p` (SkyMap.axpy, minkasi/maps/skymap.py:428-440).
#include "mk_common.cuh"

namespace {

constexpr int RB = 256;       // threads per reduction CTA
constexpr int RMAX = 1024;    // max reduction CTAs
constexpr int NSLOT = 2;      // simultaneous reductions per kernel

struct Scratch {
  double partial[NSLOT][RMAX];
  unsigned int counter;
};

inline unsigned red_grid(int64_t n) {
  int64_t g = (n + RB * 8 - 1) / (RB * 8);
  if (g < 1) g = 1;
  if (g > RMAX) g = RMAX;
  return (unsigned)g;
}

__device__ __forceinline__ double block_sum(double v, double *sh) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x < 32) {
    t = (lane < (RB / 32)) ? sh[lane] : 0.0;
    for (int off = 16; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
  }
  return t;  // valid in thread 0
}

// Writes this CTA's partials; returns true in the single last CTA, whose
// thread 0 then receives the totals in tot[] (fixed summation order).
template <int K>
__device__ bool finish_reduce(const double (&v)[K], Scratch *sc, double (&tot)[K]) {
  __shared__ double sh[RB / 32];
  __shared__ bool last;
#pragma unroll
  for (int k = 0; k < K; k++) {
    double s = block_sum(v[k], sh);
    if (threadIdx.x == 0) sc->partial[k][blockIdx.x] = s;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicAdd(&sc->counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!last) return false;
  __threadfence();
#pragma unroll
  for (int k = 0; k < K; k++) {
    double a = 0.0;
    for (unsigned b = threadIdx.x; b < gridDim.x; b += RB) a += ((volatile double *)sc->partial[k])[b];
    tot[k] = block_sum(a, sh);
  }
  if (threadIdx.x == 0) sc->counter = 0u;  // leave the scratch ready for the next call
  return true;
}

template <typename T>
__global__ void __launch_bounds__(RB) k_dot(const T *__restrict__ a, const T *__restrict__ b, int64_t n,
                                            double *result, Scratch *sc) {
  double acc[1] = {0.0};
  for (int64_t i = (int64_t)blockIdx.x * RB + threadIdx.x; i < n; i += (int64_t)gridDim.x * RB)
    acc[0] = __dadd_rn(acc[0], __dmul_rn((double)a[i], (double)b[i]));
  double tot[1];
  if (finish_reduce<1>(acc, sc, tot) && threadIdx.x == 0) *result = tot[0];
}

template <typename T>
__global__ void k_axpy(T *__restrict__ y, const T *__restrict__ x, double alpha, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = (T)__dadd_rn((double)y[i], __dmul_rn(alpha, (double)x[i]));
}

template <typename T>
__global__ void k_mul(T *__restrict__ out, const T *__restrict__ a, const T *__restrict__ b, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = a[i] * b[i];
}

__device__ __forceinline__ bool finite(double x) { return isfinite(x); }

// r = b - Ax; z = M r; p = z; zr = r.z; rr = r.r   (pcg.py:101-121)
template <typename T>
__global__ void __launch_bounds__(RB) k_pcg_init(T *__restrict__ r, T *__restrict__ z, T *__restrict__ p,
                                                 const T *__restrict__ b, const T *__restrict__ Ax,
                                                 const T *__restrict__ M, int64_t n, double *s,
                                                 Scratch *sc) {
  double acc[2] = {0.0, 0.0};
  for (int64_t i = (int64_t)blockIdx.x * RB + threadIdx.x; i < n; i += (int64_t)gridDim.x * RB) {
    T ri = b[i] - Ax[i];
    T zi = M ? M[i] * ri : ri;
    r[i] = ri;
    z[i] = zi;
    p[i] = zi;
    acc[0] = __dadd_rn(acc[0], __dmul_rn((double)ri, (double)zi));
    acc[1] = __dadd_rn(acc[1], __dmul_rn((double)ri, (double)ri));
  }
  double tot[2];
  if (finish_reduce<2>(acc, sc, tot) && threadIdx.x == 0) {
    s[MK_S_ZR] = tot[0];
    s[MK_S_RR] = tot[1];
    s[MK_S_FLAG] = finite(tot[0]) ? 0.0 : 1.0;
    s[MK_S_ITER] = 0.0;
  }
}

// pAp = p.Ap; alpha = zr/pAp   (pcg.py:137-141)
template <typename T>
__global__ void __launch_bounds__(RB) k_pcg_pap(const T *__restrict__ p, const T *__restrict__ Ap,
                                                int64_t n, double *s, Scratch *sc) {
  double acc[1] = {0.0};
  for (int64_t i = (int64_t)blockIdx.x * RB + threadIdx.x; i < n; i += (int64_t)gridDim.x * RB)
    acc[0] = __dadd_rn(acc[0], __dmul_rn((double)p[i], (double)Ap[i]));
  double tot[1];
  if (finish_reduce<1>(acc, sc, tot) && threadIdx.x == 0) {
    double pap = tot[0];
    s[MK_S_PAP] = pap;
    double alpha = s[MK_S_ZR] / pap;
    s[MK_S_ALPHA] = alpha;
    if (!(pap > 0.0) || !finite(alpha)) s[MK_S_FLAG] = 1.0;
  }
}

// x += alpha p; r += (-alpha) Ap; z = M r; zr' = r.z; rr = r.r;
// beta = zr'/zr   (pcg.py:143-164)
template <typename T>
__global__ void __launch_bounds__(RB) k_pcg_xrz(T *__restrict__ x, T *__restrict__ r, T *__restrict__ z,
                                                const T *__restrict__ p, const T *__restrict__ Ap,
                                                const T *__restrict__ M, int64_t n, double *s,
                                                Scratch *sc) {
  const bool stop = s[MK_S_FLAG] != 0.0;
  const double alpha = s[MK_S_ALPHA];
  double acc[2] = {0.0, 0.0};
  if (!stop) {
    for (int64_t i = (int64_t)blockIdx.x * RB + threadIdx.x; i < n; i += (int64_t)gridDim.x * RB) {
      x[i] = (T)__dadd_rn((double)x[i], __dmul_rn(alpha, (double)p[i]));
      T ri = (T)__dadd_rn((double)r[i], __dmul_rn(-alpha, (double)Ap[i]));
      T zi = M ? M[i] * ri : ri;
      r[i] = ri;
      z[i] = zi;
      acc[0] = __dadd_rn(acc[0], __dmul_rn((double)ri, (double)zi));
      acc[1] = __dadd_rn(acc[1], __dmul_rn((double)ri, (double)ri));
    }
  }
  double tot[2];
  if (finish_reduce<2>(acc, sc, tot) && threadIdx.x == 0 && !stop) {
    double zr_new = tot[0];
    double beta = zr_new / s[MK_S_ZR];
    s[MK_S_ZRNEW] = zr_new;
    s[MK_S_BETA] = beta;
    s[MK_S_ZR] = zr_new;
    s[MK_S_RR] = tot[1];
    s[MK_S_ITER] += 1.0;
    if (!finite(beta)) s[MK_S_FLAG] = 1.0;
  }
}

// p = z + beta p   (pcg.py:166-171)
template <typename T>
__global__ void k_pcg_p(T *__restrict__ p, const T *__restrict__ z, int64_t n, const double *s) {
  if (s[MK_S_FLAG] != 0.0) return;
  const double beta = s[MK_S_BETA];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] = (T)__dadd_rn((double)z[i], __dmul_rn(beta, (double)p[i]));
}

// Split update for an operator preconditioner z = M(r) computed between the
// two halves:  (1) x += alpha p; r += (-alpha) Ap; rr = r.r
template <typename T>
__global__ void __launch_bounds__(RB) k_pcg_xr(T *__restrict__ x, T *__restrict__ r, const T *__restrict__ p,
                                               const T *__restrict__ Ap, int64_t n, double *s, Scratch *sc) {
  const bool stop = s[MK_S_FLAG] != 0.0;
  const double alpha = s[MK_S_ALPHA];
  double acc[1] = {0.0};
  if (!stop) {
    for (int64_t i = (int64_t)blockIdx.x * RB + threadIdx.x; i < n; i += (int64_t)gridDim.x * RB) {
      x[i] = (T)__dadd_rn((double)x[i], __dmul_rn(alpha, (double)p[i]));
      T ri = (T)__dadd_rn((double)r[i], __dmul_rn(-alpha, (double)Ap[i]));
      r[i] = ri;
      acc[0] = __dadd_rn(acc[0], __dmul_rn((double)ri, (double)ri));
    }
  }
  double tot[1];
  if (finish_reduce<1>(acc, sc, tot) && threadIdx.x == 0 && !stop) s[MK_S_RR] = tot[0];
}

// (2) zr' = r.z; beta = zr'/zr; zr = zr'; iteration count += 1
template <typename T>
__global__ void __launch_bounds__(RB) k_pcg_zr(const T *__restrict__ r, const T *__restrict__ z, int64_t n,
                                               double *s, Scratch *sc) {
  const bool stop = s[MK_S_FLAG] != 0.0;
  double acc[1] = {0.0};
  if (!stop)
    for (int64_t i = (int64_t)blockIdx.x * RB + threadIdx.x; i < n; i += (int64_t)gridDim.x * RB)
      acc[0] = __dadd_rn(acc[0], __dmul_rn((double)r[i], (double)z[i]));
  double tot[1];
  if (finish_reduce<1>(acc, sc, tot) && threadIdx.x == 0 && !stop) {
    double beta = tot[0] / s[MK_S_ZR];
    s[MK_S_ZRNEW] = tot[0];
    s[MK_S_BETA] = beta;
    s[MK_S_ZR] = tot[0];
    s[MK_S_ITER] += 1.0;
    if (!finite(beta) || !(tot[0] > 0.0)) s[MK_S_FLAG] = 1.0;
  }
}

// out = d * (a + b)
template <typename T>
__global__ void k_scale_add(T *__restrict__ out, const T *__restrict__ d, const T *__restrict__ a,
                            const T *__restrict__ b, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = d[i] * (a[i] + (b ? b[i] : T(0)));
}

template <typename T>
int pcg_update_t(T *x, T *r, T *z, T *p, const T *Ap, const T *M, int64_t n, double *s,
                 Scratch *sc, cudaStream_t st) {
  unsigned g = red_grid(n);
  k_pcg_pap<T><<<g, RB, 0, st>>>(p, Ap, n, s, sc);
  k_pcg_xrz<T><<<g, RB, 0, st>>>(x, r, z, p, Ap, M, n, s, sc);
  k_pcg_p<T><<<mk_grid_fit(k_pcg_p<T>, n, 256), 256, 0, st>>>(p, z, n, s);
  return mk::launch_status("mk_pcg_update");
}

}  // namespace

extern "C" size_t mk_reduce_scratch_bytes(void) { return sizeof(Scratch); }

extern "C" int mk_dot(const void *a, const void *b, int64_t n, int dtype, double *result,
                      void *scratch, void *stream) {
  MK_CHECK_ARG(MK_DTYPE_OK(dtype), "mk_dot: bad dtype %d", dtype);
  MK_CHECK_ARG(n >= 0 && result && scratch, "mk_dot: bad argument");
  MK_CHECK_ARG(n == 0 || (a && b), "mk_dot: null input");
  cudaStream_t st = mk::as_stream(stream);
  unsigned g = red_grid(n);
  if (dtype == MK_F64)
    k_dot<double><<<g, RB, 0, st>>>((const double *)a, (const double *)b, n, result, (Scratch *)scratch);
  else
    k_dot<float><<<g, RB, 0, st>>>((const float *)a, (const float *)b, n, result, (Scratch *)scratch);
  return mk::launch_status("mk_dot");
}

extern "C" int mk_axpy(void *y, const void *x, double alpha, int64_t n, int dtype, void *stream) {
  MK_CHECK_ARG(MK_DTYPE_OK(dtype), "mk_axpy: bad dtype %d", dtype);
  if (n <= 0) return MK_OK;
  MK_CHECK_ARG(x && y, "mk_axpy: null pointer");
  cudaStream_t st = mk::as_stream(stream);
  if (dtype == MK_F64)
    k_axpy<double><<<mk_grid_fit(k_axpy<double>, n, 256), 256, 0, st>>>((double *)y, (const double *)x, alpha, n);
  else
    k_axpy<float><<<mk_grid_fit(k_axpy<float>, n, 256), 256, 0, st>>>((float *)y, (const float *)x, alpha, n);
  return mk::launch_status("mk_axpy");
}

extern "C" int mk_mul(void *out, const void *a, const void *b, int64_t n, int dtype, void *stream) {
  MK_CHECK_ARG(MK_DTYPE_OK(dtype), "mk_mul: bad dtype %d", dtype);
  if (n <= 0) return MK_OK;
  MK_CHECK_ARG(out && a && b, "mk_mul: null pointer");
  cudaStream_t st = mk::as_stream(stream);
  if (dtype == MK_F64)
    k_mul<double><<<mk_grid_fit(k_mul<double>, n, 256), 256, 0, st>>>((double *)out, (const double *)a,
                                                      (const double *)b, n);
  else
    k_mul<float><<<mk_grid_fit(k_mul<float>, n, 256), 256, 0, st>>>((float *)out, (const float *)a, (const float *)b, n);
  return mk::launch_status("mk_mul");
}

extern "C" int mk_pcg_init(void *r, void *z, void *p, const void *b, const void *Ax,
                           const void *precon, int64_t n, int dtype, double *s, void *scratch,
                           void *stream) {
  MK_CHECK_ARG(MK_DTYPE_OK(dtype), "mk_pcg_init: bad dtype %d", dtype);
  MK_CHECK_ARG(n >= 1 && r && z && p && b && Ax && s && scratch, "mk_pcg_init: bad argument");
  cudaStream_t st = mk::as_stream(stream);
  unsigned g = red_grid(n);
  if (dtype == MK_F64)
    k_pcg_init<double><<<g, RB, 0, st>>>((double *)r, (double *)z, (double *)p, (const double *)b,
                                         (const double *)Ax, (const double *)precon, n, s,
                                         (Scratch *)scratch);
  else
    k_pcg_init<float><<<g, RB, 0, st>>>((float *)r, (float *)z, (float *)p, (const float *)b,
                                        (const float *)Ax, (const float *)precon, n, s,
                                        (Scratch *)scratch);
  return mk::launch_status("mk_pcg_init");
}

extern "C" int mk_pcg_update(void *x, void *r, void *z, void *p, const void *Ap, const void *precon,
                             int64_t n, int dtype, double *s, void *scratch, void *stream) {
  MK_CHECK_ARG(MK_DTYPE_OK(dtype), "mk_pcg_update: bad dtype %d", dtype);
  MK_CHECK_ARG(n >= 1 && x && r && z && p && Ap && s && scratch, "mk_pcg_update: bad argument");
  cudaStream_t st = mk::as_stream(stream);
  if (dtype == MK_F64)
    return pcg_update_t<double>((double *)x, (double *)r, (double *)z, (double *)p,
                                (const double *)Ap, (const double *)precon, n, s,
                                (Scratch *)scratch, st);
  return pcg_update_t<float>((float *)x, (float *)r, (float *)z, (float *)p, (const float *)Ap,
                             (const float *)precon, n, s, (Scratch *)scratch, st);
}

extern "C" int mk_pcg_step_xr(void *x, void *r, const void *p, const void *Ap, int64_t n, int dtype,
                              double *s, void *scratch, void *stream) {
  MK_CHECK_ARG(MK_DTYPE_OK(dtype), "mk_pcg_step_xr: bad dtype %d", dtype);
  MK_CHECK_ARG(n >= 1 && x && r && p && Ap && s && scratch, "mk_pcg_step_xr: bad argument");
  cudaStream_t st = mk::as_stream(stream);
  unsigned g = red_grid(n);
  if (dtype == MK_F64) {
    k_pcg_pap<double><<<g, RB, 0, st>>>((const double *)p, (const double *)Ap, n, s, (Scratch *)scratch);
    k_pcg_xr<double><<<g, RB, 0, st>>>((double *)x, (double *)r, (const double *)p, (const double *)Ap, n,
                                       s, (Scratch *)scratch);
  } else {
    k_pcg_pap<float><<<g, RB, 0, st>>>((const float *)p, (const float *)Ap, n, s, (Scratch *)scratch);
    k_pcg_xr<float><<<g, RB, 0, st>>>((float *)x, (float *)r, (const float *)p, (const float *)Ap, n, s,
                                      (Scratch *)scratch);
  }
  return mk::launch_status("mk_pcg_step_xr");
}

extern "C" int mk_pcg_step_zp(const void *z, const void *r, void *p, int64_t n, int dtype, double *s,
                              void *scratch, void *stream) {
  MK_CHECK_ARG(MK_DTYPE_OK(dtype), "mk_pcg_step_zp: bad dtype %d", dtype);
  MK_CHECK_ARG(n >= 1 && z && r && p && s && scratch, "mk_pcg_step_zp: bad argument");
  cudaStream_t st = mk::as_stream(stream);
  unsigned g = red_grid(n);
  if (dtype == MK_F64) {
    k_pcg_zr<double><<<g, RB, 0, st>>>((const double *)r, (const double *)z, n, s, (Scratch *)scratch);
    k_pcg_p<double><<<mk_grid_fit(k_pcg_p<double>, n, 256), 256, 0, st>>>((double *)p, (const double *)z, n, s);
  } else {
    k_pcg_zr<float><<<g, RB, 0, st>>>((const float *)r, (const float *)z, n, s, (Scratch *)scratch);
    k_pcg_p<float><<<mk_grid_fit(k_pcg_p<float>, n, 256), 256, 0, st>>>((float *)p, (const float *)z, n, s);
  }
  return mk::launch_status("mk_pcg_step_zp");
}

extern "C" int mk_scale_add(void *out, const void *d, const void *a, const void *b, int64_t n, int dtype,
                            void *stream) {
  MK_CHECK_ARG(MK_DTYPE_OK(dtype), "mk_scale_add: bad dtype %d", dtype);
  if (n <= 0) return MK_OK;
  MK_CHECK_ARG(out && d && a, "mk_scale_add: null pointer");
  cudaStream_t st = mk::as_stream(stream);
  if (dtype == MK_F64)
    k_scale_add<double><<<mk_grid_fit(k_scale_add<double>, n, 256), 256, 0, st>>>((double *)out, (const double *)d,
                                                            (const double *)a, (const double *)b, n);
  else
    k_scale_add<float><<<mk_grid_fit(k_scale_add<float>, n, 256), 256, 0, st>>>((float *)out, (const float *)d,
                                                           (const float *)a, (const float *)b, n);
  return mk::launch_status("mk_scale_add");
}
