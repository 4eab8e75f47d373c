// DCT-I (FFTW REDFT00) and the NoiseSmoothedSVD filter on the GPU.
//
// DCT-I of a row x of length n equals the real part of the DFT of its even
// extension y (length N = 2(n-1)):  y_j = x_j (0 <= j < n),
// y_{N-j} = x_j (1 <= j <= n-2);  X_k = Re Y_k, k = 0..n-1.
// So every DCT here is: hand-written extension kernel -> batched cuFFT
// real-to-complex transform of length N -> hand-written kernel that takes the
// real part and applies whatever comes next (the inverse-spectrum weights
// and the next extension, or the endpoint halving).
//
// apply_noise (minkasi/mapmaking/noise.py:680-714) for one TOD:
//   E[:, :n]  = v . dat                         (GEMM, written with ld N)
//   E[:, n:]  = mirror                          (k_mirror)
//   F         = R2C(E)                          (cuFFT)
//   E         = extend(Re F * mywt)             (k_filter_extend)
//   F         = R2C(E)                          (cuFFT)
//   G         = Re F, columns 0 and n-1 halved  (k_real_halve; G aliases E)
//   out       = vT . G                          (GEMM)
// Halving before the second rotation equals halving after it (a column
// scale commutes with a left multiplication).  With the tensor-core rotation
// (rot_mode 2) the mirror is written by the first rotation's epilogue and the
// second rotation reads Re F in place and halves while splitting, so k_mirror
// and k_real_halve do not run.
//
// By default plans use the four-step shared-memory FFT of mk_fft4.cu /
// mk_fft4_f64.cu instead of cuFFT, in the plan's precision (directly when
// 2(n-1) factors into 2, 3, 5, 7, 11; through Bluestein's algorithm
// otherwise, up to its length limit):
//   E = v . dat;  E = DCT(E) * mywt;  E = DCT(E) with columns 0 and n-1
//   halved;  out = vT . E.
// Each DCT is two kernels (three with Bluestein) that form the even
// extension while loading and apply the weights or the halving while
// storing, two detector rows per complex transform.
#include <cublas_v2.h>
#include <cufft.h>

#include <atomic>
#include <mutex>
#include <new>
#include <vector>

#include "mk_common.cuh"
#include "mk_fft4.cuh"
#include "mk_ozaki.cuh"
#include "mk_rot.cuh"

namespace {

constexpr size_t ALIGN = 256;
inline size_t align_up(size_t x) { return (x + ALIGN - 1) / ALIGN * ALIGN; }

const char *cufft_str(cufftResult r) {
  switch (r) {
    case CUFFT_SUCCESS: return "CUFFT_SUCCESS";
    case CUFFT_INVALID_PLAN: return "CUFFT_INVALID_PLAN";
    case CUFFT_ALLOC_FAILED: return "CUFFT_ALLOC_FAILED";
    case CUFFT_INVALID_VALUE: return "CUFFT_INVALID_VALUE";
    case CUFFT_INTERNAL_ERROR: return "CUFFT_INTERNAL_ERROR";
    case CUFFT_EXEC_FAILED: return "CUFFT_EXEC_FAILED";
    case CUFFT_SETUP_FAILED: return "CUFFT_SETUP_FAILED";
    case CUFFT_INVALID_SIZE: return "CUFFT_INVALID_SIZE";
    default: return "cuFFT error";
  }
}

#define MK_CUFFT(call)                                                              \
  do {                                                                              \
    cufftResult _r = (call);                                                        \
    if (_r != CUFFT_SUCCESS) {                                                      \
      mk::set_error("%s failed: %s (%d)", #call, cufft_str(_r), (int)_r);          \
      return MK_ERR_CUFFT;                                                          \
    }                                                                               \
  } while (0)

// ---- elementwise kernels (grid: x over columns, y over rows) --------------
template <typename T>
__global__ void k_extend(const T *__restrict__ in, int64_t ld_in, T *__restrict__ E, int64_t n,
                         int64_t N, int64_t nrow) {
  for (int64_t r = blockIdx.y; r < nrow; r += gridDim.y) {
    const T *src = in + r * ld_in;
    T *dst = E + r * N;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n;
         j += (int64_t)gridDim.x * blockDim.x) {
      T v = src[j];
      dst[j] = v;
      if (j >= 1 && j <= n - 2) dst[N - j] = v;
    }
  }
}

template <typename T>
__global__ void k_mirror(T *__restrict__ E, int64_t n, int64_t N, int64_t nrow) {
  for (int64_t r = blockIdx.y; r < nrow; r += gridDim.y) {
    T *row = E + r * N;
    for (int64_t j = 1 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j <= n - 2;
         j += (int64_t)gridDim.x * blockDim.x)
      row[N - j] = row[j];
  }
}

template <typename T, typename C>
__global__ void k_real(const C *__restrict__ F, T *__restrict__ out, int64_t n, int64_t nrow) {
  for (int64_t r = blockIdx.y; r < nrow; r += gridDim.y)
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x)
      out[r * n + k] = F[r * n + k].x;
}

template <typename T, typename C>
__global__ void k_filter_extend(const C *__restrict__ F, const T *__restrict__ w, int64_t ldw,
                                T *__restrict__ E, int64_t n, int64_t N, int64_t nrow) {
  for (int64_t r = blockIdx.y; r < nrow; r += gridDim.y) {
    const C *f = F + r * n;
    const T *wr = w + r * ldw;
    T *dst = E + r * N;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
      T v = f[k].x * __ldcs(wr + k);
      dst[k] = v;
      if (k >= 1 && k <= n - 2) dst[N - k] = v;
    }
  }
}

template <typename T, typename C>
__global__ void k_real_halve(const C *__restrict__ F, T *__restrict__ G, int64_t n, int64_t nrow) {
  for (int64_t r = blockIdx.y; r < nrow; r += gridDim.y)
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
      T v = F[r * n + k].x;
      if (k == 0 || k == n - 1) v *= T(0.5);
      G[r * n + k] = v;
    }
}

dim3 rows_grid(int64_t n, int64_t nrow) {
  // enough CTAs along the row to fill the GPU several times over
  int64_t total = (int64_t)mk::sm_count() * 16;
  int64_t gy = nrow < 65535 ? nrow : 65535;
  int64_t gx = (total + gy - 1) / gy;
  int64_t need = (n + 255) / 256;
  if (gx > need) gx = need;
  if (gx < 1) gx = 1;
  return dim3((unsigned)gx, (unsigned)gy, 1);
}

// ---- plan object -----------------------------------------------------------
// 0: four-step FFT (Bluestein on it for lengths with a prime factor above
// 11), cuFFT beyond its limits; 1: cuFFT; 2: four-step for smooth lengths only
std::atomic<int> g_engine{0};

struct DctCore {
  cufftHandle fft = 0;
  bool have_fft = false;
  bool own = false;  // four-step FFT of this library (FP32 or FP64 tables and kernels)
  mk::Fft4Plan f4;
  void *T = nullptr;  // its scratch (complex, in the plan's precision)
  int64_t nrow = 0, n = 0, N = 0;
  int dtype = MK_F64;
  void *E = nullptr, *F = nullptr, *work = nullptr;
  size_t work_bytes = 0;
  // tensor-core rotation (FP32 plans): status word (plan-owned), operand
  // image (workspace: rebuilt by every rotation)
  int *tc_err = nullptr;
  void *tc_bimg = nullptr;
  // sliced FP64 rotation on the bf16 tensor cores (FP64 plans): its scratch
  // in the workspace
  void *oz_ws = nullptr;
  size_t oz_bytes = 0;
  // device memory the plan owns: the status word, then the four-step tables.
  // Never in the workspace, which plans of different shapes may share.
  void *owned = nullptr;
};

// workspace bytes of the tensor-core rotation's operand image (FP32) or of
// the sliced FP64 rotation's scratch (FP64)
size_t tc_bytes(int64_t nrow, int dtype) {
  if (dtype == MK_F64) return mk::ozaki_supported(nrow) ? align_up(mk::ozaki_ws_bytes(nrow)) : 0;
  if (!mk::rot_tc_supported(nrow)) return 0;
  return align_up(mk::rot_tc_bimg_bytes(nrow));
}

void core_free(DctCore *c) {
  if (c->have_fft) cufftDestroy(c->fft);
  c->have_fft = false;
  if (c->owned) cudaFree(c->owned);
  c->owned = nullptr;
}

// plan-owned device memory: 256 B (status word) + `extra`
int own_alloc(DctCore *c, size_t extra) {
  MK_CUDA(cudaMalloc(&c->owned, 256 + extra));
  MK_CUDA(cudaMemset(c->owned, 0, 256));
  c->tc_err = (int *)c->owned;
  return MK_OK;
}

size_t elt(int dtype) { return dtype == MK_F64 ? 8 : 4; }

int make_fft(cufftHandle *h, int64_t nrow, int64_t N, int dtype, size_t *work) {
  MK_CUFFT(cufftCreate(h));
  cufftResult r = cufftSetAutoAllocation(*h, 0);
  long long nn[1] = {(long long)N};
  long long inembed[1] = {(long long)N};
  long long onembed[1] = {(long long)(N / 2 + 1)};
  if (r == CUFFT_SUCCESS)
    r = cufftMakePlanMany64(*h, 1, nn, inembed, 1, (long long)N, onembed, 1, (long long)(N / 2 + 1),
                            dtype == MK_F64 ? CUFFT_D2Z : CUFFT_R2C, (long long)nrow, work);
  if (r != CUFFT_SUCCESS) {
    cufftDestroy(*h);
    mk::set_error("cufftMakePlanMany64(N=%lld, batch=%lld) failed: %s", (long long)N,
                  (long long)nrow, cufft_str(r));
    return MK_ERR_CUFFT;
  }
  return MK_OK;
}

bool use_own(int64_t nrow, int64_t n, int dtype, mk::Fft4Dev *d, bool *blue_ok) {
  const int e = g_engine.load();
  *blue_ok = e == 0;
  return e != 1 && (nrow + 1) / 2 <= 65535 && mk::fft4_shape(n, d, *blue_ok, dtype == MK_F64);
}

// rot: the plan rotates too (noise plans): reserve the rotation scratch
int core_bytes(int64_t nrow, int64_t n, int dtype, size_t *bytes, bool rot = true) {
  MK_CHECK_ARG(bytes, "workspace size: null output");
  MK_CHECK_ARG(MK_DTYPE_OK(dtype), "workspace size: bad dtype %d", dtype);
  MK_CHECK_ARG(nrow >= 1 && n >= 2, "DCT-I needs nrow >= 1 and n >= 2 (got %lld, %lld)",
               (long long)nrow, (long long)n);
  mk::Fft4Dev d;
  bool blue_ok;
  if (use_own(nrow, n, dtype, &d, &blue_ok)) {
    *bytes = align_up((size_t)nrow * n * elt(dtype)) + align_up(mk::fft4_t_bytes(d, nrow)) +
             (rot ? tc_bytes(nrow, dtype) : 0);
    return MK_OK;
  }
  int64_t N = 2 * (n - 1);
  cufftHandle h;
  size_t work = 0;
  int rc = make_fft(&h, nrow, N, dtype, &work);
  if (rc) return rc;
  cufftDestroy(h);
  *bytes = align_up((size_t)nrow * N * elt(dtype)) + align_up((size_t)nrow * n * 2 * elt(dtype)) +
           align_up(work) + (rot ? tc_bytes(nrow, dtype) : 0);
  return MK_OK;
}

int core_create(DctCore *c, int64_t nrow, int64_t n, int dtype, void *ws, size_t ws_bytes, bool rot = true) {
  size_t need = 0;
  int rc = core_bytes(nrow, n, dtype, &need, rot);
  if (rc) return rc;
  MK_CHECK_ARG(ws && ((uintptr_t)ws % ALIGN) == 0, "workspace must be a 256-byte aligned device pointer");
  MK_CHECK_ARG(ws_bytes >= need, "workspace too small: %zu < %zu bytes", ws_bytes, need);
  c->nrow = nrow;
  c->n = n;
  c->N = 2 * (n - 1);
  c->dtype = dtype;
  char *p = (char *)ws;
  mk::Fft4Dev d;
  bool blue_ok;
  if (use_own(nrow, n, dtype, &d, &blue_ok)) {
    c->own = true;
    c->E = p;
    p += align_up((size_t)nrow * n * elt(dtype));
    c->T = p;
    p += align_up(mk::fft4_t_bytes(d, nrow));
    if ((rot ? tc_bytes(nrow, dtype) : 0)) {
      if (dtype == MK_F64) {
        c->oz_ws = p;
        c->oz_bytes = tc_bytes(nrow, dtype);
      } else {
        c->tc_bimg = p;
      }
    }
    if ((rc = own_alloc(c, mk::fft4_table_bytes(d))) ||
        (rc = mk::fft4_init(&c->f4, n, (char *)c->owned + 256, blue_ok, dtype == MK_F64))) {
      core_free(c);
      return rc;
    }
    return MK_OK;
  }
  c->E = p;
  p += align_up((size_t)nrow * c->N * elt(dtype));
  c->F = p;
  p += align_up((size_t)nrow * n * 2 * elt(dtype));
  c->work = p;
  rc = make_fft(&c->fft, nrow, c->N, dtype, &c->work_bytes);
  if (rc) return rc;
  c->have_fft = true;
  if ((rot ? tc_bytes(nrow, dtype) : 0)) {
    if (dtype == MK_F64) {
      c->oz_ws = (char *)c->work + align_up(c->work_bytes);
      c->oz_bytes = (rot ? tc_bytes(nrow, dtype) : 0);
    } else {
      c->tc_bimg = (char *)c->work + align_up(c->work_bytes);
    }
    if ((rc = own_alloc(c, 0))) {
      core_free(c);
      return rc;
    }
  }
  cufftResult r = cufftSetWorkArea(c->fft, c->work);
  if (r != CUFFT_SUCCESS) {
    core_free(c);
    mk::set_error("cufftSetWorkArea failed: %s", cufft_str(r));
    return MK_ERR_CUFFT;
  }
  return MK_OK;
}

int core_fft(DctCore *c, cudaStream_t st) {
  MK_CUFFT(cufftSetStream(c->fft, st));
  if (c->dtype == MK_F64)
    MK_CUFFT(cufftExecD2Z(c->fft, (cufftDoubleReal *)c->E, (cufftDoubleComplex *)c->F));
  else
    MK_CUFFT(cufftExecR2C(c->fft, (cufftReal *)c->E, (cufftComplex *)c->F));
  return MK_OK;
}

// one four-step DCT-I of the plan's rows (ld n), in the plan's precision
int own_dct(DctCore *c, const void *in, void *out, int epi, const void *w, int64_t ldw, cudaStream_t st) {
  if (c->dtype == MK_F64)
    return mk::fft4_dct_f64(c->f4, (const double *)in, c->n, c->nrow, (double2 *)c->T, (double *)out, c->n, epi,
                            (const double *)w, ldw, st);
  return mk::fft4_dct(c->f4, (const float *)in, c->n, c->nrow, (float2 *)c->T, (float *)out, c->n, epi,
                      (const float *)w, ldw, st);
}

template <typename T, typename C>
int dct_exec_t(DctCore *c, const void *in, void *out, cudaStream_t st) {
  if (c->own) return own_dct(c, in, out, mk::FFT4_PLAIN, nullptr, 0, st);
  dim3 g = rows_grid(c->n, c->nrow);
  k_extend<T><<<g, 256, 0, st>>>((const T *)in, c->n, (T *)c->E, c->n, c->N, c->nrow);
  int rc = mk::launch_status("mk_dct1_exec/extend");
  if (rc) return rc;
  if ((rc = core_fft(c, st))) return rc;
  k_real<T, C><<<g, 256, 0, st>>>((const C *)c->F, (T *)out, c->n, c->nrow);
  return mk::launch_status("mk_dct1_exec/real");
}

// ---- cuBLAS handle (one per device, shared; calls serialised) -------------
std::mutex g_blas_mu;
cublasHandle_t g_blas[64] = {};
void *g_blas_ws[64] = {};

int blas_handle(cublasHandle_t *out) {
  int dev = 0;
  MK_CUDA(cudaGetDevice(&dev));
  MK_CHECK_ARG(dev >= 0 && dev < 64, "device ordinal %d out of range", dev);
  if (!g_blas[dev]) {
    cublasHandle_t h;
    if (cublasCreate(&h) != CUBLAS_STATUS_SUCCESS) {
      mk::set_error("cublasCreate failed");
      return MK_ERR_CUBLAS;
    }
    // fixed workspace, so GEMMs inside a captured CUDA graph allocate nothing
    const size_t ws = 32u << 20;
    MK_CUDA(cudaMalloc(&g_blas_ws[dev], ws));
    cublasSetWorkspace(h, g_blas_ws[dev], ws);
    cublasSetMathMode(h, CUBLAS_DEFAULT_MATH);
    g_blas[dev] = h;
  }
  *out = g_blas[dev];
  return MK_OK;
}

// R (nrow x ncol, ld ldr) = A (nrow x nrow) . X (nrow x ncol, ld ldx), all row-major.
// Column-major view: R^T = X^T A^T, i.e. gemm(N, N, m=ncol, n=nrow, k=nrow).
// emulate: 0 = native FP64 / FP32 units; 1 = cuBLAS tensor-core emulation
// (FP64: fixed-point slices, FP32: BF16x9).
int blas_rotate(int dtype, const void *A, const void *X, int64_t ldx, void *R, int64_t ldr,
                int64_t nrow, int64_t ncol, int emulate, cudaStream_t st) {
  std::lock_guard<std::mutex> lk(g_blas_mu);
  cublasHandle_t h;
  int rc = blas_handle(&h);
  if (rc) return rc;
  cublasSetStream(h, st);
  cublasMath_t mode = CUBLAS_DEFAULT_MATH;
  if (emulate) mode = dtype == MK_F64 ? CUBLAS_FP64_EMULATED_FIXEDPOINT_MATH : CUBLAS_FP32_EMULATED_BF16X9_MATH;
  cublasSetMathMode(h, mode);
  cublasSetEmulationStrategy(h, emulate ? CUBLAS_EMULATION_STRATEGY_EAGER : CUBLAS_EMULATION_STRATEGY_DEFAULT);
  cublasStatus_t s;
  if (dtype == MK_F64 && emulate) {
    // explicit emulated compute type: FP64 operands sliced into fixed-point
    // pieces on the integer tensor cores
    const double one = 1.0, zero = 0.0;
    s = cublasGemmEx_64(h, CUBLAS_OP_N, CUBLAS_OP_N, ncol, nrow, nrow, &one, X, CUDA_R_64F, ldx, A,
                        CUDA_R_64F, nrow, &zero, R, CUDA_R_64F, ldr,
                        CUBLAS_COMPUTE_64F_EMULATED_FIXEDPOINT, CUBLAS_GEMM_DEFAULT);
  } else if (dtype == MK_F64) {
    const double one = 1.0, zero = 0.0;
    s = cublasDgemm_64(h, CUBLAS_OP_N, CUBLAS_OP_N, ncol, nrow, nrow, &one, (const double *)X, ldx,
                       (const double *)A, nrow, &zero, (double *)R, ldr);
  } else {
    const float one = 1.f, zero = 0.f;
    s = cublasSgemm_64(h, CUBLAS_OP_N, CUBLAS_OP_N, ncol, nrow, nrow, &one, (const float *)X, ldx,
                       (const float *)A, nrow, &zero, (float *)R, ldr);
  }
  if (s != CUBLAS_STATUS_SUCCESS) {
    mk::set_error("cuBLAS gemm failed (status %d)", (int)s);
    return MK_ERR_CUBLAS;
  }
  return MK_OK;
}

// mode 0 (automatic) means cuBLAS here; the host autotuner picks 2 or 3 per
// workload after checking their accuracy against it.
// mirror_n: see rot_tc_f32 (only the tensor-core kernel fuses the extension;
// the caller runs k_mirror otherwise).
int rotate(DctCore *c, int mode, const void *A, const void *X, int64_t ldx, void *R, int64_t ldr,
           int64_t nrow, int64_t ncol, cudaStream_t st, int64_t mirror_n = 0, int64_t x_stride = 1,
           int halve_ends = 0) {
  const int dtype = c->dtype;
  if (mode == 0) mode = 1;
  if (mode == 2) {
    MK_CHECK_ARG(dtype == MK_F32, "tensor-core rotation (rot_mode 2) is FP32 only");
    MK_CHECK_ARG(c->tc_bimg != nullptr, "tensor-core rotation needs ndet in {32,64,128,256}");
    return mk::rot_tc_f32((const float *)A, (const float *)X, ldx, (float *)R, ldr, nrow, ncol,
                          c->tc_bimg, c->tc_err, st, mirror_n, x_stride, halve_ends);
  }
  if (mode == 4) {
    MK_CHECK_ARG(dtype == MK_F64 && c->oz_ws, "sliced tensor-core rotation (rot_mode 4) is FP64 only");
    std::lock_guard<std::mutex> lk(g_blas_mu);
    cublasHandle_t h;
    int rc = blas_handle(&h);
    if (rc) return rc;
    return mk::ozaki_rotate_f64(h, (const double *)A, (const double *)X, ldx, (double *)R, ldr, nrow, ncol,
                                c->oz_ws, c->oz_bytes, st);
  }
  MK_CHECK_ARG(mode == 1 || mode == 3, "bad rot_mode %d", mode);
  return blas_rotate(dtype, A, X, ldx, R, ldr, nrow, ncol, mode == 3, st);
}

template <typename T, typename C>
int apply_noise_t(DctCore *c, const T *v, const T *vT, const T *w, int64_t ldw, const T *dat,
                  T *out, int rot_mode, cudaStream_t st) {
  const int64_t n = c->n, N = c->N, nd = c->nrow;
  dim3 g = rows_grid(n, nd);
  int rc;
  if (c->own) {
    T *E = (T *)c->E;
    if ((rc = rotate(c, rot_mode, v, dat, n, E, n, nd, n, st))) return rc;
    if ((rc = own_dct(c, E, E, mk::FFT4_FILTER, w, ldw, st))) return rc;
    if ((rc = own_dct(c, E, E, mk::FFT4_HALVE, nullptr, 0, st))) return rc;
    return rotate(c, rot_mode, vT, E, n, out, n, nd, n, st);
  }
  const bool fused_mirror = (rot_mode == 2);  // the tensor-core epilogue writes the extension
  rc = rotate(c, rot_mode, v, dat, n, c->E, N, nd, n, st, fused_mirror ? N : 0);
  if (rc) return rc;
  if (!fused_mirror) {
    k_mirror<T><<<g, 256, 0, st>>>((T *)c->E, n, N, nd);
    if ((rc = mk::launch_status("apply_noise/mirror"))) return rc;
  }
  if ((rc = core_fft(c, st))) return rc;
  k_filter_extend<T, C><<<g, 256, 0, st>>>((const C *)c->F, w, ldw, (T *)c->E, n, N, nd);
  if ((rc = mk::launch_status("apply_noise/filter"))) return rc;
  if ((rc = core_fft(c, st))) return rc;
  if (fused_mirror) {
    // the tensor-core kernel reads the real parts of F in place (stride 2)
    // and halves the end columns while splitting its operand
    return rotate(c, rot_mode, vT, c->F, 2 * n, out, n, nd, n, st, 0, 2, 1);
  }
  k_real_halve<T, C><<<g, 256, 0, st>>>((const C *)c->F, (T *)c->E, n, nd);
  if ((rc = mk::launch_status("apply_noise/halve"))) return rc;
  return rotate(c, rot_mode, vT, c->E, n, out, n, nd, n, st);
}

}  // namespace

struct mk_dct_plan {
  DctCore core;
};
struct mk_noise_plan {
  DctCore core;
};

extern "C" int mk_dct1_workspace_bytes(int64_t nrow, int64_t n, int dtype, size_t *bytes) {
  return core_bytes(nrow, n, dtype, bytes, false);
}

extern "C" int mk_dct1_plan_create(mk_dct_plan **plan, int64_t nrow, int64_t n, int dtype,
                                   void *workspace, size_t workspace_bytes) {
  MK_CHECK_ARG(plan, "mk_dct1_plan_create: null plan pointer");
  *plan = nullptr;
  mk_dct_plan *p = new (std::nothrow) mk_dct_plan;
  if (!p) return MK_ERR_NOMEM;
  int rc = core_create(&p->core, nrow, n, dtype, workspace, workspace_bytes, false);
  if (rc) {
    delete p;
    return rc;
  }
  *plan = p;
  return MK_OK;
}

extern "C" int mk_dct1_exec(mk_dct_plan *plan, const void *in, void *out, void *stream) {
  MK_CHECK_ARG(plan && in && out, "mk_dct1_exec: null pointer");
  cudaStream_t st = mk::as_stream(stream);
  return plan->core.dtype == MK_F64 ? dct_exec_t<double, cufftDoubleComplex>(&plan->core, in, out, st)
                                    : dct_exec_t<float, cufftComplex>(&plan->core, in, out, st);
}

extern "C" int mk_dct1_plan_destroy(mk_dct_plan *plan) {
  if (!plan) return MK_OK;
  core_free(&plan->core);
  delete plan;
  return MK_OK;
}

extern "C" int mk_noise_workspace_bytes(int64_t ndet, int64_t ndata, int dtype, size_t *bytes) {
  return core_bytes(ndet, ndata, dtype, bytes);
}

extern "C" int mk_noise_plan_create(mk_noise_plan **plan, int64_t ndet, int64_t ndata, int dtype,
                                    void *workspace, size_t workspace_bytes) {
  MK_CHECK_ARG(plan, "mk_noise_plan_create: null plan pointer");
  *plan = nullptr;
  mk_noise_plan *p = new (std::nothrow) mk_noise_plan;
  if (!p) return MK_ERR_NOMEM;
  int rc = core_create(&p->core, ndet, ndata, dtype, workspace, workspace_bytes);
  if (rc) {
    delete p;
    return rc;
  }
  *plan = p;
  return MK_OK;
}

extern "C" int mk_apply_noise(mk_noise_plan *plan, const void *v, const void *vT, const void *mywt,
                              int64_t mywt_ld, const void *dat, void *out, int rot_mode,
                              void *stream) {
  MK_CHECK_ARG(plan && v && vT && mywt && dat && out, "mk_apply_noise: null pointer");
  MK_CHECK_ARG(mywt_ld >= plan->core.n, "mk_apply_noise: mywt_ld %lld < ndata %lld",
               (long long)mywt_ld, (long long)plan->core.n);
  cudaStream_t st = mk::as_stream(stream);
  if (plan->core.dtype == MK_F64)
    return apply_noise_t<double, cufftDoubleComplex>(&plan->core, (const double *)v,
                                                     (const double *)vT, (const double *)mywt,
                                                     mywt_ld, (const double *)dat, (double *)out,
                                                     rot_mode, st);
  return apply_noise_t<float, cufftComplex>(&plan->core, (const float *)v, (const float *)vT,
                                            (const float *)mywt, mywt_ld, (const float *)dat,
                                            (float *)out, rot_mode, st);
}

extern "C" int mk_noise_plan_destroy(mk_noise_plan *plan) {
  if (!plan) return MK_OK;
  core_free(&plan->core);
  delete plan;
  return MK_OK;
}

extern "C" int mk_rotate(mk_noise_plan *plan, const void *A, const void *X, void *R, int rot_mode,
                         void *stream) {
  MK_CHECK_ARG(plan && A && X && R, "mk_rotate: null pointer");
  MK_CHECK_ARG(X != R, "mk_rotate: R must not alias X");
  const int64_t nd = plan->core.nrow, n = plan->core.n;
  return rotate(&plan->core, rot_mode, A, X, n, R, n, nd, n, mk::as_stream(stream));
}

extern "C" int mk_noise_status(mk_noise_plan *plan, int *code, void *stream) {
  MK_CHECK_ARG(plan && code, "mk_noise_status: null pointer");
  *code = 0;
  if (!plan->core.tc_err) return MK_OK;
  cudaStream_t st = mk::as_stream(stream);
  MK_CUDA(cudaMemcpyAsync(code, plan->core.tc_err, sizeof(int), cudaMemcpyDeviceToHost, st));
  MK_CUDA(cudaMemsetAsync(plan->core.tc_err, 0, sizeof(int), st));
  MK_CUDA(cudaStreamSynchronize(st));
  return MK_OK;
}

// ---- many TODs, one filter call ---------------------------------------------
// apply_noise in place on every TOD of a group: the v and vT rotations of all
// TODs with the same detector count run as one tensor-core launch each (the
// rotation works in place: a tile's inputs are all read before its outputs
// are written), and each TOD's two DCT-I passes run on its own plan.  The
// rotation operand images are built once, when the group is created.
struct mk_noise_group {
  struct Tod {
    DctCore *core;
    const float *w;
    int64_t ldw;
    float *data;
  };
  struct Class {  // the TODs with one detector count
    int64_t ndet = 0, ntile = 0;
    int njobs = 0;
    mk::RotJob *jobs_v = nullptr, *jobs_vT = nullptr;  // device tables
  };
  std::vector<Tod> tods;
  std::vector<Class> classes;
  void *mem = nullptr;  // operand images, job tables, status word
  int *err = nullptr;
};

extern "C" int mk_noise_group_destroy(mk_noise_group *g) {
  if (!g) return MK_OK;
  cudaFree(g->mem);
  delete g;
  return MK_OK;
}

extern "C" int mk_noise_group_create(mk_noise_group **group, int ntod, mk_noise_plan *const *plans,
                                     const float *const *v, const float *const *vT, const float *const *mywt,
                                     const int64_t *ldw, float *const *data, void *stream) {
  MK_CHECK_ARG(group, "mk_noise_group_create: null group pointer");
  *group = nullptr;
  MK_CHECK_ARG(ntod >= 1 && plans && v && vT && mywt && ldw && data, "mk_noise_group_create: bad arguments");
  for (int t = 0; t < ntod; t++) {
    MK_CHECK_ARG(plans[t] && v[t] && vT[t] && mywt[t] && data[t], "mk_noise_group_create: TOD %d: null pointer",
                 t);
    const DctCore &c = plans[t]->core;
    MK_CHECK_ARG(c.dtype == MK_F32 && mk::rot_tc_supported(c.nrow),
                 "mk_noise_group_create: TOD %d: needs an FP32 plan with ndet in {32,64,128,256}", t);
    MK_CHECK_ARG(ldw[t] >= c.n, "mk_noise_group_create: TOD %d: ldw below ndata", t);
  }
  mk_noise_group *g = new (std::nothrow) mk_noise_group;
  MK_CHECK_ARG(g, "mk_noise_group_create: out of host memory");
  std::vector<int64_t> nds;
  for (int t = 0; t < ntod; t++) {
    const int64_t nd = plans[t]->core.nrow;
    bool seen = false;
    for (int64_t x : nds) seen |= (x == nd);
    if (!seen) nds.push_back(nd);
  }
  // one allocation: per TOD two operand images, per class two job tables, the status word
  size_t bytes = 256, img_total = 0;
  for (int t = 0; t < ntod; t++) img_total += 2 * align_up(mk::rot_tc_bimg_bytes(plans[t]->core.nrow));
  bytes += img_total + 2 * nds.size() * align_up((size_t)ntod * sizeof(mk::RotJob));
  if (cudaMalloc(&g->mem, bytes) != cudaSuccess) {
    delete g;
    mk::set_error("mk_noise_group_create: cudaMalloc of %zu bytes failed", bytes);
    return MK_ERR_CUDA;
  }
  cudaStream_t st = mk::as_stream(stream);
  char *p = (char *)g->mem;
  g->err = (int *)p;
  int rc = cudaMemsetAsync(g->err, 0, sizeof(int), st) == cudaSuccess ? MK_OK : MK_ERR_CUDA;
  p += 256;
  std::vector<const char *> img_v(ntod), img_vT(ntod);
  for (int t = 0; t < ntod && !rc; t++) {
    const DctCore &c = plans[t]->core;
    const size_t ib = align_up(mk::rot_tc_bimg_bytes(c.nrow));
    img_v[t] = p;
    rc = mk::rot_tc_bprep(v[t], c.nrow, p, st);
    p += ib;
    img_vT[t] = p;
    if (!rc) rc = mk::rot_tc_bprep(vT[t], c.nrow, p, st);
    p += ib;
    g->tods.push_back({&plans[t]->core, mywt[t], ldw[t], data[t]});
  }
  for (size_t k = 0; k < nds.size() && !rc; k++) {
    mk_noise_group::Class cl;
    cl.ndet = nds[k];
    std::vector<mk::RotJob> jv, jvT;
    for (int t = 0; t < ntod; t++) {
      const DctCore &c = plans[t]->core;
      if (c.nrow != cl.ndet) continue;
      const int64_t tiles = (c.n + 127) / 128;
      jv.push_back({data[t], data[t], img_v[t], c.n, c.n, c.n, cl.ntile});
      jvT.push_back({data[t], data[t], img_vT[t], c.n, c.n, c.n, cl.ntile});
      cl.ntile += tiles;
    }
    cl.njobs = (int)jv.size();
    const size_t tb = align_up((size_t)ntod * sizeof(mk::RotJob));
    cl.jobs_v = (mk::RotJob *)p;
    p += tb;
    cl.jobs_vT = (mk::RotJob *)p;
    p += tb;
    if (cudaMemcpyAsync(cl.jobs_v, jv.data(), jv.size() * sizeof(mk::RotJob), cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        cudaMemcpyAsync(cl.jobs_vT, jvT.data(), jvT.size() * sizeof(mk::RotJob), cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
      mk::set_error("mk_noise_group_create: uploading the job tables failed");
      rc = MK_ERR_CUDA;
    }
    g->classes.push_back(cl);
  }
  if (rc) {
    mk_noise_group_destroy(g);
    return rc;
  }
  *group = g;
  return MK_OK;
}

extern "C" int mk_noise_group_exec(mk_noise_group *g, void *stream) {
  MK_CHECK_ARG(g, "mk_noise_group_exec: null group");
  cudaStream_t st = mk::as_stream(stream);
  int rc;
  for (const auto &cl : g->classes)
    if ((rc = mk::rot_tc_group(cl.jobs_v, cl.njobs, cl.ntile, cl.ndet, g->err, st))) return rc;
  for (const auto &t : g->tods) {
    DctCore *c = t.core;
    if (c->own) {
      if ((rc = own_dct(c, t.data, t.data, mk::FFT4_FILTER, t.w, t.ldw, st))) return rc;
      if ((rc = own_dct(c, t.data, t.data, mk::FFT4_HALVE, nullptr, 0, st))) return rc;
      continue;
    }
    // a cuFFT plan: extension, transform, filter + extension, transform,
    // real part with the end columns halved, back into the TOD
    const int64_t n = c->n, N = c->N, nd = c->nrow;
    const dim3 gr = rows_grid(n, nd);
    k_extend<float><<<gr, 256, 0, st>>>(t.data, n, (float *)c->E, n, N, nd);
    if ((rc = mk::launch_status("noise group/extend"))) return rc;
    if ((rc = core_fft(c, st))) return rc;
    k_filter_extend<float, cufftComplex><<<gr, 256, 0, st>>>((const cufftComplex *)c->F, t.w, t.ldw,
                                                               (float *)c->E, n, N, nd);
    if ((rc = mk::launch_status("noise group/filter"))) return rc;
    if ((rc = core_fft(c, st))) return rc;
    k_real_halve<float, cufftComplex><<<gr, 256, 0, st>>>((const cufftComplex *)c->F, t.data, n, nd);
    if ((rc = mk::launch_status("noise group/halve"))) return rc;
  }
  for (const auto &cl : g->classes)
    if ((rc = mk::rot_tc_group(cl.jobs_vT, cl.njobs, cl.ntile, cl.ndet, g->err, st))) return rc;
  return MK_OK;
}

extern "C" int mk_noise_group_status(mk_noise_group *g, int *code, void *stream) {
  MK_CHECK_ARG(g && code, "mk_noise_group_status: null pointer");
  cudaStream_t st = mk::as_stream(stream);
  MK_CUDA(cudaMemcpyAsync(code, g->err, sizeof(int), cudaMemcpyDeviceToHost, st));
  MK_CUDA(cudaMemsetAsync(g->err, 0, sizeof(int), st));
  MK_CUDA(cudaStreamSynchronize(st));
  return MK_OK;
}

extern "C" int mk_set_dct_engine(int engine) {
  MK_CHECK_ARG(engine >= 0 && engine <= 2, "mk_set_dct_engine: engine must be 0, 1 or 2 (got %d)", engine);
  g_engine.store(engine);
  return MK_OK;
}

extern "C" int mk_get_dct_engine(void) { return g_engine.load(); }

static int engine_of(const DctCore &c) { return !c.own ? 1 : c.f4.d.blue ? 2 : 0; }

extern "C" int mk_dct1_engine(const mk_dct_plan *plan) { return plan ? engine_of(plan->core) : 1; }

extern "C" int mk_noise_engine(const mk_noise_plan *plan) { return plan ? engine_of(plan->core) : 1; }

extern "C" int mk_set_fft4_split(int rank) {
  MK_CHECK_ARG(rank >= 0 && rank < 16, "mk_set_fft4_split: rank must be 0..15 (got %d)", rank);
  mk::fft4_set_split_rank(rank);
  return MK_OK;
}

extern "C" int mk_get_fft4_split(void) { return mk::fft4_split_rank(); }

extern "C" int mk_noise_split(const mk_noise_plan *plan, int *L1, int *L2) {
  MK_CHECK_ARG(plan && L1 && L2, "mk_noise_split: null argument");
  const bool four = plan->core.own;
  *L1 = four ? plan->core.f4.d.L1 : 0;
  *L2 = four ? plan->core.f4.d.L2 : 0;
  return MK_OK;
}

extern "C" int mk_dct1_describe(int64_t n, int *engine, int64_t *L, int *L1, int *L2) {
  MK_CHECK_ARG(engine && L && L1 && L2, "mk_dct1_describe: null output");
  MK_CHECK_ARG(n >= 2, "mk_dct1_describe: n must be >= 2 (got %lld)", (long long)n);
  const int e = g_engine.load();
  mk::Fft4Dev d;
  if (e != 1 && mk::fft4_shape(n, &d, e == 0)) {
    *engine = d.blue ? 2 : 0;
    *L = d.L;
    *L1 = d.L1;
    *L2 = d.L2;
  } else {
    *engine = 1;
    *L = 2 * (n - 1);
    *L1 = *L2 = 0;
  }
  return MK_OK;
}
