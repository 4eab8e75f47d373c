/*
 * mkgpu.h -- C ABI of libmkgpu.so, the GB300 (sm_103a) mapmaking hot path.
 *
 * Conventions shared by every entry point:
 *  - All array pointers are DEVICE pointers (e.g. torch.Tensor.data_ptr()),
 *    C-contiguous, owned by the caller.  The library owns only plan objects
 *    (cuFFT plans, small reduction scratch) that it creates and destroys.
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default
 *    stream).  Every call is stream-ordered and does not synchronise the host
 *    unless its comment says so.
 *  - Every function returns an int status: MK_OK (0) or an MK_ERR_* code;
 *    mk_last_error() returns a message for the last failure on the calling
 *    host thread.  Asynchronous kernel faults surface at the next call that
 *    synchronises, like any CUDA call.
 *  - dtype selects the arithmetic of the arrays named "dtype-typed":
 *    MK_F64 (double) or MK_F32 (float).  Pixel indices are int32, flattened
 *    as x*ny + y, exactly the reference's ipix.
 *  - Layout of TOD arrays: (ndet, ndata) row-major, i.e. detector-major,
 *    the reference's dat_calib layout.
 *
 * Reference interfaces replaced (paths in the minkasi project):
 *  mk_map2tod          <- map2tod_omp / map2tod_simple, minkasi/lib/minkasi.c:116-144,
 *                         bound in minkasi/lib/minkasi.py (map2tod_omp_c)
 *  mk_tod2map          <- tod2map_omp / tod2map_atomic, minkasi/lib/minkasi.c:59-66,97-112,
 *                         bound in minkasi/lib/minkasi.py:10-60 (tod2map_omp_c)
 *  mk_tod2map_sorted   <- tod2map_everyone / tod2map_cached, minkasi/lib/minkasi.c:68-95
 *                         (the reference's owner-computes variants; here deterministic)
 *  mk_pix_car / mk_pix_wcs_car <- SkyMapCar.pix_from_radec, radec2pix_car and
 *                         SkyMap.pix_from_radec, minkasi/maps/skymap.py:457-490,958-984,
 *                         minkasi/maps/utils.py:178-216
 *  mk_polmap2tod / mk_tod2polmap / mk_pol_precon_mul <- map2tod_{iqu,qu}_omp,
 *                         tod2map_{iqu,qu}_simple, tod2map_{iqu,qu}_precon_simple,
 *                         minkasi/lib/minkasi.c:146-245, and PolMap.__mul__,
 *                         minkasi/maps/polmap.py:624-684
 *  mk_cuts_* / mk_stripes_* / mk_binned_* <- tod2cuts / cuts2tod (minkasi/lib/minkasi.c:260-284),
 *                         map2tod_destriped / tod2map_destriped / *_binned_det,
 *                         minkasi/mapmaking/map2tod.py:156-253, tod2map.py:242-340
 *  mk_tod2map_rows     <- make_hits' tod2map of a ones / outer(weights, ones) TOD,
 *                         minkasi/mapmaking/tod2map.py:343-400
 *  mk_dct1_*           <- many_fft_r2r_1d / many_fftf_r2r_1d (REDFT00),
 *                         minkasi/lib/mkfftw.c:174-254, bound in minkasi/lib/mkfftw.py
 *  mk_noise_*          <- NoiseSmoothedSVD.apply_noise, minkasi/mapmaking/noise.py:680-714
 *  mk_dot / mk_axpy / mk_mul / mk_pcg_*  <- SkyMap.dot/axpy/__mul__ and the
 *                         run_pcg_wprior recurrence, minkasi/maps/skymap.py:428-440,651-666,724-740,
 *                         minkasi/mapmaking/pcg.py:101-178
 */
#ifndef MKGPU_H
#define MKGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  MK_OK = 0,
  MK_ERR_ARG = 1,      /* bad argument (null pointer, size, dtype, alignment) */
  MK_ERR_CUDA = 2,     /* CUDA runtime error */
  MK_ERR_CUFFT = 3,    /* cuFFT error */
  MK_ERR_CUBLAS = 4,   /* cuBLAS error */
  MK_ERR_RANGE = 5,    /* pixel index outside [0, npix) */
  MK_ERR_NOMEM = 6,    /* host or device allocation failed */
  MK_ERR_NUMERIC = 7   /* CG breakdown (p.Ap <= 0) or non-finite scalar */
};

enum { MK_F64 = 0, MK_F32 = 1 };

/* ---- library ---------------------------------------------------------- */
const char *mk_last_error(void);
int mk_version(void);          /* returns the ABI version number (not a status) */

/* ---- pointing projections ---------------------------------------------- */

/* dat[i] = map[ipix[i]] (do_add=0) or dat[i] += map[ipix[i]] (do_add=1),
 * i over ndet*ndata samples.  dat, map dtype-typed.  A sample whose pixel is
 * outside [0, npix) gathers 0 (the reference would read out of bounds).
 * Replaces map2tod_omp, minkasi/lib/minkasi.c:131-144. */
int mk_map2tod(void *dat, const void *map, const int32_t *ipix, int64_t ndet,
               int64_t ndata, int64_t npix, int dtype, int do_add, void *stream);

/* map[ipix[i]] += dat[i] with warp-aggregated atomic adds: runs of equal
 * consecutive pixels are summed in registers and joined across the lanes of
 * a warp, one atomic per run.  Summation order, and so the last bits, vary
 * from run to run.  Out-of-range pixels are skipped.
 * Replaces tod2map_omp / tod2map_atomic, minkasi/lib/minkasi.c:59-66,97-112. */
int mk_tod2map(void *map, const void *dat, const int32_t *ipix, int64_t ndet,
               int64_t ndata, int64_t npix, int dtype, void *stream);

/* The same sum as mk_tod2map, with the sample and pixel streams staged
 * through shared memory by bulk asynchronous copies (a ring of chunks per
 * CTA, so several chunks per SM are in flight from HBM while the previous
 * one is reduced).  dat and ipix must be 16-byte aligned device memory (not
 * host-mapped); MK_ERR_ARG otherwise.  If a copy never arrives, the kernel
 * stops after a bounded wait and mk_tod2map_status reports it.
 * Replaces tod2map_omp, minkasi/lib/minkasi.c:97-112. */
int mk_tod2map_staged(void *map, const void *dat, const int32_t *ipix, int64_t ndet,
                      int64_t ndata, int64_t npix, int dtype, void *stream);

/* *code = 1 if a mk_tod2map_staged kernel on the current device stopped on
 * a timed-out wait since the last call (its map update is then incomplete),
 * else 0.  Reads and clears the flag; synchronises `stream`.  No reference
 * counterpart (the reference's CPU loops cannot time out). */
int mk_tod2map_status(int *code, void *stream);

/* ---- pointing -> pixel index ------------------------------------------
 * ra, dec: n FP64 samples in radians (device); ipix: n int32 (device).
 * trunc = 0: SkyMapCar.pix_from_radec, minkasi/maps/skymap.py:958-984:
 *   ipix = int32(round_half_even((ra - ra0) * cosdec / pixsize) * ny
 *                + (dec - dec0) / pixsize + 0.5)
 * trunc = 1: radec2pix_car, minkasi/maps/utils.py:178-216:
 *   ipix = int((ra - ra0) * cosdec / pixsize + 0.5) * ny + int((dec - dec0) / pixsize + 0.5)
 * ra0 = lims[0], dec0 = lims[2].  Same FP64 operation order as the
 * reference and no fused multiply-adds: bit-identical indices.  A value
 * outside the int32 range (or NaN) gives INT32_MIN, as numpy does on x86-64. */
int mk_pix_car(int32_t *ipix, const double *ra, const double *dec, int64_t n, double ra0,
               double dec0, double pixsize, double cosdec, int64_t ny, int trunc, void *stream);

/* SkyMap.pix_from_radec, minkasi/maps/skymap.py:457-490, for the CAR WCS of
 * get_wcs (minkasi/maps/utils.py:13-67).  wcs6 (host): crval1, crval2,
 * crpix1, crpix2, cdelt1, cdelt2 in degrees.  World -> native rotation with
 * the default LONPOLE/LATPOLE, CAR projection, p = crpix + x / cdelt, then
 * ipix = int32(round(p1 - 1) * ny + round(p2 - 1)).  Replaces astropy's
 * wcs_world2pix on this path; FP64 trigonometry, so a coordinate within a
 * few ulp of a half-pixel boundary may round the other way than astropy. */
int mk_pix_wcs_car(int32_t *ipix, const double *ra, const double *dec, int64_t n,
                   const double *wcs6, int64_t ny, void *stream);

/* ---- polarized projections (PolMap) ------------------------------------
 * Stokes maps are pixel-major, map[p * npol + k], as the reference's
 * (nx, ny, npol) array.  With c = cos(twogamma), s = sin(twogamma):
 *   MK_POL_QU          npol 2  (Q, U)                   minkasi/lib/minkasi.c:162-174,187-194
 *   MK_POL_IQU         npol 3  (I, Q, U)                minkasi.c:146-159,176-185
 *   MK_POL_QU_PRECON   npol 3  (QQ, UU, QU)             minkasi.c:196-207
 *   MK_POL_IQU_PRECON  npol 6  (I, Q, U, QQ, QU, UU)    minkasi.c:231-245
 * The angle terms come either from cos2g/sin2g (dtype-typed, n each, made
 * once per TOD by mk_pol_sincos) or, when cos2g is NULL, from twogamma (n
 * doubles, FP64 only): the reference's argument, evaluated per call. */
enum { MK_POL_QU = 1, MK_POL_IQU = 2, MK_POL_QU_PRECON = 3, MK_POL_IQU_PRECON = 4 };

/* Stokes components per pixel of a mode (0 for an unknown mode); not a status. */
int mk_pol_npol(int mode);

/* cos2g[i] = cos(twogamma[i]), sin2g[i] = sin(twogamma[i]) (FP64 math,
 * stored in dtype).  No reference counterpart: the reference recomputes
 * them inside every projection call (minkasi.c:146-245). */
int mk_pol_sincos(void *cos2g, void *sin2g, const double *twogamma, int64_t n, int dtype,
                  void *stream);

/* dat (+)= the IQU or QU projection of map (modes MK_POL_QU / MK_POL_IQU;
 * the PRECON modes have no map2tod in the reference either).  Out-of-range
 * pixels gather 0.  Replaces map2tod_iqu_omp / map2tod_qu_omp,
 * minkasi/lib/minkasi.c:146-174, called by polmap2tod,
 * minkasi/mapmaking/map2tod.py:57-122. */
int mk_polmap2tod(void *dat, const void *map, const void *cos2g, const void *sin2g,
                  const double *twogamma, const int32_t *ipix, int64_t ndet, int64_t ndata,
                  int64_t npix, int mode, int dtype, int do_add, void *stream);

/* map += the mode's Stokes weights of dat (atomic adds; one per component
 * per run of equal pixels).  dat == NULL: d = rowval[det] (rowval == NULL:
 * 1), the hit / weight maps of make_hits on a PolMap.  Out-of-range pixels
 * are skipped.  Replaces tod2map_{qu,iqu}_simple and tod2map_{qu,iqu}_precon_simple,
 * minkasi/lib/minkasi.c:176-207,231-245, called by tod2polmap,
 * minkasi/mapmaking/tod2map.py:164-215. */
int mk_tod2polmap(void *map, const void *dat, const void *cos2g, const void *sin2g,
                  const double *twogamma, const int32_t *ipix, int64_t ndet, int64_t ndata,
                  int64_t npix, int mode, int dtype, const void *rowval, void *stream);

/* out = P . map per pixel for a PRECON map P (mode MK_POL_QU_PRECON with a
 * QU map, MK_POL_IQU_PRECON with an IQU map; out may alias map).
 * Replaces PolMap.__mul__, minkasi/maps/polmap.py:624-684. */
int mk_pol_precon_mul(void *out, const void *precon, const void *map, int64_t npix, int mode,
                      int dtype, void *stream);

/* ---- per-TOD model members of a Mapset (cuts, stripes, binned) ---------
 * dtype-typed dat / vec / pars; index arrays int64 (the reference's imap and
 * segment edges).  Indices outside their array are skipped. */

/* vec[i] (+)= dat[imap[i]], i < ncut, imap into the ndat samples of a TOD.
 * Replaces tod2cuts, minkasi/lib/minkasi.c:260-268 (CutsCompact.tod2map,
 * minkasi/tods/cuts.py:351-383). */
int mk_cuts_gather(void *vec, const void *dat, const int64_t *imap, int64_t ncut, int64_t ndat,
                   int dtype, int do_add, void *stream);

/* dat[imap[i]] (+)= vec[i] (atomic adds with do_add, so overlapping cut
 * segments add up as in the reference's serial loop).  Replaces cuts2tod,
 * minkasi/lib/minkasi.c:271-284 (CutsCompact.map2tod, cuts.py:385-417). */
int mk_cuts_scatter(void *dat, const void *vec, const int64_t *imap, int64_t ncut, int64_t ndat,
                    int dtype, int do_add, void *stream);

/* Destriper: dat[d, t] (+)= pars[d, s] for lims[s] <= t < lims[s+1];
 * pars (ndet, nseg), lims (nseg + 1) on the device.  Replaces
 * map2tod_destriped, minkasi/mapmaking/map2tod.py:156-190 (tsStripes). */
int mk_stripes_map2tod(void *dat, const void *pars, const int64_t *lims, int64_t ndet,
                       int64_t ndata, int64_t nseg, int dtype, int do_add, void *stream);

/* pars[d, s] (+)= sum of dat[d, lims[s] .. lims[s+1]-1], a fixed reduction
 * order per segment (reproducible): the transpose of mk_stripes_map2tod.
 * Replaces tod2map_destriped, minkasi/mapmaking/tod2map.py:242-269. */
int mk_stripes_tod2map(void *pars, const void *dat, const int64_t *lims, int64_t ndet,
                       int64_t ndata, int64_t nseg, int dtype, int do_add, void *stream);

/* Binned model: b(t) = int64((vec[t] - lo) * (nbin / (hi - lo))), vec FP64 of
 * ndata entries shared by the detectors (vec_per_det = 0) or (ndet, ndata).
 * dat[d, t] (+)= pars[d, b(t)] (0 outside [0, nbin) when not adding).
 * Replaces map2tod_binned_det, minkasi/mapmaking/map2tod.py:195-253 (tsBinnedAz). */
int mk_binned_map2tod(void *dat, const void *pars, const double *vec, int64_t ndet, int64_t ndata,
                      int64_t nbin, double lo, double hi, int vec_per_det, int dtype, int do_add,
                      void *stream);

/* pars[d, b] (+)= sum of dat[d, t] over the samples with b(t) = b: the exact
 * transpose of mk_binned_map2tod.  The reference's tod2map_binned_det
 * (minkasi/mapmaking/tod2map.py:272-340) writes pars[det][inds] += mat[det]
 * with numpy / numba fancy indexing, which keeps one sample per repeated bin;
 * this sums them all, as the adjoint that a PCG operator needs. */
int mk_binned_tod2map(void *pars, const void *dat, const double *vec, int64_t ndet, int64_t ndata,
                      int64_t nbin, double lo, double hi, int vec_per_det, int dtype, int do_add,
                      void *stream);

/* make_hits helper: map[ipix[d,t]] += w[d] (w == NULL: += 1).  w and map
 * dtype-typed.  Replaces the tod2map of np.ones / np.outer(weights, ones)
 * in make_hits, minkasi/mapmaking/tod2map.py:343-400. */
int mk_tod2map_rows(void *map, const void *w, const int32_t *ipix, int64_t ndet,
                    int64_t ndata, int64_t npix, int dtype, void *stream);

/* Counts pixel indices outside [0, npix) into *nbad (host pointer).
 * Synchronises `stream`.  The reference only warns on a non-int32 dtype
 * (minkasi/mapmaking/tod2map.py:48-51); this is the bounds check it lacks. */
int mk_check_pix(const int32_t *ipix, int64_t n, int64_t npix, int64_t *nbad,
                 void *stream);

/* Deterministic tod2map.  A pixel plan sorts the (fixed) pointing once:
 * for each pixel, the list of sample indices that hit it, in sample order.
 * mk_tod2map_sorted then sums each pixel's samples in that fixed order and
 * adds the sum to map[p]: bitwise reproducible run to run.  Owner-computes
 * like tod2map_everyone, minkasi/lib/minkasi.c:68-83.
 * Plan device memory: 4*(n + npix + 1) bytes plus sort scratch during
 * creation.  n must be < 2^31. */
typedef struct mk_pixplan mk_pixplan;
int mk_pixplan_create(mk_pixplan **plan, const int32_t *ipix, int64_t n,
                      int64_t npix, void *stream);
int mk_tod2map_sorted(void *map, const void *dat, const mk_pixplan *plan,
                      int dtype, void *stream);
int mk_pixplan_destroy(mk_pixplan *plan);

/* Deterministic tod2map by 64-bit fixed-point accumulation: each sample
 * contributes llrint(dat[i] * 2^s) to an int64 accumulator per pixel (integer
 * atomics, so the result is bitwise independent of their order), then
 * map[p] += acc[p] * 2^-s.  s is chosen on the device from max|dat| and
 * `hmax`, an upper bound on the number of samples hitting any one pixel
 * (fixed by the pointing; e.g. the max of the hit map), so no accumulator
 * can overflow.  Rounding: |error| <= hits * max|dat| * 2^-(62-hbits) per
 * pixel, below FP64 summation error for hmax <= 2^24.  s comes from the
 * finite samples only; a NaN or +-inf sample is added straight into its own
 * pixel (a floating-point atomic), so as in the reference's serial sum a
 * pixel ends up NaN or +-inf exactly when its samples make it so, and the
 * other pixels are unaffected.
 * `scratch`: device, 256-byte aligned, mk_tod2map_fixed_scratch_bytes(npix)
 * bytes, zeroed once before first use; every call leaves it zeroed again.
 * Calls that share a scratch must be ordered on one stream. */
size_t mk_tod2map_fixed_scratch_bytes(int64_t npix);
int mk_tod2map_fixed(void *map, const void *dat, const int32_t *ipix, int64_t ndet,
                     int64_t ndata, int64_t npix, int64_t hmax, int dtype, void *scratch,
                     void *stream);

/* mk_tod2map_fixed without a scratch argument.  This entry point has no
 * counterpart in the reference.  It exists for callers that cannot allocate
 * device memory: a host binding that only forwards pointers it was handed,
 * or a process whose memory pool owns the GPU and must not be bypassed by a
 * cudaMalloc.  It allocates nothing.  Its accumulator is a device array
 * built into the library (a 256-byte header plus 8 bytes per pixel for up to
 * MK_NOALLOC_MAX_NPIX pixels, 32 MiB), which every GPU that loads the
 * library holds until the process exits.  npix above the limit is rejected
 * with MK_ERR_ARG, and so is a negative npix.  The first call on a device
 * looks up that array's device address (cudaGetSymbolAddress, with that
 * device current) and caches it for the life of the process; make this first
 * call before any stream capture.  A cudaDeviceReset unloads the module and
 * leaves the cached address stale: do not call this entry point on a device
 * after resetting it.  All calls share the one array, which
 * every complete call leaves zeroed: calls that overlap on the GPU (on
 * different streams, or from different host threads without ordering) race
 * and give wrong maps.  Inputs, outputs and results are as mk_tod2map_fixed. */
#define MK_NOALLOC_MAX_NPIX (4194304LL)
int mk_tod2map_fixed_noalloc(void *map, const void *dat, const int32_t *ipix, int64_t ndet,
                             int64_t ndata, int64_t npix, int64_t hmax, int dtype,
                             void *stream);

/* ---- DCT-I and the SmoothedSVD noise filter --------------------------- */

/* Batched unnormalised DCT-I (FFTW REDFT00) of nrow rows of length n >= 2:
 * X_k = x_0 + (-1)^k x_{n-1} + 2 sum_{j=1}^{n-2} x_j cos(pi j k/(n-1)).
 * The DCT-I is the real part of bins 0..n-1 of the DFT of the even
 * extension (length 2(n-1)).  Plans of both precisions use this library's
 * four-step shared-memory FFT (two rows per complex transform, the
 * extension formed while loading; FP64 plans run it in double precision):
 * two kernels per DCT when 2(n-1) factors into 2, 3, 5, 7, 11, three
 * (Bluestein's algorithm) otherwise, and a batched cuFFT real-to-complex
 * transform of the extension beyond its length limit or with engine 1.
 * `in` and `out` are (nrow, n) dtype-typed and may alias.  The plan uses a
 * workspace of mk_dct1_workspace_bytes() bytes that the CALLER provides
 * (device pointer, 256-byte aligned) and keeps alive while the plan is used.
 * The workspace holds only scratch of one call, so plans of any shapes may
 * share one (sized for the largest) when their calls are stream-ordered.
 * What a plan keeps between calls (cuFFT's plan data; the four-step
 * engine's twiddle and permutation tables, at most a few hundred KB; the
 * tensor-core status word) is device memory the plan allocates at creation
 * and frees on destroy.
 * Replaces many_fft_r2r_1d / many_fftf_r2r_1d, minkasi/lib/mkfftw.c:174-254. */
typedef struct mk_dct_plan mk_dct_plan;
int mk_dct1_workspace_bytes(int64_t nrow, int64_t n, int dtype, size_t *bytes);
int mk_dct1_plan_create(mk_dct_plan **plan, int64_t nrow, int64_t n, int dtype,
                        void *workspace, size_t workspace_bytes);
int mk_dct1_exec(mk_dct_plan *plan, const void *in, void *out, void *stream);
int mk_dct1_plan_destroy(mk_dct_plan *plan);

/* Transform for DCT / noise plans created after the call: engine 0
 * (default) as described above, 1 = cuFFT for every plan, 2 = the four-step
 * FFT only where 2(n-1) factors into 2, 3, 5, 7, 11.  mk_dct1_engine /
 * mk_noise_engine report what a plan uses (0 = four-step FFT, 2 = four-step
 * FFT through Bluestein, 1 = cuFFT). */
int mk_set_dct_engine(int engine);
int mk_get_dct_engine(void);
int mk_dct1_engine(const mk_dct_plan *plan);
/* What an FP32 plan for rows of length n would use under the current
 * engine, without creating it (host only, no GPU needed): *engine as
 * mk_dct1_engine, *L the transform length (2(n-1), or Bluestein's M), and
 * its four-step split *L1 x *L2 (0 x 0 for cuFFT). */
int mk_dct1_describe(int64_t n, int *engine, int64_t *L, int *L1, int *L2);
/* The four-step split (the tile shape of the two passes) that FP32 plans
 * created after the call take: rank 0 (default) = the divisor pair L1 x L2
 * of the transform length closest to sqrt(L), rank r = the r-th next
 * closest (the last one when there are fewer).  The autotuner times a few
 * ranks per TOD shape.  mk_noise_split reports a noise plan's L1 x L2
 * (0 x 0 for cuFFT).  No reference counterpart (FFTW plans its own). */
int mk_set_fft4_split(int rank);
int mk_get_fft4_split(void);

/* NoiseSmoothedSVD.apply_noise, minkasi/mapmaking/noise.py:680-714:
 *   out = halve_ends( vT . DCT1( mywt[:, :ndata] * DCT1( v . dat ) ) )
 * where halve_ends multiplies columns 0 and ndata-1 by 1/2.  v, vT are
 * (ndet, ndet); mywt is (ndet, mywt_ld) with mywt_ld >= ndata (the reference
 * slices mywt[:, :nn]); dat and out are (ndet, ndata); all dtype-typed.
 * `out` may alias `dat`.  Prewhitening (noisevec) is folded into v and vT by
 * the caller.  The plan shares the DCT workspace contract above and may be
 * used for any TOD of the same (ndet, ndata).  rot_mode selects the
 * detector-rotation GEMM: 0 = automatic, 1 = cuBLAS on the FP64 / FP32 units
 * (DGEMM / SGEMM), 2 = this library's tensor-core kernel (FP32 only: 3xTF32
 * split products, FP32 accumulate), 3 = cuBLAS tensor-core emulation (FP64:
 * fixed-point slices; FP32: BF16x9), 4 = FP64 only: this library's exact
 * slicing of both operands into 8 integer slices of 7 bits after power-of-two
 * row / column scaling, their products as bf16 tensor-core GEMMs with FP32
 * accumulation (exact: every sum stays below 2^24), combined in int64 and
 * rounded to FP64 once (ndet <= 1040; the plan's workspace holds its
 * scratch, about 1 GB at ndet = 256). */
typedef struct mk_noise_plan mk_noise_plan;
int mk_noise_workspace_bytes(int64_t ndet, int64_t ndata, int dtype, size_t *bytes);
int mk_noise_plan_create(mk_noise_plan **plan, int64_t ndet, int64_t ndata, int dtype,
                         void *workspace, size_t workspace_bytes);
int mk_apply_noise(mk_noise_plan *plan, const void *v, const void *vT, const void *mywt,
                   int64_t mywt_ld, const void *dat, void *out, int rot_mode, void *stream);
int mk_noise_plan_destroy(mk_noise_plan *plan);
int mk_noise_engine(const mk_noise_plan *plan);
int mk_noise_split(const mk_noise_plan *plan, int *L1, int *L2);

/* The detector rotation alone, R = A . X, for the plan's (ndet, ndata):
 * A (ndet, ndet), X and R (ndet, ndata), dtype-typed, R must not alias X.
 * rot_mode as for mk_apply_noise.  Same GEMM as np.dot(self.v, dat),
 * minkasi/mapmaking/noise.py:704. */
int mk_rotate(mk_noise_plan *plan, const void *A, const void *X, void *R, int rot_mode,
              void *stream);

/* Device status of the plan's tensor-core kernels: *code = 1 if one of
 * their bounded waits timed out since the last call (the kernel then stops,
 * frees its tensor memory and leaves its output incomplete), else 0.  Reads
 * and clears the word; synchronises `stream`. */
int mk_noise_status(mk_noise_plan *plan, int *code, void *stream);

/* NoiseSmoothedSVD.apply_noise of many TODs in one call, in place on each
 * TOD's (ndet, ndata) float32 timestream data[t] (the batched operator's
 * pooled buffer): the v and vT detector rotations of all TODs with the same
 * detector count run as one tensor-core launch each (3xTF32, as rot_mode 2),
 * and each TOD's two DCT-I run on its plan (plans[t]: FP32, any DCT engine,
 * ndet in {32, 64, 128, 256}).  Same arithmetic as mk_apply_noise with
 * rot_mode 2 on each TOD, bit for bit.  The group keeps the rotation
 * operand images of v and vT (built at creation: 8 ndet^2 bytes each) and
 * the device job tables; the data pointers, v, vT and mywt must stay valid
 * and unchanged while it is used.  Plans that share a workspace must have
 * their calls ordered on one stream.  mk_noise_group_status reports (and
 * clears) a timed-out wait inside the rotation kernel.  Replaces the
 * per-TOD loop of minkasi/tods/core.py:517-580 (Tod.apply_noise) inside
 * TodVec.dot (core.py:967-1026). */
typedef struct mk_noise_group mk_noise_group;
int mk_noise_group_create(mk_noise_group **group, int ntod, mk_noise_plan *const *plans,
                          const float *const *v, const float *const *vT, const float *const *mywt,
                          const int64_t *ldw, float *const *data, void *stream);
int mk_noise_group_exec(mk_noise_group *group, void *stream);
int mk_noise_group_status(mk_noise_group *group, int *code, void *stream);
int mk_noise_group_destroy(mk_noise_group *group);

/* ---- map-space vector algebra and the PCG recurrence ------------------- */

/* *result (DEVICE double) = sum_i a[i]*b[i], accumulated in FP64 with a
 * fixed reduction tree (bitwise reproducible).  a, b dtype-typed.
 * `scratch` is a device buffer of at least mk_reduce_scratch_bytes() bytes,
 * zeroed once by the caller before first use (the kernel leaves it zeroed).
 * Replaces SkyMap.dot (np.sum(a*b)), minkasi/maps/skymap.py:651-666. */
size_t mk_reduce_scratch_bytes(void);
int mk_dot(const void *a, const void *b, int64_t n, int dtype, double *result,
           void *scratch, void *stream);

/* y = y + alpha*x with host scalar alpha (SkyMap.axpy, skymap.py:428-440). */
int mk_axpy(void *y, const void *x, double alpha, int64_t n, int dtype, void *stream);
/* out = a * b elementwise (SkyMap.__mul__, skymap.py:724-740). */
int mk_mul(void *out, const void *a, const void *b, int64_t n, int dtype, void *stream);

/* One PCG update with every scalar kept on the device, so an iteration can
 * be captured in a CUDA graph with no host round trip.  `s` is a device
 * array of MK_PCG_NSCALAR doubles; on entry s[MK_S_ZR] holds z.r.
 * Follows run_pcg_wprior, minkasi/mapmaking/pcg.py:137-171:
 *   pAp = p.Ap; alpha = zr/pAp; x += alpha p; r += (-alpha) Ap;
 *   z = precon*r (precon NULL: z = r); zr' = r.z; beta = zr'/zr;
 *   p = z + beta p;  also s[MK_S_RR] = r.r.
 * x, r, z, p, Ap, precon are dtype-typed maps of n pixels.  `scratch` as for
 * mk_dot.  If pAp <= 0 or a scalar is non-finite, s[MK_S_FLAG] is set to 1
 * and x, r, p are left unchanged from that point on. */
enum { MK_S_ZR = 0, MK_S_PAP = 1, MK_S_ALPHA = 2, MK_S_ZRNEW = 3, MK_S_BETA = 4,
       MK_S_RR = 5, MK_S_FLAG = 6, MK_S_ITER = 7, MK_PCG_NSCALAR = 8 };
int mk_pcg_update(void *x, void *r, void *z, void *p, const void *Ap, const void *precon,
                  int64_t n, int dtype, double *s, void *scratch, void *stream);

/* PCG start: r = b - Ax; z = precon*r; p = z; s[MK_S_ZR] = r.z; s[MK_S_RR] = r.r;
 * flag and iteration counter cleared.  pcg.py:101-121. */
int mk_pcg_init(void *r, void *z, void *p, const void *b, const void *Ax,
                const void *precon, int64_t n, int dtype, double *s, void *scratch,
                void *stream);

/* Split form of mk_pcg_update for an operator preconditioner z = M(r)
 * (e.g. the learned SPD convolutional preconditioner) computed between the
 * two calls:  mk_pcg_step_xr: pAp, alpha, x += alpha p, r += (-alpha) Ap,
 * s[MK_S_RR] = r.r;  then the caller computes z = M(r);  mk_pcg_step_zp:
 * zr' = r.z, beta = zr'/zr, p = z + beta p.  Same recurrence as
 * minkasi/mapmaking/pcg.py:137-171 with `precon * r` generalised to M(r). */
int mk_pcg_step_xr(void *x, void *r, const void *p, const void *Ap, int64_t n, int dtype,
                   double *s, void *scratch, void *stream);
int mk_pcg_step_zp(const void *z, const void *r, void *p, int64_t n, int dtype, double *s,
                   void *scratch, void *stream);

/* out = d * (a + b) elementwise (b may be NULL); dtype-typed maps. */
int mk_scale_add(void *out, const void *d, const void *a, const void *b, int64_t n, int dtype,
                 void *stream);

/* ---- learned preconditioner: 3x3 convolutions (no reference counterpart;
 * they implement the SPD map-space preconditioner M = D^-1/2 (I + K^T K) D^-1/2
 * that replaces the elementwise `precon * r` of minkasi/mapmaking/pcg.py:157-158)
 * Layout [B][C][H][W] float32, 1 <= C <= 16, zero padding, w [Cout][Cin][3][3].
 *   fwd : y[b,co,p] = sum_{ci,d} w[co,ci,d] x[b,ci,p+d]
 *   adj : x[b,ci,q] = sum_{co,d} w[co,ci,d] y[b,co,q-d]   (exact adjoint of fwd)
 *   wgrad: g[co,ci,d] = sum_{b,p} h[b,co,p] x[b,ci,p+d]   (reproducible order)
 */
int mk_conv3x3_fwd(const float *x, const float *w, float *y, int B, int Cin, int Cout, int H,
                   int W, void *stream);
int mk_conv3x3_adj(const float *y, const float *w, float *x, int B, int Cin, int Cout, int H,
                   int W, void *stream);
size_t mk_conv3x3_wgrad_scratch_bytes(int B, int Cin, int Cout, int H, int W);
int mk_conv3x3_wgrad(const float *x, const float *h, float *g, int B, int Cin, int Cout, int H,
                     int W, void *scratch, size_t scratch_bytes, void *stream);

/* z = M r for the learned preconditioner on one H x W map, in one call:
 *   u = dsq * r,  z = dsq * (u + K^T K u),  K = L_n ... L_1,
 * dsq = D^-1/2 (0 on unhit pixels).  Layer l maps channels[l-1] ->
 * channels[l] (channels[0] = 1, all <= 16) with weights[l-1] (a host array
 * of device pointers, each [channels[l]][channels[l-1]][3][3] float32).  The
 * first and last convolutions form u and z themselves; the 2(n-1) others
 * run FP32 through `work` (mk_learned_precon_work_bytes).  z, r, dsq are
 * dtype-typed maps; z may alias r.  Replaces the elementwise `precon * r`
 * of minkasi/mapmaking/pcg.py:157-158 (no reference counterpart). */
size_t mk_learned_precon_work_bytes(int H, int W, int nlayer, const int *channels);
int mk_learned_precon_apply(void *z, const void *r, const void *dsq, int H, int W, int nlayer,
                            const int *channels, const float *const *weights, float *work,
                            size_t work_bytes, int dtype, void *stream);

/* The same preconditioner as one stencil: the layers are linear and
 * shift-invariant, so K^T K is a single-channel convolution with a
 * (2 half + 1)^2 kernel C, its impulse response (half = 2n for n layers;
 * 17 x 17 for 4).  This call computes
 *   u = dsq * r,  z = dsq * (u + C * u),  (C * u)[y][x] = sum C[dy][dx] u[y+dy-half][x+dx-half]
 * with u = 0 outside the map, in one launch, FP32 stencil sums.  `kern` is
 * the device array C, (2 half + 1)^2 float32, half <= 8; a symmetric C gives
 * a symmetric M.  Wherever u vanishes within `half` pixels of the map edge
 * this equals mk_learned_precon_apply; nearer the edge it zero-pads once
 * instead of after every layer (still SPD for C = the impulse response of
 * K^T K).  z, r, dsq are dtype-typed maps; z must not alias r.
 * pool > 1 applies the network on a coarser grid (the multi-scale form):
 *   z = dsq * (u + P^T C * P u)
 * with P the pool x pool block mean (pixels outside the map count as 0) and
 * P^T its transpose; the footprint is then pool (2 half + 1) pixels.  It
 * needs `work` of mk_learned_precon_stencil_work_bytes(H, W, pool) bytes
 * (two coarse maps); pool == 1 needs none. */
size_t mk_learned_precon_stencil_work_bytes(int H, int W, int pool);
int mk_learned_precon_stencil(void *z, const void *r, const void *dsq, int H, int W, int half,
                              const float *kern, int pool, void *work, size_t work_bytes, int dtype,
                              void *stream);

#ifdef __cplusplus
}
#endif
#endif /* MKGPU_H */
