// Pointing -> pixel index: the int32 ipix stream of a TOD from its RA/dec
// timestreams (radians, FP64), computed on the GPU.
//
//   mk_pix_car (trunc=0)  SkyMapCar.pix_from_radec   minkasi/maps/skymap.py:958-984
//   mk_pix_car (trunc=1)  radec2pix_car              minkasi/maps/utils.py:178-216
//   mk_pix_wcs_car        SkyMap.pix_from_radec      minkasi/maps/skymap.py:457-490, i.e.
//                         astropy's world->pixel for the CAR WCS that get_wcs builds
//                         (minkasi/maps/utils.py:13-67)
//
// The two flat formulas are evaluated in the reference's operation order with
// every operation rounded on its own (__dsub_rn, __dmul_rn, __ddiv_rn,
// __dadd_rn: no contraction into fused multiply-adds), so the indices are
// bit-identical to the reference's.
//
// The WCS path restates the FITS celestial-coordinate equations (Calabretta &
// Greisen 2002, A&A 395, 1077): the world -> native spherical rotation (their
// eq. 5) about the celestial pole (alpha_p, delta_p) that the reference point
// (crval) and the default LONPOLE/LATPOLE give (eqs. 8-10, with the CAR native
// reference point (phi0, theta0) = (0, 0)), then the CAR projection x = phi,
// y = theta (degrees) and the linear step p = crpix + x / cdelt.  Its
// trigonometry is CUDA's, so a pixel whose coordinate lies within a few ulp
// of a rounding boundary can differ from astropy's.
//
// All kernels are streams over the samples: 16 B read, 4 B written per sample.
#include <math.h>

#include "mk_common.cuh"

namespace {

// double -> int32 by truncation (the C cast of numpy's astype("int32"));
// NaN and values outside the int32 range give INT32_MIN, as numpy does on
// x86-64.
__device__ __forceinline__ int32_t trunc_i32(double v) {
  if (!(v > -2147483649.0 && v < 2147483648.0)) return INT32_MIN;
  return __double2int_rz(v);
}

__device__ __forceinline__ int64_t trunc_i64(double v) {
  if (!(v > -9.2233720368547758e18 && v < 9.2233720368547758e18)) return INT64_MIN;
  return __double2ll_rz(v);
}

template <bool TRUNC>
__global__ void __launch_bounds__(256) k_pix_car(int32_t *__restrict__ ipix, const double *__restrict__ ra,
                                                 const double *__restrict__ dec, int64_t n, double ra0,
                                                 double dec0, double pixsize, double cosdec, int64_t ny) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const double nyd = (double)ny;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const double a = __ldcs(ra + i), d = __ldcs(dec + i);
    // ((ra - lims[0]) * cosdec) / pixsize and (dec - lims[2]) / pixsize
    const double xs = __ddiv_rn(__dmul_rn(__dsub_rn(a, ra0), cosdec), pixsize);
    const double ys = __ddiv_rn(__dsub_rn(d, dec0), pixsize);
    int32_t p;
    if (TRUNC) {
      // int(x + 0.5) each, then xpix * ny + ypix in integers
      const int64_t xp = trunc_i64(__dadd_rn(xs, 0.5));
      const int64_t yp = trunc_i64(__dadd_rn(ys, 0.5));
      p = (int32_t)(uint32_t)((uint64_t)xp * (uint64_t)ny + (uint64_t)yp);
    } else {
      // np.round(x) (half to even), y + 0.5, then (xpix * ny + ypix) -> int32
      const double xp = rint(xs);
      const double yp = __dadd_rn(ys, 0.5);
      p = trunc_i32(__dadd_rn(__dmul_rn(xp, nyd), yp));
    }
    __stcs(ipix + i, p);
  }
}

struct WcsCar {
  double alpha_p;        // celestial longitude of the native pole (deg)
  double sin_dp, cos_dp; // of the celestial latitude of the native pole
  double phi_p;          // native longitude of the celestial pole, LONPOLE (deg)
  double crpix1, crpix2, cdelt1, cdelt2;
};

__global__ void __launch_bounds__(256) k_pix_wcs_car(int32_t *__restrict__ ipix, const double *__restrict__ ra,
                                                     const double *__restrict__ dec, int64_t n, WcsCar w,
                                                     int64_t ny) {
  const double R2D = 180.0 / M_PI, D2R = M_PI / 180.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const double nyd = (double)ny;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    // the reference hands astropy degrees: ra * 180 / pi
    const double a = __ddiv_rn(__dmul_rn(__ldcs(ra + i), 180.0), M_PI);
    const double d = __ddiv_rn(__dmul_rn(__ldcs(dec + i), 180.0), M_PI);
    double sd, cd, sl, cl;
    sincos(d * D2R, &sd, &cd);
    sincos((a - w.alpha_p) * D2R, &sl, &cl);
    // native spherical coordinates (C&G eq. 5)
    const double xr = sd * w.cos_dp - cd * w.sin_dp * cl;
    const double yr = -cd * sl;
    double phi = w.phi_p + atan2(yr, xr) * R2D;
    if (phi > 180.0) phi -= 360.0;
    else if (phi < -180.0) phi += 360.0;
    double z = sd * w.sin_dp + cd * w.cos_dp * cl;
    z = z > 1.0 ? 1.0 : (z < -1.0 ? -1.0 : z);
    const double theta = asin(z) * R2D;
    // CAR: (x, y) = (phi, theta); pixel (1-based) = crpix + x / cdelt
    const double p1 = w.crpix1 + phi / w.cdelt1;
    const double p2 = w.crpix2 + theta / w.cdelt2;
    const double xp = rint(p1 - 1.0), yp = rint(p2 - 1.0);
    __stcs(ipix + i, trunc_i32(__dadd_rn(__dmul_rn(xp, nyd), yp)));
  }
}

}  // namespace

extern "C" int mk_pix_car(int32_t *ipix, const double *ra, const double *dec, int64_t n, double ra0,
                          double dec0, double pixsize, double cosdec, int64_t ny, int trunc, void *stream) {
  MK_CHECK_ARG(n >= 0 && ny > 0, "mk_pix_car: bad size (n=%lld, ny=%lld)", (long long)n, (long long)ny);
  MK_CHECK_ARG(pixsize != 0.0, "mk_pix_car: pixsize is zero");
  if (n == 0) return MK_OK;
  MK_CHECK_ARG(ipix && ra && dec, "mk_pix_car: null pointer");
  cudaStream_t st = mk::as_stream(stream);
  if (trunc)
    k_pix_car<true><<<mk_grid_fit(k_pix_car<true>, n, 256), 256, 0, st>>>(ipix, ra, dec, n, ra0, dec0, pixsize,
                                                                           cosdec, ny);
  else
    k_pix_car<false><<<mk_grid_fit(k_pix_car<false>, n, 256), 256, 0, st>>>(ipix, ra, dec, n, ra0, dec0, pixsize,
                                                                             cosdec, ny);
  return mk::launch_status("mk_pix_car");
}

extern "C" int mk_pix_wcs_car(int32_t *ipix, const double *ra, const double *dec, int64_t n,
                              const double *wcs6, int64_t ny, void *stream) {
  MK_CHECK_ARG(n >= 0 && ny > 0, "mk_pix_wcs_car: bad size (n=%lld, ny=%lld)", (long long)n, (long long)ny);
  MK_CHECK_ARG(wcs6, "mk_pix_wcs_car: null wcs");
  const double ra0 = wcs6[0], dec0 = wcs6[1];
  MK_CHECK_ARG(dec0 >= -90.0 && dec0 <= 90.0, "mk_pix_wcs_car: crval2 %g outside [-90, 90]", dec0);
  MK_CHECK_ARG(wcs6[4] != 0.0 && wcs6[5] != 0.0, "mk_pix_wcs_car: zero cdelt");
  if (n == 0) return MK_OK;
  MK_CHECK_ARG(ipix && ra && dec, "mk_pix_wcs_car: null pointer");
  // celestial pole for native reference point (0, 0): LONPOLE defaults to 0
  // when crval2 >= 0 (else 180); of the two pole latitudes, LATPOLE = +90
  // picks 90 - crval2 (resp. 90 + crval2); alpha_p follows from C&G eq. 9
  WcsCar w;
  double delta_p;
  if (dec0 >= 0.0) {
    w.phi_p = 0.0;
    delta_p = 90.0 - dec0;
    w.alpha_p = ra0 - 180.0;
  } else {
    w.phi_p = 180.0;
    delta_p = 90.0 + dec0;
    w.alpha_p = ra0;
  }
  w.sin_dp = sin(delta_p * M_PI / 180.0);
  w.cos_dp = cos(delta_p * M_PI / 180.0);
  w.crpix1 = wcs6[2];
  w.crpix2 = wcs6[3];
  w.cdelt1 = wcs6[4];
  w.cdelt2 = wcs6[5];
  cudaStream_t st = mk::as_stream(stream);
  k_pix_wcs_car<<<mk_grid_fit(k_pix_wcs_car, n, 256), 256, 0, st>>>(ipix, ra, dec, n, w, ny);
  return mk::launch_status("mk_pix_wcs_car");
}
