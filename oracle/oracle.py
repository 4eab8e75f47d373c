"""CPU oracle for the minkasi mapmaking hot path.

TEST INFRASTRUCTURE ONLY.  Only tests/, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import this
module, and only as the checker or as the timed CPU baseline.  The product
package (``minkasi_gb300``) never imports it.

Each function restates one piece of the reference's FP64 arithmetic, with the
reference file:line it follows (paths relative to the minkasi project root):

* ``map2tod`` / ``tod2map``  -> minkasi/lib/minkasi.c:131-144 / :97-112
  (through the C restatement in ``oracle/mk_oracle.c``)
* ``dct1``                   -> FFTW REDFT00 as called by
  minkasi/tools/fft.py:290-344 -> minkasi/lib/mkfftw.c:174-212, and its
  scipy fallback minkasi/tools/py_fft.py:254-285 (``scipy.fft.dct(type=1)``)
* ``apply_noise``            -> NoiseSmoothedSVD.apply_noise,
  minkasi/mapmaking/noise.py:680-714
* ``smooth_many_vecs``       -> minkasi/tools/smooth.py:49-78
* ``noise_model``            -> NoiseSmoothedSVD.__init__,
  minkasi/mapmaking/noise.py:604-678
* ``det_weights``            -> NoiseSmoothedSVD.get_det_weights, noise.py:761-772
* ``todvec_dot``             -> Tod.dot / TodVec.dot, minkasi/tods/core.py:649-691,967-1026
* ``make_rhs``               -> TodVec.make_rhs, minkasi/tods/core.py:1028-1047
* ``make_hits``              -> minkasi/mapmaking/tod2map.py:343-400
* ``run_pcg``                -> minkasi/mapmaking/pcg.py:22-238
* ``find_good_fft_lens`` / ``truncate_len`` -> minkasi/tools/py_fft.py:300-395,
  minkasi/tods/processing.py:648-682
* ``pix_car`` / ``pix_car_trunc`` -> SkyMapCar.pix_from_radec,
  minkasi/maps/skymap.py:958-984 / radec2pix_car, minkasi/maps/utils.py:178-216
* ``polmap2tod`` / ``tod2polmap`` -> minkasi/lib/minkasi.c:146-245 (via
  minkasi/mapmaking/map2tod.py:57-122, tod2map.py:164-215)
* ``pol_invert`` / ``pol_precon_mul`` -> PolMap.invert / PolMap.__mul__,
  minkasi/maps/polmap.py:300-384,624-684
* ``cuts_gather`` / ``cuts_scatter`` -> tod2cuts / cuts2tod, minkasi/lib/minkasi.c:260-284
* ``stripe_edges`` / ``stripes_map2tod`` / ``stripes_tod2map`` -> split_partitioned_vec,
  tsStripes (minkasi/mapmaking/timestream.py:442-531), map2tod_destriped
  (minkasi/mapmaking/map2tod.py:156-190); tod2map_destriped
  (minkasi/mapmaking/tod2map.py:242-269) as the transpose of map2tod_destriped
* ``binned_map2tod`` / ``binned_tod2map`` -> map2tod_binned_det / tod2map_binned_det
  (map2tod.py:195-253, tod2map.py:272-340), the latter as a true histogram
* ``car_wcs`` / ``pix_wcs_car``  -> get_wcs (minkasi/maps/utils.py:13-67) and
  SkyMap.pix_from_radec (minkasi/maps/skymap.py:457-490); astropy's CAR
  world->pixel is restated from the published FITS equations (Calabretta &
  Greisen 2002).  astropy is not installed, so this one is parity unpinned.

Parity of this oracle with the reference itself is pinned by
``tests/test_oracle_golden.py`` against fixtures that
``tests/golden/make_golden.py`` produced by running the reference code.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np
import scipy.fft

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def build() -> str:
    """Compile oracle/mk_oracle.so (gcc + OpenMP) if it is missing or stale."""
    so = os.path.join(_HERE, "mk_oracle.so")
    src = os.path.join(_HERE, "mk_oracle.c")
    if not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE, "mk_oracle.so"], check=True)
    return so


def lib():
    """ctypes handle on the C restatement (built on first use)."""
    global _LIB
    if _LIB is None:
        h = ctypes.CDLL(build())
        vp, i64, i32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
        for name in ("orc_map2tod", "orc_map2tod_f32"):
            getattr(h, name).argtypes = [vp, vp, i64, i64, vp, i32, i32]
            getattr(h, name).restype = None
        h.orc_map2tod_serial.argtypes = [vp, vp, i64, i64, vp, i32]
        for name in ("orc_tod2map", "orc_tod2map_f32"):
            getattr(h, name).argtypes = [vp, vp, i64, i64, vp, i64, i32]
            getattr(h, name).restype = ctypes.c_int
        h.orc_tod2map_serial.argtypes = [vp, vp, i64, i64, vp]
        h.orc_tod2map_atomic.argtypes = [vp, vp, i64, i64, vp, i32]
        h.orc_count_bad_pix.argtypes = [vp, i64, i64]
        h.orc_count_bad_pix.restype = ctypes.c_int64
        h.orc_max_threads.restype = ctypes.c_int
        _LIB = h
    return _LIB


def ref_lib():
    """ctypes handle on oracle/_ref/libminkasi.so (the reference's own C,
    compiled by ``make -C oracle ref``), or None where it was not built."""
    p = os.path.join(_HERE, "_ref", "libminkasi.so")
    if not os.path.exists(p):
        return None
    h = ctypes.CDLL(p)
    vp, i32 = ctypes.c_void_p, ctypes.c_int
    h.map2tod_omp.argtypes = [vp, vp, i32, i32, vp, i32]
    h.tod2map_omp.argtypes = [vp, vp, i32, i32, vp, i32]
    h.tod2map_simple.argtypes = [vp, vp, i32, i32, vp]
    h.set_nthread.argtypes = [i32]
    return h


def _c(a: np.ndarray) -> int:
    assert a.flags.c_contiguous
    return a.ctypes.data


# --------------------------------------------------------------------------
# projections
# --------------------------------------------------------------------------
def map2tod(dat: np.ndarray, map: np.ndarray, ipix: np.ndarray, do_add: bool = True,
            nthread: int = 0) -> None:
    """dat (+)= map.flat[ipix]  (minkasi.c:131-144)."""
    assert ipix.dtype == np.int32 and ipix.shape == dat.shape
    ndet, ndata = dat.shape
    if dat.dtype == np.float64:
        assert map.dtype == np.float64
        lib().orc_map2tod(_c(dat), _c(map), ndet, ndata, _c(ipix), int(do_add), nthread)
    else:
        assert dat.dtype == np.float32 and map.dtype == np.float32
        lib().orc_map2tod_f32(_c(dat), _c(map), ndet, ndata, _c(ipix), int(do_add), nthread)


def tod2map(map: np.ndarray, dat: np.ndarray, ipix: np.ndarray, nthread: int = 0) -> None:
    """map.flat[ipix] += dat  (minkasi.c:97-112), deterministic for fixed nthread."""
    assert ipix.dtype == np.int32 and ipix.shape == dat.shape
    ndet, ndata = dat.shape
    fn = lib().orc_tod2map if dat.dtype == np.float64 else lib().orc_tod2map_f32
    assert map.dtype == dat.dtype
    rc = fn(_c(map), _c(dat), ndet, ndata, _c(ipix), map.size, nthread)
    if rc != 0:
        raise MemoryError("oracle tod2map could not allocate its private maps")


def tod2map_serial(map: np.ndarray, dat: np.ndarray, ipix: np.ndarray) -> None:
    """Serial scatter in sample order (minkasi.c:50-55)."""
    ndet, ndata = dat.shape
    lib().orc_tod2map_serial(_c(map), _c(dat), ndet, ndata, _c(ipix))


# --------------------------------------------------------------------------
# DCT-I and the SmoothedSVD noise filter
# --------------------------------------------------------------------------
def dct1(x: np.ndarray, workers: int = 1) -> np.ndarray:
    """Unnormalised DCT-I (FFTW REDFT00) along the last axis:
    X_k = x_0 + (-1)^k x_{n-1} + 2 sum_{j=1}^{n-2} x_j cos(pi j k/(n-1)).
    Same transform the reference's fallback applies row by row
    (py_fft.py:254-285 -> scipy.fft.dct(type=1))."""
    return scipy.fft.dct(np.asarray(x), type=1, axis=-1, workers=workers)


def apply_noise(v: np.ndarray, vT: np.ndarray, mywt: np.ndarray, dat: np.ndarray,
                noisevec: Optional[np.ndarray] = None, workers: int = 1) -> np.ndarray:
    """NoiseSmoothedSVD.apply_noise (noise.py:680-714):
    dd = vT . DCT1(mywt[:, :n] * DCT1(v . dat)), columns 0 and -1 halved,
    with the optional prewhitening division before and after."""
    noisemat = None
    if noisevec is not None:
        noisemat = np.repeat([noisevec], dat.shape[1], axis=0).T
        dat = dat / noisemat
    dat_rot = np.dot(v, dat)
    datft = dct1(dat_rot, workers)
    nn = datft.shape[1]
    datft = datft * mywt[:, :nn]
    dat_rot = dct1(datft, workers)
    dd = np.dot(vT, dat_rot)
    dd[:, 0] = 0.5 * dd[:, 0]
    dd[:, -1] = 0.5 * dd[:, -1]
    if noisemat is not None:
        dd = dd / noisemat
    return dd


def smooth_many_vecs(vecs: np.ndarray, fwhm: float = 20.0) -> np.ndarray:
    """Gaussian smoothing of each row as a DCT-I convolution (smooth.py:49-78)."""
    n = vecs.shape[1]
    x = np.arange(n)
    sig = fwhm / np.sqrt(8 * np.log(2))
    to_conv = np.exp(-0.5 * (x / sig) ** 2)
    tot = to_conv[0] + to_conv[-1] + 2 * to_conv[1:-1].sum()
    to_conv = to_conv / tot
    to_conv_ft = dct1(to_conv)
    xtrans = dct1(vecs)
    xtrans *= to_conv_ft
    back = dct1(xtrans)
    return back / (2 * (n - 1))


def noise_model(dat: np.ndarray, fwhm: float = 50.0, u: Optional[np.ndarray] = None,
                prewhiten: bool = False):
    """NoiseSmoothedSVD.__init__ (noise.py:604-678).  Returns (v, vT, mywt, noisevec).

    ``u`` plays the role of the reference's ``u_in``: when given, vT = inv(v)
    (noise.py:657-663).  When it is None the left singular vectors come from a
    thin SVD, which equals the reference's full-matrices SVD in its ``u``
    factor (the reference's own full SVD needs an nsamp x nsamp matrix) and
    vT = v.T as in the reference."""
    noisevec = None
    if prewhiten:
        noisevec = np.median(np.abs(np.diff(dat, axis=1)), axis=1)
        dat = dat / np.repeat([noisevec], dat.shape[1], axis=0).T
    if u is None:
        uu, _, _ = np.linalg.svd(dat, full_matrices=False)
        v = np.array(uu.T)
        vT = v.T.copy()
    else:
        v = np.array(u.T)
        vT = np.linalg.inv(v)
    dat_rot = np.dot(v, dat)
    dat_trans = dct1(dat_rot)
    spec = smooth_many_vecs(dat_trans ** 2, fwhm)
    spec[:, 1:] = 1.0 / spec[:, 1:]
    spec[:, 0] = 0
    return v, vT, spec, noisevec


def det_weights(v: np.ndarray, vT: np.ndarray, mywt: np.ndarray) -> np.ndarray:
    """NoiseSmoothedSVD.get_det_weights (noise.py:761-772)."""
    mode_wt = np.sum(mywt, axis=1)
    tmp = np.dot(vT, np.dot(np.diag(mode_wt), v))
    return np.diag(tmp).copy() * 2.0


# --------------------------------------------------------------------------
# the operator A = sum_tod P^T N P, the RHS, hits and PCG
# --------------------------------------------------------------------------
@dataclass
class OracleTod:
    ipix: np.ndarray            # (ndet, ndata) int32
    v: np.ndarray               # (ndet, ndet)
    vT: np.ndarray              # (ndet, ndet)
    mywt: np.ndarray            # (ndet, >= ndata)
    dat: Optional[np.ndarray] = None      # dat_calib (ndet, ndata)
    noisevec: Optional[np.ndarray] = None


def todvec_dot(tods: Sequence[OracleTod], x: np.ndarray, workers: int = 1,
               nthread: int = 0) -> np.ndarray:
    """TodVec.dot with one SkyMap (core.py:967-1026 -> Tod.dot :649-691):
    out = sum_tod P^T N P x."""
    out = np.zeros_like(x)
    for t in tods:
        tmp = np.zeros(t.ipix.shape, dtype=x.dtype)
        map2tod(tmp, x, t.ipix, True, nthread)
        tmp = apply_noise(t.v, t.vT, t.mywt, tmp, t.noisevec, workers)
        tod2map(out, np.ascontiguousarray(tmp), t.ipix, nthread)
    return out


def make_rhs(tods: Sequence[OracleTod], npix_shape, workers: int = 1) -> np.ndarray:
    """TodVec.make_rhs (core.py:1028-1047): b = sum_tod P^T N d."""
    b = np.zeros(npix_shape)
    for t in tods:
        dd = apply_noise(t.v, t.vT, t.mywt, t.dat, t.noisevec, workers)
        tod2map(b, np.ascontiguousarray(dd), t.ipix)
    return b


def make_hits(tods: Sequence[OracleTod], npix_shape, do_weights: bool = False) -> np.ndarray:
    """make_hits (tod2map.py:343-400): tod2map of ones (or of per-detector
    weights from det_weights) summed over TODs."""
    hits = np.zeros(npix_shape)
    for t in tods:
        if do_weights:
            w = det_weights(t.v, t.vT, t.mywt)
            tmp = np.outer(w, np.ones(t.ipix.shape[1]))
        else:
            tmp = np.ones(t.ipix.shape)
        tod2map(hits, tmp, t.ipix)
    return hits


def jacobi_from_hits(hits: np.ndarray) -> np.ndarray:
    """precon = 1/hits where hits > 0, else 0
    (examples/minkasi_mpi_example.py:99-105)."""
    p = np.zeros_like(hits)
    ii = hits > 0
    p[ii] = 1.0 / hits[ii]
    return p


def run_pcg(b: np.ndarray, x0: np.ndarray, apply_A, precon: Optional[np.ndarray] = None,
            maxiter: int = 25, history: Optional[List[dict]] = None) -> np.ndarray:
    """run_pcg_wprior without prior (pcg.py:22-200, wrapper :203-238): fixed
    ``maxiter`` iterations, same order of updates, np.sum dots."""
    Ax = apply_A(x0)
    r = b - Ax
    z = precon * r if precon is not None else r.copy()
    p = z.copy()
    zr = float(np.sum(r * z))
    x = x0.copy()
    for i in range(maxiter):
        Ap = apply_A(p)
        pAp = float(np.sum(p * Ap))
        alpha = zr / pAp
        x = x + alpha * p
        r = r + (-alpha) * Ap
        z = precon * r if precon is not None else r.copy()
        zr_new = float(np.sum(r * z))
        beta = zr_new / zr
        p = z + beta * p
        zr = zr_new
        if history is not None:
            history.append({"iter": i, "alpha": alpha, "beta": beta, "zr": zr})
    return x


# --------------------------------------------------------------------------
# TOD length truncation
# --------------------------------------------------------------------------
def _nsphere_vol(npp: int) -> float:
    if npp % 2:
        nn = (npp - 1) / 2
        return 2 ** (nn + 1) * np.pi ** nn / np.prod(np.arange(1, npp + 1, 2))
    nn = npp / 2
    return (np.pi ** nn) / np.prod(np.arange(1, nn + 1))


def find_good_fft_lens(n: int, primes: Sequence[int] = (2, 3, 5, 7)) -> np.ndarray:
    """All products of ``primes`` up to about n, enumerated in log2 space
    (py_fft.py:300-395)."""
    lp = np.log2(np.asarray(primes, dtype=float))
    r = np.log2(n + 0.5)
    out: List[float] = []

    def rec(level: int, lcur: float):
        if level == len(lp) - 1:
            out.extend(np.arange(lcur, r + 1e-3, lp[level]).tolist())
            return
        for fac in np.arange(lcur, r, lp[level]):
            rec(level + 1, fac)

    rec(0, 0.0)
    return np.sort(np.asarray(np.round(2 ** np.asarray(out)), dtype=int))


def truncate_len(ndata: int, primes: Sequence[int] = (2, 3, 5, 7, 11)) -> int:
    """Length that truncate_tod (processing.py:648-682) cuts ndata down to."""
    new = int(find_good_fft_lens(ndata - 1, primes).max()) + 1
    return new if new < ndata else ndata


# ---------------------------------------------------------------- pointing
def pix_car(ra: np.ndarray, dec: np.ndarray, lims, pixsize: float, ny: int,
            cosdec: Optional[float] = None) -> np.ndarray:
    """SkyMapCar.pix_from_radec (minkasi/maps/skymap.py:958-984): x rounded
    half-to-even, y + 0.5, the sum truncated to int32."""
    if cosdec is None:
        cosdec = np.cos(0.5 * (lims[2] + lims[3]))
    xpix = np.round((ra - lims[0]) * cosdec / pixsize)
    ypix = ((dec - lims[2]) / pixsize) + 0.5
    return np.asarray(xpix * ny + ypix, dtype="int32")


def pix_car_trunc(ra: np.ndarray, dec: np.ndarray, lims, pixsize: float, cosdec: float,
                  ny: int) -> np.ndarray:
    """radec2pix_car (minkasi/maps/utils.py:178-216): int(x + 0.5) and
    int(y + 0.5) (truncation toward zero), then xpix * ny + ypix."""
    xs = ((np.ravel(ra) - lims[0]) * cosdec / pixsize + 0.5)
    ys = ((np.ravel(dec) - lims[2]) / pixsize + 0.5)
    xp = np.trunc(xs).astype(np.int64)
    yp = np.trunc(ys).astype(np.int64)
    return (xp * ny + yp).astype(np.int32).reshape(np.shape(ra))


def car_wcs(lims, pixsize: float, ref_equ: bool = False) -> np.ndarray:
    """crval1, crval2, crpix1, crpix2, cdelt1, cdelt2 (degrees) of the CAR WCS
    that get_wcs builds (minkasi/maps/utils.py:47-66; CAR forces cosdec = 1)."""
    cosdec = 1.0
    if ref_equ:
        crval = [0.0, 0.0]
        crpix = [lims[1] / pixsize + 1, -lims[2] / pixsize + 1]
    else:
        crpix = [1.0, 1.0]
        crval = [lims[1] * 180 / np.pi, lims[2] * 180 / np.pi]
    cdelt = [-pixsize / cosdec * 180 / np.pi, pixsize * 180 / np.pi]
    return np.array(crval + crpix + cdelt, dtype=np.float64)


def wcs_car_world2pix(ra_deg: np.ndarray, dec_deg: np.ndarray, w: np.ndarray):
    """1-based pixel coordinates of a CAR WCS (Calabretta & Greisen 2002):
    celestial pole from crval with the defaults LONPOLE = 0 (180 if crval2 <
    0) and LATPOLE = +90 (eqs. 8-10, native reference point (0, 0)), the
    rotation to native (phi, theta) (eq. 5), CAR x = phi, y = theta, then
    p = crpix + x / cdelt."""
    ra0, dec0 = w[0], w[1]
    if dec0 >= 0:
        phi_p, delta_p, alpha_p = 0.0, 90.0 - dec0, ra0 - 180.0
    else:
        phi_p, delta_p, alpha_p = 180.0, 90.0 + dec0, ra0
    d2r = np.pi / 180
    sdp, cdp = np.sin(delta_p * d2r), np.cos(delta_p * d2r)
    sd, cd = np.sin(dec_deg * d2r), np.cos(dec_deg * d2r)
    dl = (ra_deg - alpha_p) * d2r
    sl, cl = np.sin(dl), np.cos(dl)
    phi = phi_p + np.arctan2(-cd * sl, sd * cdp - cd * sdp * cl) / d2r
    phi = np.where(phi > 180, phi - 360, np.where(phi < -180, phi + 360, phi))
    theta = np.arcsin(np.clip(sd * sdp + cd * cdp * cl, -1, 1)) / d2r
    return w[2] + phi / w[4], w[3] + theta / w[5]


def pix_wcs_car(ra: np.ndarray, dec: np.ndarray, w: np.ndarray, ny: int) -> np.ndarray:
    """SkyMap.pix_from_radec (minkasi/maps/skymap.py:457-490) on a CAR WCS."""
    p1, p2 = wcs_car_world2pix(ra * 180 / np.pi, dec * 180 / np.pi, w)
    xpix = np.round(p1 - 1)
    ypix = np.round(p2 - 1)
    return np.asarray(xpix * ny + ypix, dtype="int32")


# ---------------------------------------------------------------- polarization
def polmap2tod(dat: np.ndarray, map: np.ndarray, poltag: str, twogamma: np.ndarray,
               ipix: np.ndarray, do_add: bool = False) -> None:
    """map2tod_iqu_omp / map2tod_qu_omp (minkasi.c:146-174), in place."""
    c, s = np.cos(twogamma), np.sin(twogamma)
    m = map.reshape(-1, map.shape[-1])[ipix]
    if poltag == "IQU":
        v = m[..., 0] + m[..., 1] * c + m[..., 2] * s
    elif poltag == "QU":
        v = m[..., 0] * c + m[..., 1] * s
    else:
        raise ValueError(poltag)
    if do_add:
        dat += v
    else:
        dat[:] = v


def tod2polmap(map: np.ndarray, dat: np.ndarray, poltag: str, twogamma: np.ndarray,
               ipix: np.ndarray) -> None:
    """tod2map_{qu,iqu}_simple, tod2map_{qu,iqu}_precon_simple
    (minkasi.c:176-207,231-245), in place, serial order (np.add.at)."""
    c, s = np.cos(twogamma).ravel(), np.sin(twogamma).ravel()
    d = dat.ravel()
    terms = {"IQU": [d, d * c, d * s], "QU": [d * c, d * s],
             "QU_PRECON": [d * c * c, d * s * s, d * s * c],
             "IQU_PRECON": [d, d * c, d * s, d * c * c, d * s * c, d * s * s]}[poltag]
    flat = map.reshape(-1, len(terms))
    p = ipix.ravel()
    for k, t in enumerate(terms):
        np.add.at(flat[:, k], p, t)


def pol_invert(map: np.ndarray, poltag: str, thresh: float = 1e-6) -> np.ndarray:
    """PolMap.invert for QU_PRECON / IQU_PRECON (polmap.py:300-384)."""
    nx, ny = map.shape[:2]
    n = nx * ny
    out = map.copy()
    if poltag == "QU_PRECON":
        t = np.zeros((n, 2, 2))
        t[:, 0, 0] = map[:, :, 0].ravel()
        t[:, 1, 1] = map[:, :, 1].ravel()
        t[:, 0, 1] = t[:, 1, 0] = map[:, :, 2].ravel()
        t = np.linalg.pinv(t, thresh)
        out[:, :, 0], out[:, :, 1], out[:, :, 2] = (t[:, 0, 0].reshape(nx, ny), t[:, 1, 1].reshape(nx, ny),
                                                    t[:, 0, 1].reshape(nx, ny))
        return out
    idx = (((0, 0), 0), ((0, 1), 1), ((0, 2), 2), ((1, 1), 3), ((1, 2), 4), ((2, 2), 5))
    t = np.zeros((n, 3, 3))
    for (i, j), k in idx:
        t[:, i, j] = t[:, j, i] = map[:, :, k].ravel()
    dets = np.linalg.det(t)
    isbad = dets < thresh * dets.max()
    inds = isbad & (t[:, 0, 0] > 0)
    vec = t[inds, 0, 0]
    t = np.linalg.pinv(t, thresh)
    t[isbad] = 0
    t[inds, 0, 0] = 1.0 / vec
    for (i, j), k in idx:
        out[:, :, k] = t[:, i, j].reshape(nx, ny)
    return out


def pol_precon_mul(precon: np.ndarray, map: np.ndarray, poltag: str) -> np.ndarray:
    """PolMap.__mul__ of a PRECON map and a Stokes map (polmap.py:624-684)."""
    a, x = precon, map
    out = np.empty_like(x)
    if poltag == "QU_PRECON":
        out[..., 0] = a[..., 0] * x[..., 0] + a[..., 2] * x[..., 1]
        out[..., 1] = a[..., 2] * x[..., 0] + a[..., 1] * x[..., 1]
    else:
        out[..., 0] = a[..., 0] * x[..., 0] + a[..., 1] * x[..., 1] + a[..., 2] * x[..., 2]
        out[..., 1] = a[..., 1] * x[..., 0] + a[..., 3] * x[..., 1] + a[..., 4] * x[..., 2]
        out[..., 2] = a[..., 2] * x[..., 0] + a[..., 4] * x[..., 1] + a[..., 5] * x[..., 2]
    return out


# ---------------------------------------------------------------- cuts and timestream models
def cuts_gather(vec: np.ndarray, dat: np.ndarray, imap: np.ndarray, do_add: bool = True) -> None:
    """tod2cuts (minkasi.c:260-268)."""
    v = np.ravel(dat)[imap]
    if do_add:
        vec += v
    else:
        vec[:] = v


def cuts_scatter(dat: np.ndarray, vec: np.ndarray, imap: np.ndarray, do_add: bool = True) -> None:
    """cuts2tod (minkasi.c:271-284), serial order."""
    flat = dat.reshape(-1)
    if do_add:
        np.add.at(flat, imap, vec)
    else:
        flat[imap] = vec


def stripe_edges(ndata: int, tvec: np.ndarray, seg_len: int = 500, tthresh: float = 10) -> np.ndarray:
    """tsStripes segment edges: partition_interval / split_partitioned_vec
    (timestream.py:442-483) at the time gaps > tthresh * median dt."""
    def part(start, stop):
        if (stop - start) <= seg_len:
            return np.asarray([start, stop], dtype="int")
        nseg = (stop - start) // seg_len
        sl = (stop - start) // nseg
        nextra = (stop - start) - sl * nseg
        inds = np.arange(start, stop + 1, sl)
        if nextra > 0:
            vec = np.zeros(len(inds), dtype="int")
            vec[1:nextra + 1] = 1
            inds = inds + np.cumsum(vec)
        return inds

    dt = np.median(np.diff(tvec))
    breaks = list(np.where(np.abs(np.diff(tvec)) > tthresh * dt)[0])
    if breaks and breaks[0] == 0:
        breaks = breaks[1:]
    if breaks and breaks[-1] == ndata:
        breaks = breaks[:-1]
    if not breaks:
        return part(0, ndata)
    edges = np.hstack([0, breaks, ndata])
    segs = [part(edges[i], edges[i + 1])[:-1] if i < len(edges) - 2 else part(edges[i], edges[i + 1])
            for i in range(len(edges) - 1)]
    return np.hstack(segs)


def stripes_map2tod(dat: np.ndarray, pars: np.ndarray, lims: np.ndarray, do_add: bool = True) -> None:
    """map2tod_destriped (map2tod.py:156-190)."""
    for s in range(len(lims) - 1):
        if do_add:
            dat[:, lims[s]:lims[s + 1]] += pars[:, s][:, None]
        else:
            dat[:, lims[s]:lims[s + 1]] = pars[:, s][:, None]


def stripes_tod2map(pars: np.ndarray, dat: np.ndarray, lims: np.ndarray, do_add: bool = True) -> None:
    """Segment sums: the transpose of map2tod_destriped (the intent of
    tod2map_destriped, tod2map.py:242-269)."""
    if not do_add:
        pars[:] = 0
    for s in range(len(lims) - 1):
        pars[:, s] += np.sum(dat[:, lims[s]:lims[s + 1]], axis=1)


def _bins(vec: np.ndarray, lims, nbin: int) -> np.ndarray:
    fac = nbin / (lims[1] - lims[0])
    return np.asarray((vec - lims[0]) * fac, dtype="int64")


def binned_map2tod(dat: np.ndarray, pars: np.ndarray, vec: np.ndarray, lims, nbin: int,
                   do_add: bool = True) -> None:
    """map2tod_binned_det (map2tod.py:195-253), vec shared by the detectors."""
    inds = _bins(vec, lims, nbin)
    if not do_add:
        dat[:] = 0
    dat += pars[:, inds]


def binned_tod2map(pars: np.ndarray, dat: np.ndarray, vec: np.ndarray, lims, nbin: int,
                   do_add: bool = True) -> None:
    """Histogram of dat per detector: the transpose of binned_map2tod."""
    inds = _bins(vec, lims, nbin)
    if not do_add:
        pars[:] = 0
    for d in range(dat.shape[0]):
        np.add.at(pars[d], inds, dat[d])
