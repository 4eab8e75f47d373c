"""Generate the golden fixtures in tests/golden/*.npz by running the REFERENCE
minkasi code (its Python + its own C library compiled from source) on small
seeded inputs.  Run here, where the reference tree is mounted:

    python tests/golden/make_golden.py

Every fixture stores its inputs and the reference's outputs, so the tests
(oracle and GPU) need neither the reference nor this script at run time.

Reference entry points exercised (paths in the minkasi project):
  map2tod            minkasi/mapmaking/map2tod.py:19-54  -> minkasi/lib/minkasi.c:116-144
  tod2map_omp/simple minkasi/mapmaking/tod2map.py:29-128 -> minkasi/lib/minkasi.c:50-112
  fft_r2r            minkasi/tools/py_fft.py:254-285 (scipy DCT-I, the shipped default)
  NoiseSmoothedSVD   minkasi/mapmaking/noise.py:584-772
  smooth_many_vecs   minkasi/tools/smooth.py:49-78
  Tod / TodVec.dot / make_rhs   minkasi/tods/core.py:517-691,967-1047
  make_hits          minkasi/mapmaking/tod2map.py:343-400
  run_pcg            minkasi/mapmaking/pcg.py:22-238
  truncate_tod / find_good_fft_lens  minkasi/tods/processing.py:648-682, minkasi/tools/py_fft.py:364-395
  SkyMapCar.pix_from_radec  minkasi/maps/skymap.py:958-984
  radec2pix_car      minkasi/maps/utils.py:178-216 (its pure-Python path: numba is absent)
  CutsCompact / tsStripes / tsBinnedAz  minkasi/tods/cuts.py:201-490,
                     minkasi/mapmaking/timestream.py:442-560, map2tod.py:156-253, tod2map.py:242-340
  polmap2tod / tod2polmap / PolMap  minkasi/mapmaking/map2tod.py:57-122, tod2map.py:164-215,
                     minkasi/maps/polmap.py:273-684 -> minkasi/lib/minkasi.c:146-245

    python tests/golden/make_golden.py [case ...]   # default: every case
"""
import contextlib
import io
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import ref_import  # noqa: E402

mk = ref_import.import_reference()
from minkasi.mapmaking import map2tod as ref_m2t  # noqa: E402
from minkasi.mapmaking import tod2map as ref_t2m  # noqa: E402
from minkasi.mapmaking.noise import NoiseSmoothedSVD  # noqa: E402
from minkasi.mapmaking.pcg import run_pcg  # noqa: E402
from minkasi.maps import Mapset, SkyMap  # noqa: E402
from minkasi.tods import Tod, TodVec  # noqa: E402
from minkasi.tods import processing  # noqa: E402
from minkasi.tools import py_fft, smooth  # noqa: E402


def quiet(fn, *a, **k):
    with contextlib.redirect_stdout(io.StringIO()):
        return fn(*a, **k)


def save(name, **arrs):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **arrs)
    print(f"wrote {name}: {os.path.getsize(path)/1024:.1f} KiB")


def bare_skymap(nx, ny):
    """A SkyMap without astropy: the attributes SkyMap.map2tod/tod2map/dot/
    axpy/copy/__mul__ read (skymap.py:400-440,542-609,651-666,724-740)."""
    m = SkyMap.__new__(SkyMap)
    m.nx, m.ny = nx, ny
    m.map = np.zeros((nx, ny))
    m.caches = None
    m.tag = "ipix"
    m.purge_pixellization = False
    return m


def synth_tod(rng, ndet, ndata, nx, ny, cm_amp=3.0, knee_frac=0.02):
    """Small daisy-like pointing + white / 1-f / common-mode noise."""
    t = np.arange(ndata)
    r = 0.4 * min(nx, ny) * np.sin(2 * np.pi * t / 611.0 + rng.uniform(0, 6))
    th = 2 * np.pi * t / 1777.0 + rng.uniform(0, 6)
    offs = rng.uniform(-1.5, 1.5, size=(ndet, 2))
    x = nx / 2 + r * np.cos(th) + offs[:, :1]
    y = ny / 2 + r * np.sin(th) + offs[:, 1:]
    x = np.clip(np.round(x), 0, nx - 1)
    y = np.clip(np.round(y), 0, ny - 1)
    ipix = np.asarray(x * ny + y, dtype=np.int32)
    white = rng.standard_normal((ndet, ndata))
    f = np.fft.rfftfreq(ndata)
    f[0] = f[1]
    amp = np.sqrt(1 + (knee_frac / f) ** 2)
    red = np.fft.irfft(np.fft.rfft(rng.standard_normal((ndet, ndata))) * amp, n=ndata)
    cm = cm_amp * np.fft.irfft(np.fft.rfft(rng.standard_normal(ndata)) * amp, n=ndata)
    return ipix, white + red + cm[None, :]


def case_proj(rng):
    ndet, ndata, nx, ny = 7, 1001, 37, 23
    npix = nx * ny
    ipix = rng.integers(0, npix, size=(ndet, ndata)).astype(np.int32)
    ipix[0, 0], ipix[-1, -1] = 0, npix - 1
    # runs of repeated pixels, as a slow scan produces
    ipix[3] = np.repeat(rng.integers(0, npix, size=ndata // 7 + 1), 7)[:ndata]
    dat = rng.standard_normal((ndet, ndata))
    map_ = rng.standard_normal((nx, ny))
    d_add = dat.copy()
    ref_m2t.map2tod(d_add, map_, ipix, do_add=True, do_omp=True)
    d_set = dat.copy()
    ref_m2t.map2tod(d_set, map_, ipix, do_add=False, do_omp=True)
    d_add_s = dat.copy()
    ref_m2t.map2tod(d_add_s, map_, ipix, do_add=True, do_omp=False)
    m_omp = map_.copy()
    quiet(ref_t2m.tod2map_omp, m_omp, dat, ipix)
    m_simple = map_.copy()
    quiet(ref_t2m.tod2map_simple, m_simple, dat, ipix)
    save("proj.npz", ipix=ipix, dat=dat, map=map_, map2tod_add=d_add, map2tod_set=d_set,
         map2tod_add_simple=d_add_s, tod2map_omp=m_omp, tod2map_simple=m_simple)


def case_dct(rng):
    out = {}
    for i, shape in enumerate([(3, 2), (2, 3), (4, 17), (4, 257), (3, 1000), (5, 1025), (1, 4097)]):
        x = rng.standard_normal(shape)
        out[f"x{i}"] = x
        out[f"y{i}"] = py_fft.fft_r2r(x)
    v = rng.standard_normal(513)
    out["vec_x"], out["vec_y"] = v, py_fft.fft_r2r(v)
    s = np.abs(rng.standard_normal((3, 600))) + 0.1
    out["smooth_x"], out["smooth_y"] = s, smooth.smooth_many_vecs(s, 50.0)
    save("dct.npz", **out)


def case_noise(rng):
    ndet, ndata = 10, 1025
    _, dat = synth_tod(rng, ndet, ndata, 16, 16)
    nm = quiet(NoiseSmoothedSVD, dat, fwhm=50.0)
    nm_pw = quiet(NoiseSmoothedSVD, dat, fwhm=50.0, prewhiten=True)
    u_thin, _, _ = np.linalg.svd(dat, full_matrices=False)
    nm_u = quiet(NoiseSmoothedSVD, dat, fwhm=50.0, u_in=u_thin)
    x = rng.standard_normal((ndet, ndata))
    x_short = rng.standard_normal((ndet, 700))
    save("noise.npz", dat=dat, x=x, x_short=x_short,
         v=nm.v, vT=nm.vT, mywt=nm.mywt, dd=nm.apply_noise(x), dd_short=nm.apply_noise(x_short),
         detw=nm.get_det_weights(),
         pw_v=nm_pw.v, pw_vT=nm_pw.vT, pw_mywt=nm_pw.mywt, pw_noisevec=nm_pw.noisevec,
         pw_dd=nm_pw.apply_noise(x),
         u_thin=u_thin, u_v=nm_u.v, u_vT=nm_u.vT, u_mywt=nm_u.mywt, u_dd=nm_u.apply_noise(x))


def case_solve(rng):
    nx, ny = 20, 24
    shapes = [(8, 1537), (6, 1201)]
    todvec = TodVec()
    store = {}
    for k, (ndet, ndata) in enumerate(shapes):
        ipix, noise = synth_tod(rng, ndet, ndata, nx, ny)
        sky = np.exp(-((np.arange(nx)[:, None] - nx / 2) ** 2 + (np.arange(ny)[None, :] - ny / 2) ** 2) / 18.0)
        dat = np.ascontiguousarray(sky.ravel()[ipix] * 5.0 + noise)
        info = {"dat_calib": dat, "ipix": ipix}
        tod = Tod(info)
        quiet(tod.set_noise, NoiseSmoothedSVD)
        quiet(todvec.add_tod, tod)
        t = todvec.tods[-1]
        store[f"t{k}_ipix"], store[f"t{k}_dat"] = ipix, dat
        store[f"t{k}_v"], store[f"t{k}_vT"], store[f"t{k}_mywt"] = t.noise.v, t.noise.vT, t.noise.mywt
    m = bare_skymap(nx, ny)
    hits = quiet(ref_t2m.make_hits, todvec, m)
    whits = quiet(ref_t2m.make_hits, todvec, m, do_weights=True)
    mapset = Mapset()
    mapset.add_map(m)
    rhs = mapset.copy()
    quiet(todvec.make_rhs, rhs)
    xr = mapset.copy()
    xr.maps[0].map[:] = rng.standard_normal((nx, ny))
    ax = quiet(todvec.dot, xr)
    x0 = rhs.copy()
    x0.clear()
    precon = mapset.copy()
    tmp = hits.map.copy()
    ii = tmp > 0
    tmp[ii] = 1.0 / tmp[ii]
    precon.maps[0].map[:] = tmp
    xs = quiet(run_pcg, rhs, x0, todvec, precon, maxiter=8)
    save("solve.npz", nx=nx, ny=ny, ntod=len(shapes), hits=hits.map, whits=whits.map,
         rhs=rhs.maps[0].map, xr=xr.maps[0].map, Axr=ax.maps[0].map, precon=tmp,
         pcg8=xs.maps[0].map, **store)


def case_lens():
    ndata = np.array([1000, 1025, 2049, 65536, 131072, 200001, 262144, 300000, 450001, 524288,
                      600000, 50000, 123457, 499999])
    new = []
    for n in ndata:
        info = {"dat_calib": np.zeros((1, int(n)), dtype=np.float32)}
        quiet(processing.truncate_tod, info)
        new.append(info["dat_calib"].shape[1])
    good = py_fft.find_good_fft_lens(1000, [2, 3, 5, 7, 11])
    save("lens.npz", ndata=ndata, truncated=np.array(new), good1000=good)


def case_pointing():
    """Pixel indices of SkyMapCar.pix_from_radec and radec2pix_car for
    pointings inside and around the map limits, north and south of the
    equator (points off the map exercise truncation toward zero)."""
    from minkasi.maps import utils as map_utils
    from minkasi.maps.skymap import SkyMapCar
    rng = np.random.default_rng(11)
    arcsec = np.pi / 180 / 3600
    out = {}
    for k, (ra_c, dec_c) in enumerate(((3.5, 0.31), (0.7, -0.42))):
        pixsize = 2.0 * arcsec
        half = 600 * arcsec
        lims = np.array([ra_c - half, ra_c + half, dec_c - half, dec_c + half])
        cosdec = np.cos(0.5 * (lims[2] + lims[3]))
        ny = int((lims[3] - lims[2]) / pixsize) + 3
        ra = ra_c + rng.uniform(-1.1, 1.1, size=(6, 1500)) * half / cosdec
        dec = dec_c + rng.uniform(-1.1, 1.1, size=(6, 1500)) * half
        m = SkyMapCar.__new__(SkyMapCar)
        m.lims, m.pixsize, m.ny, m.cosdec = lims, pixsize, ny, None
        car = m.pix_from_radec(ra, dec)
        trunc = np.zeros(ra.size, dtype=np.int32)
        map_utils.radec2pix_car(ra, dec, trunc, lims, pixsize, cosdec, ny)
        out.update({f"c{k}_ra": ra, f"c{k}_dec": dec, f"c{k}_lims": lims, f"c{k}_pixsize": pixsize,
                    f"c{k}_ny": ny, f"c{k}_cosdec": m.cosdec, f"c{k}_car": car,
                    f"c{k}_trunc": trunc.reshape(ra.shape)})
    save("pointing.npz", ncase=2, **out)


def bare_polmap(nx, ny, poltag):
    """A PolMap without astropy: the attributes its projections, make_hits,
    copy, set_polstate, invert and __mul__ read (polmap.py:197-684)."""
    from minkasi.maps.polmap import PolMap
    m = PolMap.__new__(PolMap)
    m.nx, m.ny, m.tag, m.purge_pixellization, m.caches = nx, ny, "ipix", False, None
    quiet(m.set_polstate, poltag)
    return m


def case_pol():
    """PolMap projections through the reference's own C (polmap2tod /
    tod2polmap -> minkasi.c:146-245), make_hits on IQU and QU maps, the
    preconditioner inversion and the PRECON x map product."""
    from minkasi.mapmaking.map2tod import polmap2tod
    from minkasi.mapmaking.tod2map import make_hits, tod2polmap
    rng = np.random.default_rng(23)
    nx, ny, ndet, ndata = 20, 17, 6, 1000
    walk = np.cumsum(rng.integers(-1, 2, size=(ndet, ndata)), axis=1) // 4
    ipix = np.mod(walk + rng.integers(0, nx * ny, size=(ndet, 1)), nx * ny).astype(np.int32)
    twogamma = rng.uniform(0, 2 * np.pi, size=(ndet, ndata))
    dat = rng.standard_normal((ndet, ndata))
    out = {"ipix": ipix, "twogamma": twogamma, "dat": dat, "nx": nx, "ny": ny}
    for tag, npol in (("IQU", 3), ("QU", 2)):
        mp = rng.standard_normal((nx, ny, npol))
        out[f"map_{tag}"] = mp
        for add in (0, 1):
            d = dat.copy()
            polmap2tod(d, mp, tag, twogamma, ipix, do_add=bool(add))
            out[f"m2t_{tag}_{add}"] = d
    for tag, npol in (("IQU", 3), ("QU", 2), ("QU_PRECON", 3), ("IQU_PRECON", 6)):
        m0 = rng.standard_normal((nx, ny, npol))
        out[f"t2m_in_{tag}"] = m0.copy()
        tod2polmap(m0, dat, tag, twogamma, ipix)
        out[f"t2m_{tag}"] = m0
    tods = TodVec()
    for k in range(2):
        info = {"dat_calib": dat * (k + 1), "ipix": np.roll(ipix, 7 * k, axis=1).copy(),
                "twogamma_saved": np.roll(twogamma, 3 * k, axis=1).copy()}
        tods.add_tod(Tod(info))
        out[f"hits_t{k}_ipix"] = info["ipix"]
        out[f"hits_t{k}_twogamma"] = info["twogamma_saved"]
    for tag in ("IQU", "QU"):
        h = quiet(make_hits, tods, bare_polmap(nx, ny, tag))
        out[f"hits_{tag}"] = h.map.copy()
        inv = h.copy()
        quiet(inv.invert)
        out[f"inv_{tag}"] = inv.map.copy()
        x = bare_polmap(nx, ny, tag)
        x.map[:] = rng.standard_normal(x.map.shape)
        out[f"mulx_{tag}"] = x.map.copy()
        out[f"mul_{tag}"] = (inv * x).map.copy()
    save("pol.npz", **out)


def case_tsmodel():
    """CutsCompact (tod2cuts / cuts2tod through the reference's C), the
    destriper (tsStripes segment edges, map2tod_destriped,
    set_prior_from_corr, apply_prior) and the binned model
    (map2tod_binned_det, tod2map_binned_det)."""
    from minkasi.mapmaking import map2tod as m2t
    from minkasi.mapmaking import tod2map as t2m
    from minkasi.mapmaking.timestream import tsStripes
    from minkasi.tods.cuts import CutsCompact
    rng = np.random.default_rng(31)
    ndet, ndata = 5, 3000
    dat = rng.standard_normal((ndet, ndata))
    out = {"dat": dat}
    # cuts: a mask with short runs of False per detector
    mask = rng.random((ndet, ndata)) > 0.02
    mask = mask & np.roll(mask, 1, axis=1) & np.roll(mask, 2, axis=1)
    tod = Tod({"dat_calib": dat.copy(), "fname": "t0"})
    cc = quiet(CutsCompact, tod)
    cc.cuts_from_array(mask)
    quiet(cc.get_imap)
    cc.tod2map(tod, dat)
    out.update(cut_mask=mask, cut_imap=cc.imap, cut_map=cc.map.copy())
    cc.map[:] = rng.standard_normal(cc.map.size)
    out["cut_vals"] = cc.map.copy()
    for add in (0, 1):
        d = dat.copy()
        cc.map2tod(tod, d, do_add=bool(add))
        out[f"cut_m2t_{add}"] = d
    # stripes: a time vector with two gaps
    ctime = np.arange(ndata) * 0.01
    ctime[1100:] += 5.0
    ctime[2400:] += 3.0
    tod_s = Tod({"dat_calib": dat.copy(), "fname": "t0", "ctime": ctime})
    st = tsStripes(tod_s, seg_len=170)
    pars = rng.standard_normal(st.params.shape)
    out.update(ctime=ctime, stripe_inds=np.asarray(st.inds), stripe_pars=pars)
    for add in (0, 1):
        d = dat.copy()
        m2t.map2tod_destriped(d, pars, st.inds, do_add=bool(add))
        out[f"stripe_m2t_{add}"] = d
    # tod2map_destriped raises on numpy's path (an (ndet, 1) operand added
    # into an (ndet,) slice), so it yields no fixture; its transpose
    # relation with map2tod_destriped is what the tests check
    corr = np.abs(rng.standard_normal((ndet, st.nseg + 7))) + 0.1
    st.set_prior_from_corr(corr, thresh=0.5)
    out.update(stripe_corr=corr, stripe_prior=st.params.copy())
    x = tsStripes(tod_s, seg_len=170)
    x.params = rng.standard_normal(x.params.shape)
    ax = tsStripes(tod_s, seg_len=170)
    ax.params = rng.standard_normal(ax.params.shape)
    out.update(stripe_x=x.params.copy(), stripe_ax0=ax.params.copy())
    st.apply_prior(x, ax)
    out["stripe_ax"] = ax.params
    # binned: azimuth shared by the detectors
    az = np.mod(0.3 + np.cumsum(np.abs(rng.standard_normal(ndata))) * 0.01, 2 * np.pi)
    nbin = 37
    bpars = rng.standard_normal((ndet, nbin))
    out.update(az=az, bin_pars=bpars, nbin=nbin)
    for add in (0, 1):
        d = dat.copy()
        m2t.map2tod_binned_det(d, bpars, az, (0, 2 * np.pi), nbin, do_add=bool(add))
        out[f"bin_m2t_{add}"] = d
    # the reference's tod2map_binned_det; it agrees with a histogram on the
    # bins that a single sample hits
    az1 = np.sort(rng.uniform(0, 2 * np.pi, size=ndata))
    nbin1 = 100000
    p1 = np.zeros((ndet, nbin1))
    t2m.tod2map_binned_det(dat, p1, az1, (0, 2 * np.pi), nbin1, do_add=True)
    out.update(az_unique=az1, nbin_unique=nbin1, bin_t2m_unique=p1)
    save("tsmodel.npz", **out)


CASES = {"proj": case_proj, "dct": case_dct, "noise": case_noise, "solve": case_solve}

if __name__ == "__main__":
    want = sys.argv[1:]
    if not want or any(w in CASES for w in want):
        # these share one generator, so they are made together, in order
        rng = np.random.default_rng(0)
        for name, fn in CASES.items():
            fn(rng)
    if not want or "lens" in want:
        case_lens()
    if not want or "pointing" in want:
        case_pointing()
    if not want or "pol" in want:
        case_pol()
    if not want or "tsmodel" in want:
        case_tsmodel()
