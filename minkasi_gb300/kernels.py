"""Tensor-level wrappers over the libmkgpu C ABI.

Every function takes CUDA torch tensors (C-contiguous, float64 or float32 data,
int32 pixel indices), launches on torch's current stream, and raises
``MkError`` on a non-zero status.  There is no CPU path: a CPU tensor is an
error, and so is a missing library.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Tuple

import torch

from . import _lib
from ._lib import MK_F32, MK_F64, check

_DT = {torch.float64: MK_F64, torch.float32: MK_F32}


def lib():
    return _lib.load()


def _stream() -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t: Optional[torch.Tensor]):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _dev(t: torch.Tensor, name: str) -> None:
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor (no CPU fallback)")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be C-contiguous")


def _dev_or_pinned(t: torch.Tensor, name: str) -> None:
    """A CUDA tensor, or a pinned host tensor that the kernel reads in place
    (zero copy: with unified addressing a pinned host pointer is valid on the
    device, and on a Grace-Blackwell node the reads travel over NVLink-C2C)."""
    if not (t.is_cuda or (t.device.type == "cpu" and t.is_pinned())):
        raise ValueError(f"{name} must be a CUDA tensor or a pinned host tensor (no CPU fallback)")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be C-contiguous")


def dtype_code(t: torch.Tensor) -> int:
    try:
        return _DT[t.dtype]
    except KeyError:
        raise TypeError(f"unsupported dtype {t.dtype}; use float64 or float32") from None


def _ipix(ipix: torch.Tensor, shape) -> None:
    _dev(ipix, "ipix")
    if ipix.dtype != torch.int32:
        raise TypeError("ipix must be int32 (the reference's pixel index type)")
    if ipix.numel() != int(torch.Size(shape).numel()):
        raise ValueError(f"ipix has {ipix.numel()} entries, data has {torch.Size(shape).numel()}")


def _nd(t: torch.Tensor):
    if t.dim() == 2:
        return t.shape[0], t.shape[1]
    return 1, t.numel()


# ---------------------------------------------------------------------------
# projections
# ---------------------------------------------------------------------------
def map2tod(dat: torch.Tensor, map: torch.Tensor, ipix: torch.Tensor, do_add: bool = True) -> None:
    """dat (+)= map.flat[ipix]  (mk_map2tod; minkasi.c:131-144)."""
    _dev(dat, "dat"), _dev(map, "map"), _ipix(ipix, dat.shape)
    if map.dtype != dat.dtype:
        raise TypeError("map and dat must have the same dtype")
    ndet, ndata = _nd(dat)
    check(lib().mk_map2tod(_p(dat), _p(map), _p(ipix), ndet, ndata, map.numel(), dtype_code(dat),
                           int(bool(do_add)), _stream()), "map2tod")


def tod2map(map: torch.Tensor, dat: torch.Tensor, ipix: torch.Tensor) -> None:
    """map.flat[ipix] += dat with warp-aggregated atomics (mk_tod2map).
    ``dat`` may be a pinned host tensor, read in place by the kernel."""
    _dev_or_pinned(dat, "dat"), _dev(map, "map"), _ipix(ipix, dat.shape)
    if map.dtype != dat.dtype:
        raise TypeError("map and dat must have the same dtype")
    ndet, ndata = _nd(dat)
    check(lib().mk_tod2map(_p(map), _p(dat), _p(ipix), ndet, ndata, map.numel(), dtype_code(dat),
                           _stream()), "tod2map")


def tod2map_staged(map: torch.Tensor, dat: torch.Tensor, ipix: torch.Tensor) -> None:
    """map.flat[ipix] += dat, streams staged through shared memory by bulk
    copies (mk_tod2map_staged).  Device tensors, 16-byte aligned."""
    _dev(dat, "dat"), _dev(map, "map"), _ipix(ipix, dat.shape)
    if map.dtype != dat.dtype:
        raise TypeError("map and dat must have the same dtype")
    ndet, ndata = _nd(dat)
    check(lib().mk_tod2map_staged(_p(map), _p(dat), _p(ipix), ndet, ndata, map.numel(),
                                  dtype_code(dat), _stream()), "tod2map_staged")


def tod2map_status() -> int:
    """1 if a staged tod2map kernel stopped on a timed-out wait since the last call."""
    code = ctypes.c_int(0)
    check(lib().mk_tod2map_status(ctypes.byref(code), _stream()), "tod2map_status")
    return int(code.value)


def _radec(ra: torch.Tensor, dec: torch.Tensor, out: Optional[torch.Tensor]) -> torch.Tensor:
    _dev(ra, "ra"), _dev(dec, "dec")
    if ra.dtype != torch.float64 or dec.dtype != torch.float64:
        raise TypeError("ra and dec must be float64 (radians)")
    if ra.shape != dec.shape:
        raise ValueError("ra and dec must have the same shape")
    if out is None:
        out = torch.empty(ra.shape, dtype=torch.int32, device=ra.device)
    else:
        _dev(out, "out")
        if out.dtype != torch.int32 or out.shape != ra.shape:
            raise ValueError("out must be int32 with the shape of ra")
    return out


def pix_car(ra: torch.Tensor, dec: torch.Tensor, ra0: float, dec0: float, pixsize: float,
            cosdec: float, ny: int, trunc: bool = False,
            out: Optional[torch.Tensor] = None) -> torch.Tensor:
    """int32 pixel indices from RA/dec (radians): SkyMapCar.pix_from_radec
    (trunc=False) or radec2pix_car (trunc=True), bit-identical (mk_pix_car)."""
    out = _radec(ra, dec, out)
    check(lib().mk_pix_car(_p(out), _p(ra), _p(dec), ra.numel(), float(ra0), float(dec0),
                           float(pixsize), float(cosdec), int(ny), int(bool(trunc)), _stream()),
          "pix_car")
    return out


def pix_wcs_car(ra: torch.Tensor, dec: torch.Tensor, wcs6, ny: int,
                out: Optional[torch.Tensor] = None) -> torch.Tensor:
    """int32 pixel indices through a CAR WCS given as (crval1, crval2, crpix1,
    crpix2, cdelt1, cdelt2) in degrees (mk_pix_wcs_car)."""
    out = _radec(ra, dec, out)
    w = (ctypes.c_double * 6)(*[float(v) for v in wcs6])
    check(lib().mk_pix_wcs_car(_p(out), _p(ra), _p(dec), ra.numel(), ctypes.cast(w, ctypes.c_void_p),
                               int(ny), _stream()), "pix_wcs_car")
    return out


POL_MODES = {"QU": 1, "IQU": 2, "QU_PRECON": 3, "IQU_PRECON": 4}


def pol_sincos(twogamma: torch.Tensor, dtype: torch.dtype = torch.float64):
    """(cos(twogamma), sin(twogamma)) in ``dtype`` (mk_pol_sincos)."""
    _dev(twogamma, "twogamma")
    if twogamma.dtype != torch.float64:
        raise TypeError("twogamma must be float64")
    c = torch.empty(twogamma.shape, dtype=dtype, device=twogamma.device)
    s = torch.empty_like(c)
    check(lib().mk_pol_sincos(_p(c), _p(s), _p(twogamma), twogamma.numel(), _DT[dtype], _stream()),
          "pol_sincos")
    return c, s


def _pol_args(map: torch.Tensor, ipix: torch.Tensor, angle, n: int):
    _dev(map, "map"), _dev(ipix, "ipix")
    if ipix.dtype != torch.int32 or ipix.numel() != n:
        raise ValueError("ipix must be int32 with one entry per sample")
    if isinstance(angle, tuple):
        c, s = angle
        _dev(c, "cos2g"), _dev(s, "sin2g")
        if c.dtype != map.dtype or s.dtype != map.dtype or c.numel() != n or s.numel() != n:
            raise ValueError("cos2g / sin2g must match the map dtype and the sample count")
        return _p(c), _p(s), None
    _dev(angle, "twogamma")
    if angle.dtype != torch.float64 or angle.numel() != n:
        raise ValueError("twogamma must be float64 with one entry per sample")
    return None, None, _p(angle)


def polmap2tod(dat: torch.Tensor, map: torch.Tensor, mode: str, angle, ipix: torch.Tensor,
               do_add: bool = False) -> None:
    """dat (+)= the QU / IQU projection of a (nx, ny, npol) map (mk_polmap2tod).
    ``angle``: a (cos2g, sin2g) pair of the map's dtype, or float64 twogamma."""
    _dev(dat, "dat")
    if dat.dtype != map.dtype:
        raise TypeError("map and dat must have the same dtype")
    ndet, ndata = _nd(dat)
    c, s, tg = _pol_args(map, ipix, angle, dat.numel())
    npol = lib().mk_pol_npol(POL_MODES[mode])
    check(lib().mk_polmap2tod(_p(dat), _p(map), c, s, tg, _p(ipix), ndet, ndata, map.numel() // npol,
                              POL_MODES[mode], dtype_code(map), int(bool(do_add)), _stream()), "polmap2tod")


def tod2polmap(map: torch.Tensor, dat: Optional[torch.Tensor], mode: str, angle, ipix: torch.Tensor,
               rowval: Optional[torch.Tensor] = None, shape=None) -> None:
    """map += the mode's Stokes weights of dat (mk_tod2polmap).  dat None:
    per-detector ``rowval`` (or 1) for each sample of ``shape`` (hit maps)."""
    if dat is not None:
        _dev(dat, "dat")
        if dat.dtype != map.dtype:
            raise TypeError("map and dat must have the same dtype")
        ndet, ndata = _nd(dat)
    else:
        ndet, ndata = int(shape[0]), int(shape[1])
        if rowval is not None:
            _dev(rowval, "rowval")
            if rowval.dtype != map.dtype or rowval.numel() != ndet:
                raise ValueError("rowval must have one entry per detector and the map's dtype")
    c, s, tg = _pol_args(map, ipix, angle, ndet * ndata)
    npol = lib().mk_pol_npol(POL_MODES[mode])
    check(lib().mk_tod2polmap(_p(map), _p(dat), c, s, tg, _p(ipix), ndet, ndata, map.numel() // npol,
                              POL_MODES[mode], dtype_code(map), _p(rowval), _stream()), "tod2polmap")


def pol_precon_mul(out: torch.Tensor, precon: torch.Tensor, map: torch.Tensor, mode: str) -> None:
    """out = P . map per pixel (mk_pol_precon_mul); mode QU_PRECON or IQU_PRECON."""
    for t, nm in ((out, "out"), (precon, "precon"), (map, "map")):
        _dev(t, nm)
        if t.dtype != map.dtype:
            raise TypeError("out, precon and map must share a dtype")
    npol = lib().mk_pol_npol(POL_MODES[mode])
    npix = precon.numel() // npol
    check(lib().mk_pol_precon_mul(_p(out), _p(precon), _p(map), npix, POL_MODES[mode], dtype_code(map),
                                  _stream()), "pol_precon_mul")


def _i64(t: torch.Tensor, name: str) -> None:
    _dev(t, name)
    if t.dtype != torch.int64:
        raise TypeError(f"{name} must be int64")


def cuts_gather(vec: torch.Tensor, dat: torch.Tensor, imap: torch.Tensor, do_add: bool = True) -> None:
    """vec (+)= dat.flat[imap]  (mk_cuts_gather; tod2cuts)."""
    _dev(vec, "vec"), _dev(dat, "dat"), _i64(imap, "imap")
    if vec.dtype != dat.dtype or vec.numel() != imap.numel():
        raise ValueError("vec must match dat's dtype and have one entry per index")
    check(lib().mk_cuts_gather(_p(vec), _p(dat), _p(imap), imap.numel(), dat.numel(), dtype_code(dat),
                               int(bool(do_add)), _stream()), "cuts_gather")


def cuts_scatter(dat: torch.Tensor, vec: torch.Tensor, imap: torch.Tensor, do_add: bool = True) -> None:
    """dat.flat[imap] (+)= vec  (mk_cuts_scatter; cuts2tod)."""
    _dev(vec, "vec"), _dev(dat, "dat"), _i64(imap, "imap")
    if vec.dtype != dat.dtype or vec.numel() != imap.numel():
        raise ValueError("vec must match dat's dtype and have one entry per index")
    check(lib().mk_cuts_scatter(_p(dat), _p(vec), _p(imap), imap.numel(), dat.numel(), dtype_code(dat),
                                int(bool(do_add)), _stream()), "cuts_scatter")


def _stripes_args(dat, pars, lims):
    _dev(dat, "dat"), _dev(pars, "pars"), _i64(lims, "lims")
    ndet, ndata = _nd(dat)
    nseg = lims.numel() - 1
    if pars.dtype != dat.dtype or pars.numel() != ndet * nseg:
        raise ValueError("pars must be (ndet, nseg) of dat's dtype")
    return ndet, ndata, nseg


def stripes_map2tod(dat: torch.Tensor, pars: torch.Tensor, lims: torch.Tensor, do_add: bool = True) -> None:
    """dat[d, lims[s]:lims[s+1]] (+)= pars[d, s]  (mk_stripes_map2tod)."""
    ndet, ndata, nseg = _stripes_args(dat, pars, lims)
    check(lib().mk_stripes_map2tod(_p(dat), _p(pars), _p(lims), ndet, ndata, nseg, dtype_code(dat),
                                   int(bool(do_add)), _stream()), "stripes_map2tod")


def stripes_tod2map(pars: torch.Tensor, dat: torch.Tensor, lims: torch.Tensor, do_add: bool = True) -> None:
    """pars[d, s] (+)= dat[d, lims[s]:lims[s+1]].sum()  (mk_stripes_tod2map)."""
    ndet, ndata, nseg = _stripes_args(dat, pars, lims)
    check(lib().mk_stripes_tod2map(_p(pars), _p(dat), _p(lims), ndet, ndata, nseg, dtype_code(dat),
                                   int(bool(do_add)), _stream()), "stripes_tod2map")


def _binned_args(dat, pars, vec):
    _dev(dat, "dat"), _dev(pars, "pars"), _dev(vec, "vec")
    if vec.dtype != torch.float64:
        raise TypeError("vec must be float64")
    ndet, ndata = _nd(dat)
    if vec.numel() not in (ndata, ndet * ndata):
        raise ValueError("vec must have ndata or ndet*ndata entries")
    if pars.dtype != dat.dtype or pars.dim() != 2 or pars.shape[0] != ndet:
        raise ValueError("pars must be (ndet, nbin) of dat's dtype")
    return ndet, ndata, pars.shape[1], int(vec.numel() == ndet * ndata and ndet > 1)


def binned_map2tod(dat: torch.Tensor, pars: torch.Tensor, vec: torch.Tensor, lims, do_add: bool = True) -> None:
    """dat[d, t] (+)= pars[d, bin(vec[t])]  (mk_binned_map2tod)."""
    ndet, ndata, nbin, per_det = _binned_args(dat, pars, vec)
    check(lib().mk_binned_map2tod(_p(dat), _p(pars), _p(vec), ndet, ndata, nbin, float(lims[0]), float(lims[1]),
                                  per_det, dtype_code(dat), int(bool(do_add)), _stream()), "binned_map2tod")


def binned_tod2map(pars: torch.Tensor, dat: torch.Tensor, vec: torch.Tensor, lims, do_add: bool = True) -> None:
    """pars[d, b] (+)= sum of dat[d, t] with bin(vec[t]) = b  (mk_binned_tod2map)."""
    ndet, ndata, nbin, per_det = _binned_args(dat, pars, vec)
    check(lib().mk_binned_tod2map(_p(pars), _p(dat), _p(vec), ndet, ndata, nbin, float(lims[0]), float(lims[1]),
                                  per_det, dtype_code(dat), int(bool(do_add)), _stream()), "binned_tod2map")


def tod2map_rows(map: torch.Tensor, ipix: torch.Tensor, w: Optional[torch.Tensor] = None) -> None:
    """map.flat[ipix[d, t]] += w[d] (1 when w is None) -- hit / weight maps."""
    _dev(map, "map"), _dev(ipix, "ipix")
    if ipix.dtype != torch.int32:
        raise TypeError("ipix must be int32")
    ndet, ndata = _nd(ipix)
    if w is not None:
        _dev(w, "w")
        if w.dtype != map.dtype or w.numel() != ndet:
            raise ValueError("w must have one entry per detector and the map's dtype")
    check(lib().mk_tod2map_rows(_p(map), _p(w), _p(ipix), ndet, ndata, map.numel(),
                                dtype_code(map), _stream()), "tod2map_rows")


class FixedScratch:
    """Accumulator scratch for the deterministic fixed-point tod2map."""

    def __init__(self, npix: int, device=None):
        device = device or torch.device("cuda", torch.cuda.current_device())
        self.npix = int(npix)
        nb = int(lib().mk_tod2map_fixed_scratch_bytes(self.npix))
        self.buf = torch.zeros(nb, dtype=torch.uint8, device=device)


def tod2map_fixed(map: torch.Tensor, dat: torch.Tensor, ipix: torch.Tensor, hmax: int,
                  scratch: FixedScratch) -> None:
    """Bitwise-reproducible map.flat[ipix] += dat (mk_tod2map_fixed); hmax
    bounds the number of samples that hit any one pixel."""
    _dev(dat, "dat"), _dev(map, "map"), _ipix(ipix, dat.shape)
    if map.dtype != dat.dtype or scratch.npix != map.numel():
        raise ValueError("tod2map_fixed: dtype or scratch size mismatch")
    ndet, ndata = _nd(dat)
    check(lib().mk_tod2map_fixed(_p(map), _p(dat), _p(ipix), ndet, ndata, map.numel(), int(hmax),
                                 dtype_code(dat), _p(scratch.buf), _stream()), "tod2map_fixed")


def check_pix(ipix: torch.Tensor, npix: int) -> int:
    """Number of pixel indices outside [0, npix) (synchronises the stream)."""
    _dev(ipix, "ipix")
    nbad = ctypes.c_int64(0)
    check(lib().mk_check_pix(_p(ipix), ipix.numel(), int(npix), ctypes.byref(nbad), _stream()),
          "check_pix")
    return int(nbad.value)


class PixPlan:
    """Sorted pixel plan for the deterministic tod2map (mk_pixplan_*)."""

    def __init__(self, ipix: torch.Tensor, npix: int):
        _dev(ipix, "ipix")
        self.npix, self.n = int(npix), ipix.numel()
        h = ctypes.c_void_p()
        check(lib().mk_pixplan_create(ctypes.byref(h), _p(ipix), self.n, self.npix, _stream()),
              "pixplan_create")
        self._h = h

    def tod2map(self, map: torch.Tensor, dat: torch.Tensor) -> None:
        _dev(map, "map"), _dev(dat, "dat")
        if dat.numel() != self.n or map.numel() != self.npix or map.dtype != dat.dtype:
            raise ValueError("dat / map do not match the plan")
        check(lib().mk_tod2map_sorted(_p(map), _p(dat), self._h, dtype_code(dat), _stream()),
              "tod2map_sorted")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().mk_pixplan_destroy(h)
            except Exception:
                pass
            self._h = None


# ---------------------------------------------------------------------------
# DCT-I and apply_noise
# ---------------------------------------------------------------------------
def _workspace(nbytes: int, device) -> torch.Tensor:
    # torch's caching allocator returns 512-byte aligned blocks
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)


def set_dct_engine(engine: int) -> None:
    """Transform used by DCT / noise plans created from now on: 0 (default)
    the four-step shared-memory FFT, in the plan's precision (through
    Bluestein's algorithm when 2(n-1) has a prime factor above 11); 1 cuFFT
    always; 2 the four-step FFT only where 2(n-1) factors into 2, 3, 5, 7,
    11."""
    check(lib().mk_set_dct_engine(int(engine)), "set_dct_engine")


def set_fft4_split(rank: int) -> None:
    """Four-step split for plans created afterwards: 0 = L1 x L2 closest to
    sqrt(L), r = the r-th next closest divisor pair (mk_set_fft4_split)."""
    check(lib().mk_set_fft4_split(int(rank)), "set_fft4_split")


def fft4_split() -> int:
    return int(lib().mk_get_fft4_split())


def dct_engine() -> int:
    return int(lib().mk_get_dct_engine())


def dct_describe(n: int) -> dict:
    """The transform an FP32 DCT / noise plan for rows of length n would use
    under the current engine: {"engine", "L", "L1", "L2"} (host only)."""
    e, L1, L2 = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    L = ctypes.c_int64()
    check(lib().mk_dct1_describe(int(n), ctypes.byref(e), ctypes.byref(L), ctypes.byref(L1), ctypes.byref(L2)),
          "dct_describe")
    return {"engine": e.value, "L": L.value, "L1": L1.value, "L2": L2.value}


class DCT1:
    """Batched unnormalised DCT-I (REDFT00) of (nrow, n) arrays."""

    def __init__(self, nrow: int, n: int, dtype=torch.float64, device=None,
                 workspace: Optional[torch.Tensor] = None):
        self.nrow, self.n, self.dtype = int(nrow), int(n), dtype
        code = _DT[dtype]
        nb = ctypes.c_size_t(0)
        check(lib().mk_dct1_workspace_bytes(self.nrow, self.n, code, ctypes.byref(nb)), "dct1 size")
        self.workspace_bytes = int(nb.value)
        device = device or torch.device("cuda", torch.cuda.current_device())
        self.ws = workspace if workspace is not None else _workspace(self.workspace_bytes, device)
        h = ctypes.c_void_p()
        check(lib().mk_dct1_plan_create(ctypes.byref(h), self.nrow, self.n, code, _p(self.ws),
                                        self.ws.numel()), "dct1 plan")
        self._h = h

    def __call__(self, x: torch.Tensor, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        _dev(x, "x")
        if x.dtype != self.dtype or _nd(x) != (self.nrow, self.n):
            raise ValueError(f"x must be {self.dtype} of shape ({self.nrow}, {self.n})")
        if out is None:
            out = torch.empty_like(x)
        check(lib().mk_dct1_exec(self._h, _p(x), _p(out), _stream()), "dct1")
        return out

    @property
    def engine(self) -> int:
        """0: four-step FFT, 2: four-step FFT through Bluestein, 1: cuFFT."""
        return int(lib().mk_dct1_engine(self._h))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().mk_dct1_plan_destroy(h)
            except Exception:
                pass
            self._h = None


def noise_workspace_bytes(ndet: int, ndata: int, dtype=torch.float64) -> int:
    nb = ctypes.c_size_t(0)
    check(lib().mk_noise_workspace_bytes(int(ndet), int(ndata), _DT[dtype], ctypes.byref(nb)),
          "noise workspace size")
    return int(nb.value)


class NoisePlan:
    """apply_noise for TODs of one (ndet, ndata) shape; the workspace may be
    shared between plans that run on the same stream."""

    def __init__(self, ndet: int, ndata: int, dtype=torch.float64, device=None,
                 workspace: Optional[torch.Tensor] = None):
        self.ndet, self.ndata, self.dtype = int(ndet), int(ndata), dtype
        self.workspace_bytes = noise_workspace_bytes(ndet, ndata, dtype)
        device = device or torch.device("cuda", torch.cuda.current_device())
        self.ws = workspace if workspace is not None else _workspace(self.workspace_bytes, device)
        if self.ws.numel() < self.workspace_bytes:
            raise ValueError("shared workspace too small for this TOD shape")
        h = ctypes.c_void_p()
        check(lib().mk_noise_plan_create(ctypes.byref(h), self.ndet, self.ndata, _DT[dtype],
                                         _p(self.ws), self.ws.numel()), "noise plan")
        self._h = h

    @property
    def engine(self) -> int:
        """0: four-step FFT, 2: four-step FFT through Bluestein, 1: cuFFT."""
        return int(lib().mk_noise_engine(self._h))

    @property
    def split(self) -> Tuple[int, int]:
        """The four-step split L1 x L2 of this plan's transform ((0, 0) for cuFFT)."""
        a, b = ctypes.c_int(0), ctypes.c_int(0)
        check(lib().mk_noise_split(self._h, ctypes.byref(a), ctypes.byref(b)), "noise split")
        return int(a.value), int(b.value)

    def rotate(self, A: torch.Tensor, X: torch.Tensor, out: Optional[torch.Tensor] = None,
               rot_mode: int = 0) -> torch.Tensor:
        """R = A . X for this plan's shape (mk_rotate)."""
        for t, nm in ((A, "A"), (X, "X")):
            _dev(t, nm)
            if t.dtype != self.dtype:
                raise TypeError(f"{nm} must be {self.dtype}")
        if tuple(X.shape) != (self.ndet, self.ndata) or tuple(A.shape) != (self.ndet, self.ndet):
            raise ValueError("rotate: shapes do not match the plan")
        if out is None:
            out = torch.empty_like(X)
        check(lib().mk_rotate(self._h, _p(A), _p(X), _p(out), int(rot_mode), _stream()), "rotate")
        return out

    def status(self) -> int:
        """1 if a tensor-core kernel of this plan timed out since the last call."""
        code = ctypes.c_int(0)
        check(lib().mk_noise_status(self._h, ctypes.byref(code), _stream()), "noise_status")
        return int(code.value)

    def apply(self, v: torch.Tensor, vT: torch.Tensor, mywt: torch.Tensor, dat: torch.Tensor,
              out: Optional[torch.Tensor] = None, rot_mode: int = 0) -> torch.Tensor:
        for t, nm in ((v, "v"), (vT, "vT"), (mywt, "mywt"), (dat, "dat")):
            _dev(t, nm)
            if t.dtype != self.dtype:
                raise TypeError(f"{nm} must be {self.dtype}")
        if tuple(dat.shape) != (self.ndet, self.ndata):
            raise ValueError(f"dat shape {tuple(dat.shape)} != plan ({self.ndet}, {self.ndata})")
        if mywt.dim() != 2 or mywt.shape[0] != self.ndet or mywt.shape[1] < self.ndata:
            raise ValueError("mywt must be (ndet, >= ndata)")
        if out is None:
            out = torch.empty_like(dat)
        check(lib().mk_apply_noise(self._h, _p(v), _p(vT), _p(mywt), mywt.shape[1], _p(dat),
                                   _p(out), int(rot_mode), _stream()), "apply_noise")
        return out

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().mk_noise_plan_destroy(h)
            except Exception:
                pass
            self._h = None


class NoiseGroup:
    """apply_noise in place on many FP32 TODs in one call (mk_noise_group_*):
    one tensor-core launch per detector count for each of the v and vT
    rotations, and each TOD's two DCT-I on its own plan.  ``plans[t]``,
    ``ops[t] = (v, vT, mywt)`` and ``data[t]`` (an (ndet, ndata) float32
    view) are kept referenced for the life of the group."""

    def __init__(self, plans, ops, data):
        n = len(plans)
        if not (n == len(ops) == len(data)) or n == 0:
            raise ValueError("NoiseGroup: one plan, operand triple and data view per TOD")
        for p, (v, vT, w), d in zip(plans, ops, data):
            for t, nm in ((v, "v"), (vT, "vT"), (w, "mywt"), (d, "data")):
                _dev(t, nm)
                if t.dtype != torch.float32:
                    raise TypeError(f"NoiseGroup: {nm} must be float32")
            if tuple(d.shape) != (p.ndet, p.ndata) or not d.is_contiguous():
                raise ValueError("NoiseGroup: data must be contiguous (ndet, ndata) views")
        self._keep = (list(plans), list(ops), list(data))
        vp = ctypes.c_void_p
        arr = lambda xs: (vp * n)(*[x for x in xs])
        h = ctypes.c_void_p()
        ldw = (ctypes.c_int64 * n)(*[int(w.shape[1]) for _, _, w in ops])
        check(lib().mk_noise_group_create(ctypes.byref(h), n, arr([p._h.value for p in plans]),
                                          arr([v.data_ptr() for v, _, _ in ops]),
                                          arr([vT.data_ptr() for _, vT, _ in ops]),
                                          arr([w.data_ptr() for _, _, w in ops]), ldw,
                                          arr([d.data_ptr() for d in data]), _stream()), "noise group")
        self._h = h

    def apply(self) -> None:
        check(lib().mk_noise_group_exec(self._h, _stream()), "noise group exec")

    def status(self) -> int:
        """1 if a tensor-core wait of the group timed out since the last call."""
        code = ctypes.c_int(0)
        check(lib().mk_noise_group_status(self._h, ctypes.byref(code), _stream()), "noise group status")
        return int(code.value)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().mk_noise_group_destroy(h)
            except Exception:
                pass
            self._h = None


# ---------------------------------------------------------------------------
# map algebra and the PCG recurrence
# ---------------------------------------------------------------------------
class Reducer:
    """Owns the FP64 reduction scratch used by dot / pcg kernels."""

    def __init__(self, device=None):
        device = device or torch.device("cuda", torch.cuda.current_device())
        self.scratch = torch.zeros(int(lib().mk_reduce_scratch_bytes()), dtype=torch.uint8,
                                   device=device)

    def dot(self, a: torch.Tensor, b: torch.Tensor, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        _dev(a, "a"), _dev(b, "b")
        if a.dtype != b.dtype or a.numel() != b.numel():
            raise ValueError("dot: operands differ in dtype or size")
        if out is None:
            out = torch.empty((), dtype=torch.float64, device=a.device)
        check(lib().mk_dot(_p(a), _p(b), a.numel(), dtype_code(a), _p(out), _p(self.scratch),
                           _stream()), "dot")
        return out


def axpy(y: torch.Tensor, x: torch.Tensor, alpha: float) -> None:
    _dev(y, "y"), _dev(x, "x")
    check(lib().mk_axpy(_p(y), _p(x), float(alpha), y.numel(), dtype_code(y), _stream()), "axpy")


def mul(out: torch.Tensor, a: torch.Tensor, b: torch.Tensor) -> None:
    _dev(out, "out"), _dev(a, "a"), _dev(b, "b")
    check(lib().mk_mul(_p(out), _p(a), _p(b), out.numel(), dtype_code(out), _stream()), "mul")


def pcg_init(r, z, p, b, Ax, precon, s, reducer: Reducer) -> None:
    check(lib().mk_pcg_init(_p(r), _p(z), _p(p), _p(b), _p(Ax), _p(precon), r.numel(),
                            dtype_code(r), _p(s), _p(reducer.scratch), _stream()), "pcg_init")


def pcg_step_xr(x, r, p, Ap, s, reducer: Reducer) -> None:
    check(lib().mk_pcg_step_xr(_p(x), _p(r), _p(p), _p(Ap), x.numel(), dtype_code(x), _p(s),
                               _p(reducer.scratch), _stream()), "pcg_step_xr")


def pcg_step_zp(z, r, p, s, reducer: Reducer) -> None:
    check(lib().mk_pcg_step_zp(_p(z), _p(r), _p(p), z.numel(), dtype_code(z), _p(s),
                               _p(reducer.scratch), _stream()), "pcg_step_zp")


def pcg_update(x, r, z, p, Ap, precon, s, reducer: Reducer) -> None:
    check(lib().mk_pcg_update(_p(x), _p(r), _p(z), _p(p), _p(Ap), _p(precon), x.numel(),
                              dtype_code(x), _p(s), _p(reducer.scratch), _stream()), "pcg_update")
