"""Device-resident maps: SkyMap and Mapset.

Mirrors the reference's ``minkasi.maps.SkyMap`` (minkasi/maps/skymap.py:38-790)
and ``minkasi.maps.Mapset`` (minkasi/maps/mapset.py:17-231) for the parts the
mapmaking hot path uses.  ``SkyMap.map`` is an (nx, ny) CUDA tensor (float64
by default) instead of a numpy array; numpy arrays are accepted wherever the
reference takes one and are copied to the device.  Every operation runs a
CUDA kernel of libmkgpu: there is no CPU fallback.
"""
from __future__ import annotations

import copy
import math
import os
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import kernels as K
from . import parallel


def default_device() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("minkasi_gb300 needs a CUDA device (no CPU fallback)")
    return torch.device("cuda", torch.cuda.current_device())


def as_device(a, dtype=None, device=None) -> torch.Tensor:
    """numpy / torch -> contiguous CUDA tensor (no copy if already there)."""
    device = device or default_device()
    if isinstance(a, torch.Tensor):
        t = a.to(device=device, dtype=dtype or a.dtype)
    else:
        arr = np.asarray(a)
        t = torch.from_numpy(np.ascontiguousarray(arr)).to(device)
        if dtype is not None:
            t = t.to(dtype)
    return t.contiguous()


class SkyMap:
    """A CAR sky map held on the GPU (minkasi/maps/skymap.py:38-790).

    Parameters follow the reference.  The WCS is the CAR WCS of get_wcs
    (minkasi/maps/utils.py:13-67), kept as (crval1, crval2, crpix1, crpix2,
    cdelt1, cdelt2) in degrees (``self.wcs``; ``mywcs`` may pass such a
    6-sequence).  Pointing -> pixel runs on the GPU (mk_pix_wcs_car), the map
    size follows get_npix (skymap.py:206-234), and pixel indices supplied by
    the caller in ``tod.info[tag]`` take precedence, as in the reference
    (SkyMap.get_pix, skymap.py:492-540).
    """

    def __init__(self, lims=None, pixsize: float = 0.0, proj: str = "CAR", pad: int = 2,
                 square: bool = False, multiple=False, primes=None, cosdec: Optional[float] = None,
                 nx: Optional[int] = None, ny: Optional[int] = None, mywcs=None, tag: str = "ipix",
                 purge_pixellization: bool = False, ref_equ: bool = False,
                 dtype: torch.dtype = torch.float64, device=None):
        if proj != "CAR":
            raise ValueError(f"Unknown projection type, {proj}")
        self.lims = None if lims is None else list(lims)
        self.proj = proj
        self.pad = pad
        self.primes = primes
        self.ref_equ = ref_equ
        self.wcs = None
        if mywcs is not None:
            self.wcs = [float(v) for v in mywcs]
            if len(self.wcs) != 6:
                raise ValueError("mywcs: (crval1, crval2, crpix1, crpix2, cdelt1, cdelt2) in degrees")
            pixsize = self.wcs[5] * np.pi / 180
        elif self.lims is not None and pixsize != 0:
            self.wcs = car_wcs(self.lims, pixsize, ref_equ)
        self.pixsize = float(pixsize)
        self.cosdec = cosdec
        if nx is None or ny is None:
            if self.lims is None or self.wcs is None:
                raise ValueError("SkyMap needs (lims, pixsize) or explicit nx, ny")
            gx, gy = self.get_npix(pad)
            nx = gx if nx is None else nx
            ny = gy if ny is None else ny
        self.nx, self.ny = int(nx), int(ny)
        self.tag = tag
        self.purge_pixellization = purge_pixellization
        self.caches = None
        self.map = torch.zeros((self.nx, self.ny), dtype=dtype, device=device or default_device())

    # ---- construction helpers ------------------------------------------
    @classmethod
    def from_shape(cls, nx: int, ny: int, dtype=torch.float64, device=None, tag: str = "ipix"):
        return cls(nx=nx, ny=ny, dtype=dtype, device=device, tag=tag)

    @property
    def npix(self) -> int:
        return self.nx * self.ny

    @property
    def dtype(self) -> torch.dtype:
        return self.map.dtype

    def get_caches(self):
        """Thread caches are a CPU device of tod2map_cached; nothing to do here."""
        self.caches = None

    def clear_caches(self):
        self.caches = None

    # ---- pointing -------------------------------------------------------
    def get_npix(self, pad: int):
        """nx, ny from the pixel coordinates of the lims corners
        (skymap.py:206-234)."""
        xs, ys = [], []
        for ra, dec in ((0, 2), (0, 3), (1, 2), (1, 3)):
            p1, p2 = car_world2pix(self.lims[ra] * 180 / np.pi, self.lims[dec] * 180 / np.pi, self.wcs)
            xs.append(round_half_even(p1))
            ys.append(round_half_even(p2))
        return int(max(xs) + pad), int(max(ys) + pad)

    def pix_from_radec(self, ra, dec) -> torch.Tensor:
        """int32 pixel indices from RA/dec in radians through the map's CAR
        WCS (SkyMap.pix_from_radec, skymap.py:457-490), on the GPU."""
        if self.wcs is None:
            raise ValueError("this SkyMap has no WCS (built from nx, ny only)")
        ra = as_device(ra, torch.float64)
        dec = as_device(dec, torch.float64)
        return K.pix_wcs_car(ra, dec, self.wcs, self.ny)

    def get_pix(self, tod, savepix: bool = True) -> torch.Tensor:
        """Cached pixellization of ``tod`` (skymap.py:492-540)."""
        if self.tag is not None:
            ipix = tod.get_saved_pix(self.tag)
            if ipix is not None:
                return tod.device_pix(self.tag, self.npix)
        ra, dec = tod.get_radec()
        ipix = self.pix_from_radec(ra, dec)
        if savepix and self.tag is not None:
            tod.save_pixellization(self.tag, ipix)
            return tod.device_pix(self.tag, self.npix)
        return ipix

    # ---- projections ----------------------------------------------------
    def map2tod(self, tod, dat, do_add: bool = True, do_omp: bool = True):
        """Project the map into ``dat`` (skymap.py:542-567).  ``dat`` is a
        CUDA tensor (updated in place) or a numpy array (updated in place
        through a device round trip)."""
        ipix = self.get_pix(tod)
        if isinstance(dat, torch.Tensor):
            K.map2tod(dat, self.map, ipix, do_add)
            return
        d = as_device(dat, self.map.dtype)
        K.map2tod(d, self.map, ipix, do_add)
        np.copyto(dat, d.cpu().numpy())

    def tod2map(self, tod, dat=None, do_add: bool = True, do_omp: bool = True):
        """Accumulate ``dat`` into the map (skymap.py:569-609)."""
        if dat is None:
            dat = tod.get_data()
        if not do_add:
            self.clear()
        ipix = self.get_pix(tod)
        if isinstance(dat, torch.Tensor) and dat.device.type == "cpu" and dat.is_pinned() \
                and dat.dtype == self.map.dtype and dat.is_contiguous():
            # pinned host timestream: chunked copies overlapped with the scatter
            _stager(self.map.device).tod2map(self.map, dat, ipix)
        else:
            d = dat if isinstance(dat, torch.Tensor) else as_device(dat, self.map.dtype)
            if not d.is_cuda:
                d = d.to(self.map.device)
            if d.dtype != self.map.dtype:
                d = d.to(self.map.dtype)
            K.tod2map(self.map, d, ipix)
        if self.purge_pixellization:
            tod.clear_saved_pix(self.tag)

    # ---- vector space ---------------------------------------------------
    def copy(self) -> "SkyMap":
        new = copy.copy(self)
        new.map = self.map.clone()
        new.lims = None if self.lims is None else list(self.lims)
        return new

    def clear(self):
        self.map.zero_()

    def axpy(self, map: "SkyMap", a: float):
        """self.map = self.map + a * map.map (skymap.py:428-440)."""
        K.axpy(self.map, map.map, float(a))

    def assign(self, arr):
        assert arr.shape[0] == self.nx and arr.shape[1] == self.ny
        self.map.copy_(as_device(arr, self.map.dtype))

    def dot(self, map: "SkyMap") -> float:
        """sum(self.map * map.map) accumulated in FP64 (skymap.py:651-666)."""
        return float(_reducer(self.map.device).dot(self.map, map.map).item())

    def __mul__(self, map: "SkyMap") -> "SkyMap":
        """Elementwise product (skymap.py:724-740)."""
        new = map.copy()
        K.mul(new.map, self.map, map.map)
        return new

    def invert(self):
        """map = 1/map where map != 0 (skymap.py:785-790)."""
        m = self.map
        nz = m.abs() > 0
        m[nz] = 1.0 / m[nz]

    def mpi_reduce(self, chunksize: float = 1e5):
        """Sum the map over ranks (skymap.py:742-783); a no-op on one rank."""
        parallel.allreduce_(self.map)

    def write(self, fname: str = "map.fits"):
        """Write the map as a FITS image, transposed, with its CAR WCS in the
        header (skymap.py:705-722), through minkasi_gb300.fits; a name ending
        in .npy saves the untransposed array with numpy instead."""
        from . import fits
        if fname.endswith(".npy"):
            os.makedirs(os.path.dirname(os.path.abspath(fname)), exist_ok=True)
            np.save(fname, self.map.detach().cpu().numpy())
            return
        cards = fits.car_header(self.wcs) if self.wcs is not None else []
        fits.write_image(fname, self.map.detach().cpu().numpy().T, cards)

    def to_numpy(self) -> np.ndarray:
        return self.map.detach().cpu().numpy()


class HostStager:
    """Host -> device staging of timestreams in pinned host memory.

    A timestream is cut into chunks of CHUNK samples.  Each chunk is copied on
    a dedicated copy stream into one of two device buffers, and the scatter of
    the chunk runs on the caller's stream as soon as its copy lands, while the
    next chunk is already copying.  Consecutive calls (one per TOD) continue
    the same two-buffer ring, so the copy engine stays busy across TODs and a
    pass over host-resident TODs runs at the host -> device copy rate.
    Ordering is by CUDA events only; the host never waits, so, as with any
    non-blocking copy, the caller must not overwrite the host buffer before
    the stream work of the call has run.
    """

    CHUNK = 1 << 24  # samples (128 MB of FP64 per buffer)

    def __init__(self, device):
        self.device = torch.device(device)
        self.copy_stream = torch.cuda.Stream(self.device)
        self.bufs = {}
        self.free = [None, None]  # event: the scatter that last read buffer i is done
        self.turn = 0

    def _buffers(self, dtype):
        if dtype not in self.bufs:
            self.bufs[dtype] = [torch.empty(self.CHUNK, dtype=dtype, device=self.device) for _ in range(2)]
            self.free = [None, None]
        return self.bufs[dtype]

    def tod2map(self, map: torch.Tensor, host: torch.Tensor, ipix: torch.Tensor) -> None:
        bufs = self._buffers(host.dtype)
        comp = torch.cuda.current_stream(self.device)
        h = host.reshape(-1)
        ip = ipix.reshape(-1)
        n = h.numel()
        for start in range(0, n, self.CHUNK):
            m = min(self.CHUNK, n - start)
            b = self.turn
            self.turn ^= 1
            if self.free[b] is not None:
                self.copy_stream.wait_event(self.free[b])
            with torch.cuda.stream(self.copy_stream):
                bufs[b][:m].copy_(h[start:start + m], non_blocking=True)
                landed = torch.cuda.Event()
                landed.record(self.copy_stream)
            comp.wait_event(landed)
            K.tod2map(map, bufs[b][:m].view(1, m), ip[start:start + m].view(1, m))
            done = torch.cuda.Event()
            done.record(comp)
            self.free[b] = done


_STAGERS = {}


def _stager(device) -> HostStager:
    key = str(device)
    if key not in _STAGERS:
        _STAGERS[key] = HostStager(device)
    return _STAGERS[key]


_REDUCERS = {}


def _reducer(device) -> K.Reducer:
    key = str(device)
    if key not in _REDUCERS:
        _REDUCERS[key] = K.Reducer(device)
    return _REDUCERS[key]


class SkyMapCar(SkyMap):
    """SkyMap with the flat CAR pixelization of SkyMapCar.pix_from_radec
    (minkasi/maps/skymap.py:952-984), computed on the GPU bit-identically."""

    def pix_from_radec(self, ra, dec) -> torch.Tensor:
        if self.cosdec is None:
            self.cosdec = np.cos(0.5 * (self.lims[2] + self.lims[3]))
        ra = as_device(ra, torch.float64)
        dec = as_device(dec, torch.float64)
        return K.pix_car(ra, dec, self.lims[0], self.lims[2], self.pixsize, float(self.cosdec),
                         self.ny, trunc=False)


def radec2pix_car(ra, dec, ipix: torch.Tensor, lims, pixsize: float, cosdec: float, ny: int) -> None:
    """Fill ``ipix`` (int32 CUDA tensor, same size as ra) in place, as
    radec2pix_car (minkasi/maps/utils.py:178-216)."""
    ra = as_device(ra, torch.float64).reshape(-1)
    dec = as_device(dec, torch.float64).reshape(-1)
    if not (isinstance(ipix, torch.Tensor) and ipix.is_cuda and ipix.is_contiguous()):
        raise ValueError("ipix must be a contiguous int32 CUDA tensor")
    K.pix_car(ra, dec, lims[0], lims[2], pixsize, cosdec, ny, trunc=True, out=ipix.view(-1))


def car_wcs(lims, pixsize: float, ref_equ: bool = False) -> List[float]:
    """(crval1, crval2, crpix1, crpix2, cdelt1, cdelt2), degrees, of the CAR
    WCS that get_wcs builds (minkasi/maps/utils.py:47-66; CAR uses cosdec = 1)."""
    cosdec = 1.0
    if ref_equ:
        crval = [0.0, 0.0]
        crpix = [lims[1] / pixsize + 1, -lims[2] / pixsize + 1]
    else:
        crpix = [1.0, 1.0]
        crval = [lims[1] * 180 / np.pi, lims[2] * 180 / np.pi]
    cdelt = [-pixsize / cosdec * 180 / np.pi, pixsize * 180 / np.pi]
    return [float(v) for v in crval + crpix + cdelt]


def car_world2pix(ra_deg: float, dec_deg: float, w) -> tuple:
    """1-based pixel coordinates of one point through a CAR WCS (the map-size
    corners; the per-sample version is the mk_pix_wcs_car kernel): rotation
    to native spherical coordinates about the pole given by crval and the
    default LONPOLE/LATPOLE (Calabretta & Greisen 2002, eqs. 5, 8-10), CAR
    x = phi, y = theta, p = crpix + x / cdelt."""
    ra0, dec0 = w[0], w[1]
    if dec0 >= 0:
        phi_p, delta_p, alpha_p = 0.0, 90.0 - dec0, ra0 - 180.0
    else:
        phi_p, delta_p, alpha_p = 180.0, 90.0 + dec0, ra0
    d2r = math.pi / 180
    sdp, cdp = math.sin(delta_p * d2r), math.cos(delta_p * d2r)
    sd, cd = math.sin(dec_deg * d2r), math.cos(dec_deg * d2r)
    sl, cl = math.sin((ra_deg - alpha_p) * d2r), math.cos((ra_deg - alpha_p) * d2r)
    phi = phi_p + math.atan2(-cd * sl, sd * cdp - cd * sdp * cl) / d2r
    if phi > 180:
        phi -= 360
    elif phi < -180:
        phi += 360
    theta = math.asin(max(-1.0, min(1.0, sd * sdp + cd * cdp * cl))) / d2r
    return w[2] + phi / w[4], w[3] + theta / w[5]


def round_half_even(x: float) -> float:
    return float(np.round(x))


class Mapset:
    """A list of maps with vector-space operations (mapset.py:67-231)."""

    def __init__(self):
        self.nmap = 0
        self.maps: List[SkyMap] = []

    def add_map(self, map: SkyMap):
        self.maps.append(map.copy())
        self.nmap += 1

    def copy(self) -> "Mapset":
        new = self.__class__()
        for m in self.maps:
            new.add_map(m.copy())
        return new

    def clear(self):
        for m in self.maps:
            m.clear()

    def _check(self, other: "Mapset"):
        if self.nmap != other.nmap:
            raise ValueError(f"nmaps don't match, this Mapset has {self.nmap} but the provided "
                             f"Mapset has {other.nmap}")

    def dot(self, mapset: "Mapset") -> float:
        self._check(mapset)
        tot = 0.0
        for a, b in zip(self.maps, mapset.maps):
            tot = tot + a.dot(b)
        return tot

    def axpy(self, mapset: "Mapset", a: float):
        self._check(mapset)
        for a_, b_ in zip(self.maps, mapset.maps):
            a_.axpy(b_, a)

    def __add__(self, mapset: "Mapset") -> "Mapset":
        mm = self.copy()
        mm.axpy(mapset, 1.0)
        return mm

    def __sub__(self, mapset: "Mapset") -> "Mapset":
        mm = self.copy()
        mm.axpy(mapset, -1.0)
        return mm

    def __mul__(self, mapset: "Mapset") -> "Mapset":
        self._check(mapset)
        mm = mapset.copy()
        for i in range(self.nmap):
            mm.maps[i] = self.maps[i] * mapset.maps[i]
        return mm

    def get_caches(self):
        for m in self.maps:
            m.get_caches()

    def clear_caches(self):
        for m in self.maps:
            m.clear_caches()

    def mpi_reduce(self):
        for m in self.maps:
            m.mpi_reduce()
