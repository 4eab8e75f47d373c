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

    Parameters follow the reference.  Without astropy, the pixelization is
    the reference's CAR layout restated with a flat-sky formula
    (x = (lims[1] - ra) * cos(dec0) / pixsize, y = (dec - lims[2]) / pixsize,
    ipix = x * ny + y); pixel indices supplied by the caller in
    ``tod.info[tag]`` always take precedence, exactly as in the reference
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
        self.pixsize = float(pixsize)
        self.proj = proj
        self.pad = pad
        self.primes = primes
        if self.lims is not None and cosdec is None:
            cosdec = math.cos(0.5 * (self.lims[2] + self.lims[3]))
        self.cosdec = cosdec
        if nx is None or ny is None:
            if self.lims is None or self.pixsize <= 0:
                raise ValueError("SkyMap needs (lims, pixsize) or explicit nx, ny")
            cnx = int(round((self.lims[1] - self.lims[0]) * self.cosdec / self.pixsize)) + 1 + pad
            cny = int(round((self.lims[3] - self.lims[2]) / self.pixsize)) + 1 + pad
            nx = cnx if nx is None else nx
            ny = cny if ny is None else ny
        self.nx, self.ny = int(nx), int(ny)
        self.tag = tag
        self.purge_pixellization = purge_pixellization
        self.caches = None
        self.wcs = mywcs
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
    def pix_from_radec(self, ra, dec) -> torch.Tensor:
        """int32 pixel indices from RA/dec in radians (flat CAR restatement of
        SkyMap.pix_from_radec, skymap.py:457-490)."""
        ra = as_device(ra, torch.float64)
        dec = as_device(dec, torch.float64)
        x = torch.round((self.lims[1] - ra) * self.cosdec / self.pixsize)
        y = torch.round((dec - self.lims[2]) / self.pixsize)
        return (x * self.ny + y).to(torch.int32).contiguous()

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
            d = dat  # pinned host timestream: the scatter kernel reads it in place
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

    def write(self, fname: str = "map.npy"):
        """Save the map.  FITS needs astropy (not a dependency here): the map
        is written as .npy next to the requested name."""
        root, ext = os.path.splitext(os.path.abspath(fname))
        os.makedirs(os.path.dirname(root), exist_ok=True)
        np.save(root + ".npy", self.map.detach().cpu().numpy())

    def to_numpy(self) -> np.ndarray:
        return self.map.detach().cpu().numpy()


_REDUCERS = {}


def _reducer(device) -> K.Reducer:
    key = str(device)
    if key not in _REDUCERS:
        _REDUCERS[key] = K.Reducer(device)
    return _REDUCERS[key]


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
