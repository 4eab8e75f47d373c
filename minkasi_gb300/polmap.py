"""Polarized maps on the GPU: PolMap (minkasi/maps/polmap.py:47-725).

A PolMap holds an (nx, ny, npol) Stokes map (an (nx, ny) map for poltag "I")
as a CUDA tensor; the pixel-major layout is the reference's, so map[x, y, k]
is Stokes component k of pixel x * ny + y.  Geometry (CAR WCS, map size,
pointing -> pixel) is SkyMap's.  The projections run the mk_polmap2tod /
mk_tod2polmap kernels with the TOD's cos(2 gamma), sin(2 gamma) computed once
on the GPU from ``tod.info['twogamma_saved']`` and cached with the TOD.
"""
from __future__ import annotations

import os
from typing import List, Optional

import numpy as np
import torch

from . import kernels as K
from .maps import SkyMap, as_device


def _poltag2pols(poltag: str) -> Optional[List[str]]:
    """minkasi/maps/polmap.py:32-44."""
    return {"I": ["I"], "IQU": ["I", "Q", "U"], "QU": ["Q", "U"],
            "IQU_PRECON": ["I", "Q", "U", "QQ", "QU", "UU"],
            "QU_PRECON": ["QQ", "UU", "QU"]}.get(poltag)


class PolMap(SkyMap):
    def __init__(self, lims, pixsize: float, poltag: str = "I", proj: str = "CAR", pad: int = 2,
                 primes=None, cosdec: Optional[float] = None, nx: Optional[int] = None,
                 ny: Optional[int] = None, mywcs=None, tag: str = "ipix",
                 purge_pixellization: bool = False, ref_equ: bool = False,
                 dtype: torch.dtype = torch.float64, device=None):
        pols = _poltag2pols(poltag)
        if pols is None:
            raise ValueError(f"Unrecognized polarization state {poltag} in PolMap.__init__")
        super().__init__(lims, pixsize, proj=proj, pad=pad, primes=primes, cosdec=cosdec, nx=nx, ny=ny,
                         mywcs=mywcs, tag=tag, purge_pixellization=purge_pixellization,
                         ref_equ=ref_equ, dtype=dtype, device=device)
        self._set_pols(poltag, pols)

    def _set_pols(self, poltag: str, pols: List[str]) -> None:
        self.poltag, self.pols, self.npol = poltag, pols, len(pols)
        shape = (self.nx, self.ny, self.npol) if self.npol > 1 else (self.nx, self.ny)
        self.map = torch.zeros(shape, dtype=self.map.dtype, device=self.map.device)

    def set_polstate(self, poltag: str) -> None:
        """New polarization state and a zeroed map (polmap.py:273-298)."""
        pols = _poltag2pols(poltag)
        if pols is None:
            print("Unrecognized polarization state " + poltag + " in PolMap.set_polstate.")
            return
        self._set_pols(poltag, pols)

    def assign(self, arr):
        assert arr.shape[0] == self.nx and arr.shape[1] == self.ny
        if self.npol > 1:
            assert arr.shape[2] == self.npol
        self.map.copy_(as_device(arr, self.map.dtype))

    # ---- projections -----------------------------------------------------
    def _angle(self, tod):
        """(cos 2 gamma, sin 2 gamma) of the TOD in the map dtype, cached."""
        return tod.device_sincos(self.map.dtype)

    def map2tod(self, tod, dat, do_add: bool = True, do_omp: bool = True):
        """polmap.py:464-502 -> polmap2tod (QU / IQU) or the SkyMap path."""
        if self.npol == 1:
            return SkyMap.map2tod(self, tod, dat, do_add, do_omp)
        if self.poltag not in ("QU", "IQU"):
            raise NotImplementedError(f"Poltag {self.poltag} is not implemented")
        ipix = self.get_pix(tod)
        d = dat if isinstance(dat, torch.Tensor) else as_device(dat, self.map.dtype)
        K.polmap2tod(d, self.map, self.poltag, self._angle(tod), ipix, do_add)
        if not isinstance(dat, torch.Tensor):
            np.copyto(dat, d.cpu().numpy())

    def tod2map(self, tod, dat=None, do_add: bool = True, do_omp: bool = True):
        """polmap.py:504-545 -> tod2polmap or the SkyMap path."""
        if self.npol == 1:
            return SkyMap.tod2map(self, tod, dat, do_add, do_omp)
        if dat is None:
            dat = tod.get_data()
        if not do_add:
            self.clear()
        ipix = self.get_pix(tod)
        d = dat if isinstance(dat, torch.Tensor) else as_device(dat, self.map.dtype)
        if not d.is_cuda:
            d = d.to(self.map.device)
        K.tod2polmap(self.map, d.to(self.map.dtype).contiguous(), self.poltag, self._angle(tod), ipix)
        if self.purge_pixellization:
            tod.clear_saved_pix(self.tag)

    def tod2map_rows(self, tod, w: Optional[torch.Tensor] = None) -> None:
        """Hit / weight accumulation (make_hits on a PolMap) without a TOD of ones."""
        ipix = self.get_pix(tod)
        if self.npol == 1:
            K.tod2map_rows(self.map.reshape(-1), ipix, w)
            return
        K.tod2polmap(self.map, None, self.poltag, self._angle(tod), ipix, rowval=w,
                     shape=tod.get_data_dims())

    # ---- vector space ------------------------------------------------------
    def __mul__(self, map: "PolMap") -> "PolMap":
        """polmap.py:624-684: elementwise for "I", else the PRECON matrix of
        each pixel times the map's Stokes vector."""
        if self.npol == 1:
            return SkyMap.__mul__(self, map)
        if map.poltag + "_PRECON" != self.poltag:
            raise ValueError("Tag from input map does not match this map")
        new = map.copy()
        K.pol_precon_mul(new.map, self.map, map.map, self.poltag)
        return new

    def invert(self, thresh: float = 1e-6):
        """Invert the per-pixel preconditioner matrices (polmap.py:300-384):
        pseudo-inverse with singular values below thresh * the largest dropped;
        for IQU_PRECON, matrices whose determinant is below thresh * the
        largest are zeroed except for 1/I where I > 0, as the reference does."""
        if self.npol == 1:
            return SkyMap.invert(self)
        m = self.map
        n = self.nx * self.ny
        if self.poltag == "QU_PRECON":
            t = torch.zeros((n, 2, 2), dtype=m.dtype, device=m.device)
            t[:, 0, 0] = m[:, :, 0].reshape(n)
            t[:, 1, 1] = m[:, :, 1].reshape(n)
            t[:, 0, 1] = m[:, :, 2].reshape(n)
            t[:, 1, 0] = m[:, :, 2].reshape(n)
            t = torch.linalg.pinv(t, rtol=thresh)
            m[:, :, 0] = t[:, 0, 0].reshape(self.nx, self.ny)
            m[:, :, 1] = t[:, 1, 1].reshape(self.nx, self.ny)
            m[:, :, 2] = t[:, 0, 1].reshape(self.nx, self.ny)
        elif self.poltag == "IQU_PRECON":
            t = torch.zeros((n, 3, 3), dtype=m.dtype, device=m.device)
            for (i, j), k in (((0, 0), 0), ((0, 1), 1), ((0, 2), 2), ((1, 1), 3), ((1, 2), 4), ((2, 2), 5)):
                t[:, i, j] = m[:, :, k].reshape(n)
                t[:, j, i] = t[:, i, j]
            dets = torch.linalg.det(t)
            isbad = dets < thresh * dets.max()
            ispos = t[:, 0, 0] > 0
            inds = isbad & ispos
            vec = t[inds, 0, 0]
            t = torch.linalg.pinv(t, rtol=thresh)
            t[isbad] = 0
            t[inds, 0, 0] = 1.0 / vec
            for (i, j), k in (((0, 0), 0), ((0, 1), 1), ((0, 2), 2), ((1, 1), 3), ((1, 2), 4), ((2, 2), 5)):
                m[:, :, k] = t[:, i, j].reshape(self.nx, self.ny)

    def write(self, fname: str = "map.fits"):
        """One FITS image per Stokes component, <name>_<pol>.fits, each
        transposed, with the map's CAR WCS (polmap.py:585-622)."""
        if self.npol == 1:
            return SkyMap.write(self, fname)
        from . import fits
        fname = os.path.abspath(fname)
        ind = fname.rfind(".")
        head, tail = (fname[:ind], fname[ind:]) if ind > 0 and fname[ind + 1:] == "fits" else (fname, ".fits")
        cards = fits.car_header(self.wcs) if self.wcs is not None else []
        m = self.map.detach().cpu().numpy()
        for i, pol in enumerate(self.pols):
            fits.write_image(head + "_" + pol + tail, np.ascontiguousarray(m[:, :, i].T), cards)

    def r_th_maps(self):
        """Radius and angle of every pixel about the map centre (polmap.py:547-566)."""
        x = torch.arange(self.nx, dtype=torch.float64, device=self.map.device)
        y = torch.arange(self.ny, dtype=torch.float64, device=self.map.device)
        x = x - x.mean()
        y = y - y.mean()
        xm, ym = torch.meshgrid(x, y, indexing="ij")
        return torch.sqrt(xm ** 2 + ym ** 2), torch.atan2(xm, ym)
