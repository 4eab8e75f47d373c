"""Time-ordered data: Tod and TodVec (minkasi/tods/core.py:30-1047).

A ``Tod`` keeps the reference's ``info`` dict (``dat_calib``, ``dx``/``dy``,
the pixellization under the map's tag, ...).  Arrays may be numpy (as the
reference's readers produce) or CUDA tensors; device copies are made once
and cached.  ``TodVec.dot`` / ``make_rhs`` run through the batched operator
of ``minkasi_gb300.engine``: every TOD's pixel indices live in one pooled
HBM buffer, so each projection is one kernel launch for all TODs.
"""
from __future__ import annotations

import copy
import time
from typing import Any, Dict, List, Optional, Tuple

import numpy as np
import torch

from . import kernels as K
from . import parallel
from .maps import Mapset, SkyMap, as_device, default_device
from .noise import NoiseSmoothedSVD


class Tod:
    """One TOD (core.py:30-783)."""

    def __init__(self, info: dict):
        self.info: dict = info.copy()
        self.jumps = None
        self.cuts = None
        self.noise = None
        self.noise_delayed = False
        self.noise_args: Tuple = ()
        self.noise_kwargs: dict = {}
        self.noise_modelclass = None
        self._dev_pix: Dict[str, torch.Tensor] = {}

    # ---- shape / data --------------------------------------------------
    def get_ndet(self) -> int:
        return int(self.info["dat_calib"].shape[0])

    def get_ndata(self) -> int:
        return int(self.info["dat_calib"].shape[1])

    def get_nsamp(self) -> int:
        return self.get_ndet() * self.get_ndata()

    def get_data_dims(self) -> Tuple[int, int]:
        return (self.get_ndet(), self.get_ndata())

    def get_data(self, dat=None):
        if dat is None:
            dat = self.info.get("dat_calib", None)
        if dat is None:
            raise ValueError("This TOD has no stored data. Populare tod.info['dat_calib']")
        return dat

    def get_tvec(self):
        """The time vector, info['ctime'] (core.py:262-271)."""
        return self.info["ctime"]

    def prior_from_skymap(self, skymap):
        """A CutsCompact prior on the samples where ``skymap`` projects to a
        non-zero value, weighted 1 / value^2 (core.py:750-780)."""
        from .tsmodels import CutsCompact
        tmp = self.get_empty(True)
        skymap.map2tod(self, tmp)
        prior = CutsCompact(self)
        prior.cuts_from_array(tmp == 0)
        prior.get_imap()
        prior.tod2map(self, tmp)
        prior.map = 1.0 / prior.map ** 2
        return prior

    def get_radec(self):
        return self.info["dx"], self.info["dy"]

    def lims(self) -> List[float]:
        dx, dy = self.info["dx"], self.info["dy"]
        f = (lambda a: float(a.min())) if not isinstance(dx, torch.Tensor) else (lambda a: float(a.min().item()))
        g = (lambda a: float(a.max())) if not isinstance(dx, torch.Tensor) else (lambda a: float(a.max().item()))
        return [f(dx), g(dx), f(dy), g(dy)]

    def get_empty(self, clear: bool = False, dtype: Optional[torch.dtype] = None):
        dt = dtype or torch.float64
        shape = (self.get_ndet(), self.get_ndata())
        dev = default_device()
        return torch.zeros(shape, dtype=dt, device=dev) if clear else torch.empty(shape, dtype=dt, device=dev)

    # ---- pixellization -------------------------------------------------
    def get_saved_pix(self, tag: str = "ipix"):
        return self.info.get(tag, None)

    def clear_saved_pix(self, tag: str = "ipix"):
        self.info.pop(tag, None)
        self._dev_pix.pop(tag, None)

    def save_pixellization(self, tag: str, ipix):
        if tag in self.info:
            print("warning - overwriting key ", tag, " in tod.save_pixellization.")
        self.info[tag] = ipix
        self._dev_pix.pop(tag, None)

    def device_pix(self, tag: str, npix: int) -> torch.Tensor:
        """int32 CUDA copy of info[tag], bounds-checked against npix once.
        The reference only warns on a wrong dtype (tod2map.py:48-51) and would
        read or write outside the map on a bad index; here it is an error."""
        t = self._dev_pix.get(tag)
        if t is None or getattr(t, "_mk_npix", None) != npix:
            src = self.info[tag]
            if isinstance(src, np.ndarray) and src.dtype != np.int32:
                raise TypeError(f"pixellization '{tag}' must be int32, got {src.dtype}")
            t = as_device(src, torch.int32)
            nbad = K.check_pix(t, npix)
            if nbad:
                raise ValueError(f"{nbad} pixel indices of '{tag}' fall outside the {npix}-pixel map")
            t._mk_npix = npix
            self._dev_pix[tag] = t
        return t

    def device_sincos(self, dtype: torch.dtype = torch.float64):
        """(cos, sin) of info['twogamma_saved'] on the device in ``dtype``,
        computed once (mk_pol_sincos) and cached with the pixellization."""
        key = ("sincos", dtype)
        t = self._dev_pix.get(key)
        if t is None:
            tg = as_device(self.info["twogamma_saved"], torch.float64)
            t = K.pol_sincos(tg.reshape(self.get_data_dims()).contiguous(), dtype)
            self._dev_pix[key] = t
        return t

    def set_tag(self, tag: Any):
        if "tag" in self.info:
            print("Warning: overwriting tag")
        self.info["tag"] = tag

    def set_pix(self, map: SkyMap):
        ipix = map.get_pix(self)
        self.save_pixellization(map.tag, ipix)

    # ---- noise -----------------------------------------------------------
    def set_noise(self, modelclass=NoiseSmoothedSVD, dat=None, delayed: bool = False, *args, **kwargs):
        if delayed:
            self.noise_args = copy.deepcopy(args)
            self.noise_kwargs = copy.deepcopy(kwargs)
            self.noise_delayed = True
            self.noise_modelclass = modelclass
        else:
            self.noise_delayed = False
            dat = self.get_data(dat)
            self.noise = modelclass(dat, *args, **kwargs)

    def get_det_weights(self):
        if self.noise is None:
            print("noise model not set in get_det_weights.")
            return None
        if hasattr(self.noise, "get_det_weights"):
            return self.noise.get_det_weights()
        print("noise model does not support detector weights in get_det_weights.")
        return None

    def apply_noise(self, dat=None):
        """Apply the noise model (core.py:517-580); returns a new array."""
        dat = self.get_data(dat)
        if self.noise_delayed:
            self.noise = self.noise_modelclass(dat, *self.noise_args, **self.noise_kwargs)
            self.noise_delayed = False
        if self.noise is None:
            raise RuntimeError("tod.noise is not set; only class-based noise models run on the GPU")
        return self.noise.apply_noise(dat)

    # ---- operator pieces ---------------------------------------------------
    def mapset2tod(self, mapset: Mapset, dat=None):
        if dat is None:
            dat = self.get_empty(True, mapset.maps[0].dtype)
        for m in mapset.maps:
            m.map2tod(self, dat)
        return dat

    def tod2mapset(self, mapset: Mapset, dat=None):
        if dat is None:
            dat = self.get_data()
        for m in mapset.maps:
            m.tod2map(self, dat)

    def dot(self, mapset: Mapset, mapset_out: Mapset, times: bool = False, mask: Optional[Mapset] = None):
        """out += P^T N P x for this TOD (core.py:649-691)."""
        t1 = time.time()
        if mask is not None:
            for i, imap in enumerate(mapset.maps):
                K.mul(imap.map, imap.map, mask.maps[i].map)
        tmp = self.mapset2tod(mapset)
        t2 = time.time()
        tmp = self.apply_noise(tmp)
        t3 = time.time()
        self.tod2mapset(mapset_out, tmp)
        if mask is not None:
            for i, imap in enumerate(mapset_out.maps):
                K.mul(imap.map, imap.map, mask.maps[i].map)
        t4 = time.time()
        if times:
            return np.asarray([t2 - t1, t3 - t2, t4 - t3])

    def iter_init(self):
        pass

    def iter_finalize(self):
        pass

    def copy(self, copy_info: bool = False) -> "Tod":
        if copy_info:
            myinfo = self.info.copy()
            for key in myinfo.keys():
                try:
                    myinfo[key] = self.info[key].copy() if not isinstance(self.info[key], torch.Tensor) \
                        else self.info[key].clone()
                except Exception:
                    pass
            tod = Tod(myinfo)
        else:
            tod = Tod(self.info)
            tod._dev_pix = dict(self._dev_pix)
        tod.jumps = None if self.jumps is None else list(self.jumps)
        tod.cuts = None if self.cuts is None else list(self.cuts)
        tod.noise = self.noise
        return tod


class TodVec:
    """A collection of TODs (core.py:786-1047)."""

    def __init__(self):
        self.tods: List[Tod] = []
        self.ntod = 0
        self._engines: Dict[Any, Any] = {}
        self._shared: Dict[str, Any] = {}   # pooled device buffers shared by the engines
        # kernel choices for the batched operator: "auto" = project autotuner
        self.tod2map_method = "auto"
        self.rot_mode = 0

    def add_tod(self, tod: Tod, copy_info: bool = False):
        self.tods.append(tod.copy(copy_info))
        self.tods[-1].set_tag(self.ntod)
        self.ntod += 1
        self._engines.clear()
        self._shared.clear()

    def lims(self) -> Optional[List[float]]:
        if self.ntod == 0:
            return None
        xmin, xmax, ymin, ymax = self.tods[0].lims()
        for t in self.tods[1:]:
            x1, x2, y1, y2 = t.lims()
            xmin, xmax, ymin, ymax = min(x1, xmin), max(x2, xmax), min(y1, ymin), max(y2, ymax)
        return [parallel.allreduce_scalar(xmin, "min"), parallel.allreduce_scalar(xmax, "max"),
                parallel.allreduce_scalar(ymin, "min"), parallel.allreduce_scalar(ymax, "max")]

    def get_nsamp(self, reduce: bool = True) -> int:
        tot = sum(t.get_nsamp() for t in self.tods)
        if reduce:
            tot = int(parallel.allreduce_scalar(tot, "sum"))
        return tot

    def set_pix(self, map: SkyMap):
        for t in self.tods:
            t.set_pix(map)

    # ---- batched operator ----------------------------------------------
    def engine(self, map: SkyMap, dtype: Optional[torch.dtype] = None, **kw):
        """The batched operator A = sum_tod P^T N P for ``map``'s pixellization,
        built once and cached (see minkasi_gb300.engine.MapmakingOperator)."""
        from .engine import MapmakingOperator

        dtype = dtype or map.dtype
        kw.setdefault("tod2map", self.tod2map_method)
        kw.setdefault("rot_mode", self.rot_mode)
        key = (map.tag, map.nx, map.ny, dtype, tuple(sorted(kw.items())))
        if key not in self._engines:
            self._engines[key] = MapmakingOperator(self, map, dtype=dtype, **kw)
        return self._engines[key]

    def _fast(self, mapset: Mapset) -> bool:
        return mapset.nmap == 1 and isinstance(mapset.maps[0], SkyMap) and \
            getattr(mapset.maps[0], "npol", 1) == 1 and self.ntod > 0 and \
            all(t.noise is not None and isinstance(t.noise, NoiseSmoothedSVD) for t in self.tods)

    def dot(self, mapset: Mapset, mapset_out: Optional[Mapset] = None, report_times: bool = False,
            cache_maps: bool = False, mask: Optional[Mapset] = None):
        """A x summed over TODs, then over ranks (core.py:967-1026)."""
        if mapset_out is None:
            mapset_out = mapset.copy()
            mapset_out.clear()
        times = np.zeros(self.ntod)
        if self._fast(mapset) and not report_times:
            if mask is not None:
                K.mul(mapset.maps[0].map, mapset.maps[0].map, mask.maps[0].map)
            eng = self.engine(mapset.maps[0])
            eng.apply(mapset.maps[0].map, mapset_out.maps[0].map, accumulate=True)
            if mask is not None:
                K.mul(mapset_out.maps[0].map, mapset_out.maps[0].map, mask.maps[0].map)
        else:
            for i, tod in enumerate(self.tods):
                t1 = time.time()
                tod.dot(mapset, mapset_out, True, mask=mask)
                torch.cuda.synchronize()
                times[i] = time.time() - t1
        mapset_out.mpi_reduce()
        if report_times:
            return mapset_out, times
        return mapset_out

    def dot_cached(self, mapset: Mapset, mapset_out: Optional[Mapset] = None,
                   mask: Optional[Mapset] = None) -> Mapset:
        return self.dot(mapset, mapset_out, mask=mask)

    def make_rhs(self, mapset: Mapset, do_clear: bool = False):
        """b = sum_tod P^T N d  (core.py:1028-1047)."""
        if do_clear:
            mapset.clear()
        if self._fast(mapset):
            self.engine(mapset.maps[0]).rhs(mapset.maps[0].map)
        else:
            for tod in self.tods:
                dat_filt = tod.apply_noise()
                for m in mapset.maps:
                    m.tod2map(tod, dat_filt)
        mapset.mpi_reduce()
