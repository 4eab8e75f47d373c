"""Batched mapmaking operator A = sum_tod P^T N P on pooled device buffers.

HBM layout (one operator, S = total samples over all TODs, P = pixels):
  ipix  : int32[S]   every TOD's pixel indices back to back (TOD order,
                     each TOD detector-major like the reference's (ndet, ndata))
  tmp   : dtype[S]   the projected / filtered timestreams, same layout
  v, vT : per TOD (ndet, ndet); mywt: per TOD (ndet, ndata) in the operator dtype
  ws    : one DCT/FFT workspace sized for the largest TOD, shared by the
          per-shape noise plans (they run in stream order)
  map   : dtype[P], L2-resident during the projections
So map2tod and tod2map are ONE launch each over all S samples, whatever the
number and shapes of the TODs.  The noise filter's detector rotations are
one launch per detector count over all TODs (kernels.NoiseGroup, in place on
tmp); its DCT-I passes run per TOD shape plan, because each TOD's FFT needs
its own length-dependent tables and scratch.

The reference does the same work TOD by TOD with a fresh (ndet, ndata)
temporary per call (minkasi/tods/core.py:582-620,649-691,967-1026).
"""
from __future__ import annotations

import os
from typing import Dict, List, Optional, Tuple

import numpy as np
import torch

from . import kernels as K
from .maps import SkyMap, as_device


class MapmakingOperator:
    def __init__(self, todvec, map: SkyMap, dtype: torch.dtype = torch.float64,
                 tod2map: str = "auto", rot_mode: int = 0):
        self.dtype = dtype
        self.device = map.map.device
        self.npix = map.npix
        self.shape = (map.nx, map.ny)
        self.tods = list(todvec.tods)
        self.tag = map.tag
        self.sizes = [t.get_nsamp() for t in self.tods]
        self.dims = [t.get_data_dims() for t in self.tods]
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes)]).astype(np.int64)
        self.S = int(self.offsets[-1])
        # one pixel-index pool and one timestream scratch per TodVec, shared by
        # its operators of every precision (FP64 and FP32 passes never overlap)
        shared = todvec._shared
        key = (self.tag, self.npix, self.S)
        if shared.get("ipix_key") == key:
            self.ipix = shared["ipix"]
        else:
            self.ipix = torch.empty(self.S, dtype=torch.int32, device=self.device)
            for t, o, n in zip(self.tods, self.offsets, self.sizes):
                src = t.device_pix(self.tag, self.npix).reshape(-1)
                self.ipix[o:o + n].copy_(src)
                view = self.ipix[o:o + n].view(t.get_data_dims())
                view._mk_npix = self.npix
                t._dev_pix[self.tag] = view  # the pool replaces the per-TOD copy
                if isinstance(t.info.get(self.tag), torch.Tensor) and t.info[self.tag].is_cuda:
                    t.info[self.tag] = view  # and frees the caller's device copy
            shared.update(ipix_key=key, ipix=self.ipix)
        nbytes = self.S * torch.finfo(dtype).bits // 8
        buf = shared.get("tmp")
        if buf is None or buf.numel() < nbytes:
            buf = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
            shared["tmp"] = buf
        self.tmp = buf[:nbytes].view(dtype)
        self.rot_mode = int(rot_mode)
        self.ops = None
        self.plans: Dict[Tuple[int, int], K.NoisePlan] = {}
        self.ws = None
        self._hmax: Optional[int] = None
        self._fixed: Optional[K.FixedScratch] = None
        self._pixplans: Optional[List[K.PixPlan]] = None
        self._group = None
        self._group_key = None
        self.method = tod2map
        if tod2map == "auto":
            from .autotune import choose_tod2map
            self.method = choose_tod2map(self)
        if all(t.noise is not None for t in self.tods):
            self.prepare_noise()

    def prepare_noise(self) -> None:
        """Noise operands in the operator dtype and one shared plan workspace;
        picks the rotation GEMM if rot_mode is 0 (automatic)."""
        if self.ops is not None:
            return
        self.ops = [t.noise.operands(self.dtype) for t in self.tods]
        shapes = sorted(set(self.dims))
        from .autotune import choose_dct_engines, with_dct_engine
        # the DCT-I transform per shape (FP32: four-step FFT or cuFFT,
        # whichever runs this shape's filter faster)
        engines = choose_dct_engines(self, shapes)
        ws_bytes = max(with_dct_engine(engines[s], lambda s=s: K.noise_workspace_bytes(s[0], s[1], self.dtype))
                       for s in shapes)
        self.ws = torch.empty(ws_bytes, dtype=torch.uint8, device=self.device)
        # cuFFT allocates its plan tables with cudaMalloc, outside torch's
        # caching allocator: hand back cached blocks first so a near-full
        # device can still build one plan per distinct TOD shape.
        torch.cuda.empty_cache()
        self.plans = {s: with_dct_engine(engines[s], lambda s=s: K.NoisePlan(s[0], s[1], self.dtype, self.device,
                                                                             workspace=self.ws))
                      for s in shapes}
        self.dct_engines = {s: p.engine for s, p in self.plans.items()}
        self.dct_splits = {s: p.split for s, p in self.plans.items()}
        if self.rot_mode == 0:
            from .autotune import choose_rot_mode
            self.rot_mode = choose_rot_mode(self)

    # ---- pieces ------------------------------------------------------------
    def views(self, buf: torch.Tensor):
        for (nd, n), o in zip(self.dims, self.offsets):
            yield buf[o:o + nd * n].view(nd, n)

    def hits(self) -> torch.Tensor:
        h = torch.zeros(self.npix, dtype=torch.float64, device=self.device)
        K.tod2map_rows(h, self.ipix)
        return h

    def hmax(self) -> int:
        if self._hmax is None:
            self._hmax = max(int(self.hits().max().item()), 1)
        return self._hmax

    def project_out(self, out: torch.Tensor, method: Optional[str] = None) -> None:
        """out += P^T tmp with the chosen tod2map kernel."""
        m = method or self.method
        if m == "atomic":
            K.tod2map(out, self.tmp, self.ipix)
        elif m == "staged":
            K.tod2map_staged(out, self.tmp, self.ipix)
        elif m == "fixed":
            if self._fixed is None:
                self._fixed = K.FixedScratch(self.npix, self.device)
            K.tod2map_fixed(out, self.tmp, self.ipix, self.hmax(), self._fixed)
        elif m == "sorted":
            if self._pixplans is None:
                self._pixplans = [K.PixPlan(self.ipix[o:o + n], self.npix)
                                  for o, n in zip(self.offsets, self.sizes)]
            for pl, o, n in zip(self._pixplans, self.offsets, self.sizes):
                pl.tod2map(out, self.tmp[o:o + n])
        else:
            raise ValueError(f"unknown tod2map method {m!r}")

    def _noise_group(self):
        """The one-call filter over all TODs (kernels.NoiseGroup) when the
        operator is FP32 with tensor-core rotations (every ndet in 32, 64,
        128, 256), else None (then the filter runs TOD by TOD)."""
        if self._group is False:
            return None
        key = self.tmp.data_ptr()
        if self._group is not None and self._group_key == key:
            return self._group
        ok = (self.dtype == torch.float32 and self.rot_mode == 2 and
              all(nd in (32, 64, 128, 256) for nd, _ in self.dims) and
              os.environ.get("MINKASI_GB300_GROUP", "1") != "0")
        if not ok:
            self._group = False
            return None
        views = list(self.views(self.tmp))
        self._group = K.NoiseGroup([self.plans[d] for d in self.dims], self.ops, views)
        self._group_key = key
        return self._group

    def noise_all(self) -> None:
        self.prepare_noise()
        grp = self._noise_group()
        if grp is not None:
            grp.apply()
            return
        for (v, vT, w), view, dims in zip(self.ops, self.views(self.tmp), self.dims):
            self.plans[dims].apply(v, vT, w, view, out=view, rot_mode=self.rot_mode)

    # ---- the operator ---------------------------------------------------------
    def apply(self, x: torch.Tensor, out: torch.Tensor, accumulate: bool = False) -> torch.Tensor:
        """out (+)= A x.  x, out: (nx, ny) or flat maps of the operator dtype."""
        xf, of = x.reshape(-1), out.reshape(-1)
        K.map2tod(self.tmp, xf, self.ipix, False)
        self.noise_all()
        if not accumulate:
            of.zero_()
        self.project_out(of)
        return out

    def rhs(self, out: torch.Tensor) -> torch.Tensor:
        """out += sum_tod P^T N d with d = tod.info['dat_calib']."""
        for t, view in zip(self.tods, self.views(self.tmp)):
            view.copy_(as_device(t.get_data(), self.dtype, self.device))
        self.noise_all()
        self.project_out(out.reshape(-1))
        return out

    def release(self) -> None:
        self._group = None
        self.tmp = None
        self.ws = None
        self.plans = {}
        self._pixplans = None
