"""NoiseSmoothedSVD on the GPU (minkasi/mapmaking/noise.py:584-772).

The model is built on the device: the left singular vectors come from a
QR of dat^T followed by the SVD of the small (ndet x ndet) R factor
(d^T = Q R, R = U S V^T  =>  d = V S (Q U)^T, so the left singular vectors of
d are the columns of V), which equals the reference's
``np.linalg.svd(dat, True)[0]`` up to the sign of each vector without forming
the ndata x ndata matrix the reference's full-matrices SVD allocates.  The
spectrum is the DCT-I power of the rotated data smoothed by a DCT-I Gaussian
convolution (minkasi/tools/smooth.py:49-78), all with libmkgpu's DCT-I.

``apply_noise`` runs libmkgpu's fused filter (mk_apply_noise).  A sign flip
of a singular vector flips the matching row of v and column of vT together,
so the operator vT diag(w) DCT v is unchanged by it.
"""
from __future__ import annotations

from collections import OrderedDict
from typing import Dict, Optional, Tuple

import numpy as np
import torch

from . import kernels as K
from .maps import as_device, default_device

_PLAN_CACHE: "OrderedDict[Tuple[int, int, torch.dtype, str], K.NoisePlan]" = OrderedDict()
_PLAN_CACHE_SIZE = 4  # each plan holds an FFT workspace of ~40 B per sample


def noise_plan(ndet: int, ndata: int, dtype: torch.dtype, device) -> K.NoisePlan:
    """Plan for one-off apply_noise calls, from a small LRU cache (the batched
    operator keeps its own plans on one shared workspace)."""
    key = (int(ndet), int(ndata), dtype, str(device))
    if key in _PLAN_CACHE:
        _PLAN_CACHE.move_to_end(key)
        return _PLAN_CACHE[key]
    while len(_PLAN_CACHE) >= _PLAN_CACHE_SIZE:
        _PLAN_CACHE.popitem(last=False)
    _PLAN_CACHE[key] = K.NoisePlan(ndet, ndata, dtype, device)
    return _PLAN_CACHE[key]


def clear_plan_cache() -> None:
    """Drop the one-off plans and their FFT workspaces."""
    _PLAN_CACHE.clear()


def dct1(x: torch.Tensor) -> torch.Tensor:
    """Unnormalised DCT-I along the last axis (fft_r2r, tools/fft.py:290-344)."""
    x2 = x.reshape(1, -1) if x.dim() == 1 else x
    out = K.DCT1(x2.shape[0], x2.shape[1], x2.dtype, x2.device)(x2.contiguous())
    return out.reshape(x.shape)


def smooth_many_vecs(vecs: torch.Tensor, fwhm: float = 20.0) -> torch.Tensor:
    """Gaussian smoothing of each row as a DCT-I convolution (smooth.py:49-78)."""
    n = vecs.shape[1]
    x = np.arange(n)
    sig = fwhm / np.sqrt(8 * np.log(2))
    to_conv = np.exp(-0.5 * (x / sig) ** 2)
    tot = to_conv[0] + to_conv[-1] + 2 * to_conv[1:-1].sum()
    to_conv = as_device(to_conv / tot, vecs.dtype, vecs.device)
    to_conv_ft = dct1(to_conv)
    xtrans = dct1(vecs)
    xtrans *= to_conv_ft[None, :]
    back = dct1(xtrans)
    return back / (2 * (n - 1))


def row_median(a: torch.Tensor) -> torch.Tensor:
    """numpy.median along the last axis: the mean of the two middle values
    for an even count (torch.median would return the lower one)."""
    s = torch.sort(a, dim=-1).values
    n = s.shape[-1]
    if n % 2:
        return s[..., n // 2].clone()
    return (s[..., n // 2 - 1] + s[..., n // 2]) / 2


def _eig_desc(c: np.ndarray) -> np.ndarray:
    w, u = np.linalg.eigh(c)
    return u[:, np.argsort(w)[::-1]]


def left_singular_vectors(dat: torch.Tensor) -> torch.Tensor:
    """u of the thin SVD of dat (ndet x ndata), columns by descending singular
    value: eigenvectors of the Gram matrix d d^T (an FP64 GEMM on the GPU),
    decomposed on the host (ndet x ndet), then refined once by
    re-diagonalising the Gram matrix of the rotated data."""
    u = _eig_desc((dat @ dat.T).cpu().numpy())
    ut = torch.from_numpy(np.ascontiguousarray(u)).to(dat.device)
    d2 = ut.T @ dat
    u = u @ _eig_desc((d2 @ d2.T).cpu().numpy())
    return torch.from_numpy(np.ascontiguousarray(u)).to(dat.device)


class NoiseSmoothedSVD:
    """Noise model: rotate into singular space, smoothed inverse spectra."""

    def __init__(self, dat_use, fwhm: float = 50.0, prewhiten: bool = False,
                 fit_powlaw: bool = False, u_in=None):
        if fit_powlaw:
            raise NotImplementedError("fit_powlaw spectra are outside the GPU hot path")
        dat = as_device(dat_use, torch.float64)
        self.noisevec: Optional[torch.Tensor] = None
        if prewhiten:
            noisevec = row_median(torch.abs(torch.diff(dat, dim=1)))
            dat = dat / noisevec[:, None]
            self.noisevec = noisevec.clone()
        if u_in is None:
            u = left_singular_vectors(dat)
            self.v = u.T.contiguous()
            self.vT = self.v.T.contiguous()
        else:
            u = as_device(u_in, torch.float64)
            assert u.shape[0] == u.shape[1]
            self.v = u.T.contiguous()
            self.vT = torch.from_numpy(np.linalg.inv(self.v.cpu().numpy())).to(self.v.device).contiguous()
        dat_rot = self.v @ dat
        dat_trans = dct1(dat_rot)
        spec = smooth_many_vecs(dat_trans ** 2, fwhm)
        spec[:, 1:] = 1.0 / spec[:, 1:]
        spec[:, 0] = 0
        self.mywt = spec.contiguous()
        self._typed: Dict[torch.dtype, Tuple[torch.Tensor, torch.Tensor, torch.Tensor]] = {}

    @classmethod
    def from_arrays(cls, v, vT, mywt, noisevec=None) -> "NoiseSmoothedSVD":
        """A model from existing arrays (e.g. a reference-built model's v, vT, mywt)."""
        self = cls.__new__(cls)
        self.v = as_device(v, torch.float64)
        self.vT = as_device(vT, torch.float64)
        self.mywt = as_device(mywt, torch.float64)
        self.noisevec = None if noisevec is None else as_device(noisevec, torch.float64)
        self._typed = {}
        return self

    # rotation matrices with the prewhitening folded in:
    #   v' = v diag(1/noisevec),  vT' = diag(1/noisevec) vT
    def operands(self, dtype: torch.dtype = torch.float64):
        if dtype not in self._typed:
            v, vT = self.v, self.vT
            if self.noisevec is not None:
                v = v / self.noisevec[None, :]
                vT = vT / self.noisevec[:, None]
            self._typed[dtype] = (v.to(dtype).contiguous(), vT.to(dtype).contiguous(),
                                  self.mywt.to(dtype).contiguous())
        return self._typed[dtype]

    def drop_operands(self, dtype: torch.dtype):
        self._typed.pop(dtype, None)

    def apply_noise(self, dat, out: Optional[torch.Tensor] = None, rot_mode: int = 0):
        """dd = halve_ends(vT . DCT1(mywt * DCT1(v . dat)))  (noise.py:680-714).
        Returns a new array of the input's kind unless ``out`` is given."""
        is_np = not isinstance(dat, torch.Tensor)
        d = as_device(dat, torch.float64 if is_np else None, self.v.device)
        v, vT, w = self.operands(d.dtype)
        plan = noise_plan(d.shape[0], d.shape[1], d.dtype, d.device)
        res = plan.apply(v, vT, w, d, out=out, rot_mode=rot_mode)
        return res.cpu().numpy() if is_np else res

    def get_det_weights(self) -> torch.Tensor:
        """2 * diag(vT diag(sum_k mywt) v)  (noise.py:761-772)."""
        mode_wt = torch.sum(self.mywt, dim=1)
        tmp = self.vT @ (mode_wt[:, None] * self.v)
        return torch.diagonal(tmp).clone() * 2.0
