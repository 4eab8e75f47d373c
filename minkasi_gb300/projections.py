"""Module-level projection functions and hit maps, mirroring
minkasi/mapmaking/map2tod.py:19-54 and minkasi/mapmaking/tod2map.py:29-400.

All of them take CUDA tensors (or numpy arrays, copied to the device and the
result copied back into the caller's array, like the reference's in-place
contract) and run libmkgpu kernels.  ``do_omp`` and the reference's choice of
CPU strategy (omp / simple / atomic / cached / everyone) map onto the GPU
kernels: one warp-aggregated atomic scatter by default, or a bitwise
reproducible variant via ``deterministic=True``.
"""
from __future__ import annotations

from typing import Optional

import numpy as np
import torch

from . import kernels as K
from .maps import SkyMap, as_device


def _inplace(arr, fn, dtype=None):
    if isinstance(arr, torch.Tensor):
        fn(arr)
        return arr
    d = as_device(arr, dtype)
    fn(d)
    np.copyto(arr, d.cpu().numpy())
    return arr


def map2tod(dat, map, ipix, do_add: bool = False, do_omp: bool = True):
    """dat (+)= map.flat[ipix] in place (map2tod.py:19-54)."""
    m = as_device(map)
    ip = as_device(ipix, torch.int32)
    _inplace(dat, lambda d: K.map2tod(d, m.reshape(-1).to(d.dtype), ip, do_add))


def tod2map_omp(map, dat, ipix, atomic: bool = False, deterministic: bool = False):
    """map.flat[ipix] += dat in place (tod2map.py:97-128)."""
    d = as_device(dat)
    ip = as_device(ipix, torch.int32)

    def run(m):
        mf = m.reshape(-1)
        dd = d.to(mf.dtype)
        if deterministic:
            hmax = max(int(torch.bincount(ip.reshape(-1).long(), minlength=mf.numel()).max().item()), 1)
            K.tod2map_fixed(mf, dd, ip, hmax, K.FixedScratch(mf.numel(), mf.device))
        else:
            K.tod2map(mf, dd, ip)

    _inplace(map, run)


def tod2map_simple(map, dat, ipix):
    """Serial-order scatter in the reference (tod2map.py:29-53); here the
    reproducible fixed-point scatter, which gives one answer for any order."""
    tod2map_omp(map, dat, ipix, deterministic=True)


tod2map_atomic = tod2map_omp
tod2map_cached = tod2map_omp


def make_hits(todvec, map: SkyMap, do_weights: bool = False) -> SkyMap:
    """Hit (or detector-weight) map summed over TODs and ranks
    (tod2map.py:343-400), without materialising a TOD of ones."""
    hits = map.copy()
    pol = getattr(map, "npol", 1) > 1
    if pol:
        hits.set_polstate(map.poltag + "_PRECON")  # PolMap: the per-pixel Stokes matrices
    hits.clear()
    flat = hits.map.reshape(-1)
    for tod in todvec.tods:
        ip = map.get_pix(tod)
        w = None
        if do_weights:
            w = tod.get_det_weights()
            if w is None:
                print("error in making weight map.  Detector weights requested, but do not appear "
                      "to be present.  Do you have a noise model?")
            else:
                w = as_device(w, flat.dtype)
        if "mask" in tod.info:
            msk = as_device(tod.info["mask"], flat.dtype)
            tmp = msk if w is None else msk * w[:, None]
            hits.tod2map(tod, tmp.contiguous())
        elif pol:
            hits.tod2map_rows(tod, w)
        else:
            K.tod2map_rows(flat, ip, w)
    hits.mpi_reduce()
    return hits


def jacobi_precon(hits: SkyMap):
    """The hits preconditioner of the reference's example scripts
    (examples/minkasi_mpi_example.py:99-105): 1/hits on hit pixels, else 0."""
    from .maps import Mapset

    p = hits.copy()
    p.invert()
    ms = Mapset()
    ms.add_map(p)
    return ms
