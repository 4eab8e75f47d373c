"""Per-TOD model members of a Mapset, on the GPU: cuts and timestream models.

Mirrors minkasi/tods/cuts.py (CutsCompact, segs_from_vec) and
minkasi/mapmaking/timestream.py (tsGeneric, tsStripes, tsBinnedAz, tsModel,
partition_interval, split_partitioned_vec).  Their parameters are CUDA
tensors; the projections run the mk_cuts_*, mk_stripes_* and mk_binned_*
kernels, and dot products use the library's reproducible FP64 reduction.
Segment and index bookkeeping (which samples are cut, where stripes start)
is set-up work on small host arrays, as in the reference.
"""
from __future__ import annotations

import copy
from typing import Dict, List, Optional, Tuple

import numpy as np
import torch

from . import kernels as K
from . import parallel
from .maps import _reducer, as_device


def _dot(a: torch.Tensor, b: torch.Tensor) -> float:
    if a.numel() == 0:
        return 0.0
    return float(_reducer(a.device).dot(a.reshape(-1), b.reshape(-1)).item())


def _tod_dat(tod, dat, dtype=torch.float64) -> torch.Tensor:
    d = tod.get_data() if dat is None else dat
    return d if isinstance(d, torch.Tensor) and d.is_cuda else as_device(d, dtype)


def _device() -> torch.device:
    return torch.device("cuda", torch.cuda.current_device())


# ---------------------------------------------------------------- cuts
def segs_from_vec(vec, pad: bool = True) -> Tuple[int, List[int], List[int]]:
    """Start/stop indices of the False runs of vec (cuts.py:19-57)."""
    vec = np.asarray(vec)
    if pad:
        vv = np.ones(len(vec) + 2, dtype="bool")
        vv[1:-1] = vec
    else:
        vv = vec.astype(bool)
    if vv.all():
        return 0, [], []
    inds = np.where(np.diff(vv))[0]
    assert len(inds) % 2 == 0
    return len(inds) // 2, list(inds[::2]), list(inds[1::2])


class CutsCompact:
    """Cut samples of a TOD as one parameter per sample (cuts.py:201-490).

    ``imap`` (int64, device) holds the flat sample index of every cut sample,
    ``map`` (FP64, device) its value.  Each detector keeps its own segment
    lists (the reference initialises them as ``[[]] * ndet``, one shared
    list, so its add_cut appends a cut to every detector)."""

    def __init__(self, tod):
        if isinstance(tod, CutsCompact):
            self.ndet, self.nseg, self.imax = tod.ndet, tod.nseg.copy(), tod.imax
            self.istart, self.istop = list(tod.istart), list(tod.istop)
            dev = tod.map.device
        else:
            self.ndet = tod.get_ndet()
            self.nseg = np.zeros(self.ndet, dtype="int")
            self.imax = tod.get_ndata()
            self.istart = [[] for _ in range(self.ndet)]
            self.istop = [[] for _ in range(self.ndet)]
            dev = _device()
        self.imap = torch.zeros(0, dtype=torch.int64, device=dev)
        self.map = torch.zeros(0, dtype=torch.float64, device=dev)

    @property
    def dtype(self) -> torch.dtype:
        return self.map.dtype

    def copy(self, deep: bool = True) -> "CutsCompact":
        c = CutsCompact(self)
        c.imap = self.imap.clone() if deep else self.imap
        c.map = self.map.clone() if deep else self.map
        return c

    def add_cut(self, det: int, istart: int, istop: int):
        if istart >= self.imax:
            return
        istop = min(istop, self.imax)
        self.nseg[det] += 1
        self.istart[det] = list(self.istart[det]) + [istart]
        self.istop[det] = list(self.istop[det]) + [istop]

    def cuts_from_array(self, cutmat):
        """Cuts where cutmat (ndet, imax) is False (cuts.py:296-310)."""
        cutmat = cutmat.detach().cpu().numpy() if isinstance(cutmat, torch.Tensor) else np.asarray(cutmat)
        for det in range(cutmat.shape[0]):
            nseg, istart, istop = segs_from_vec(cutmat[det, :])
            self.nseg[det], self.istart[det], self.istop[det] = nseg, istart, istop

    def merge_cuts(self):
        """Merge overlapping cuts of each detector (cuts.py:312-328)."""
        tmp = np.ones(self.imax + 2, dtype="bool")
        for det in range(self.ndet):
            if self.nseg[det] < 2:
                continue
            tmp[:] = True
            for a, b in zip(self.istart[det], self.istop[det]):
                tmp[a + 1:b + 1] = False
            self.nseg[det], self.istart[det], self.istop[det] = segs_from_vec(tmp, pad=False)

    def get_imap(self):
        """Flat indices of the cut samples, detector by detector, segment by
        segment (cuts.py:330-349), and a zeroed map."""
        parts = [np.arange(det * self.imax + a, det * self.imax + b, dtype=np.int64)
                 for det in range(self.ndet) for a, b in zip(self.istart[det], self.istop[det])]
        imap = np.concatenate(parts) if parts else np.zeros(0, dtype=np.int64)
        dev = self.map.device
        self.imap = torch.from_numpy(imap).to(dev)
        self.map = torch.zeros(imap.size, dtype=torch.float64, device=dev)

    def tod2map(self, tod, mat=None, do_add: bool = True, do_omp: bool = False):
        """map (+)= TOD samples at imap (tod2cuts)."""
        if mat is None and tod is None:
            raise ValueError("Both tod and mat cannot be none")
        d = _tod_dat(tod, mat, self.map.dtype)
        K.cuts_gather(self.map, d.contiguous(), self.imap, do_add)

    def map2tod(self, tod, mat=None, do_add: bool = True, do_omp: bool = False):
        """TOD samples at imap (+)= map (cuts2tod)."""
        if mat is None and tod is None:
            raise ValueError("Both tod and mat cannot be none")
        d = _tod_dat(tod, mat, self.map.dtype)
        if not d.is_contiguous():
            raise ValueError("the TOD array must be C-contiguous")
        K.cuts_scatter(d, self.map, self.imap, do_add)

    def clear(self):
        self.map.zero_()

    def dot(self, other: Optional["CutsCompact"] = None) -> float:
        return _dot(self.map, (self if other is None else other).map)

    def axpy(self, common: "CutsCompact", a: float):
        K.axpy(self.map, common.map, float(a))

    def apply_prior(self, x, Ax):
        """Ax.map += self.map * x.map (cuts.py:459-474)."""
        if self.map is None:
            return
        Ax.map = Ax.map + self.map * x.map

    def write(self, fname=None):
        pass

    def __mul__(self, to_mul: "CutsCompact") -> "CutsCompact":
        tt = self.copy()
        tt.map = self.map * to_mul.map
        return tt

    def get_caches(self):
        pass

    def clear_caches(self):
        pass

    def mpi_reduce(self):
        pass


# ---------------------------------------------------------------- timestream models
def partition_interval(start: int, stop: int, seg_len: int = 100, round_up: bool = False) -> np.ndarray:
    """Edges of near-equal segments of about seg_len covering [start, stop)
    (timestream.py:442-459)."""
    if (stop - start) <= seg_len:
        return np.asarray([start, stop], dtype="int")
    nseg = (stop - start) // seg_len
    if nseg * seg_len < (stop - start) and round_up:
        nseg = nseg + 1
    seg_len = (stop - start) // nseg
    nextra = (stop - start) - seg_len * nseg
    inds = np.arange(start, stop + 1, seg_len)
    if nextra > 0:
        vec = np.zeros(len(inds), dtype="int")
        vec[1:nextra + 1] = 1
        inds = inds + np.cumsum(vec)
    return inds


def split_partitioned_vec(start: int, stop: int, breaks=(), seg_len: int = 100) -> np.ndarray:
    """Segment edges that also break at the given sample indices
    (timestream.py:462-483)."""
    breaks = list(breaks)
    if len(breaks) == 0:
        return partition_interval(start, stop, seg_len)
    if breaks[0] == start:
        breaks = breaks[1:]
        if len(breaks) == 0:
            return partition_interval(start, stop, seg_len)
    if breaks[-1] == stop:
        breaks = breaks[:-1]
        if len(breaks) == 0:
            return partition_interval(start, stop, seg_len)
    breaks = np.hstack([start, breaks, stop])
    segs = []
    for i in range(len(breaks) - 1):
        inds = partition_interval(breaks[i], breaks[i + 1], seg_len)
        segs.append(inds[:-1] if i < len(breaks) - 2 else inds)
    return np.hstack(segs)


class tsGeneric:
    """Parameters ``params`` (CUDA tensor) with the vector-space operations
    of a Mapset member (timestream.py:36-103)."""

    def __init__(self, tod=None):
        self.fname = tod.info["fname"] if tod is not None else None

    @property
    def dtype(self) -> torch.dtype:
        return self.params.dtype

    def __mul__(self, to_mul):
        tt = self.copy()
        tt.params = self.params * to_mul.params
        return tt

    def clear(self):
        self.params.zero_()

    def dot(self, common=None) -> float:
        return _dot(self.params, (self if common is None else common).params)

    def axpy(self, common, a: float):
        K.axpy(self.params, common.params, float(a))

    def apply_prior(self, x, Ax):
        Ax.params = Ax.params + self.params * x.params

    def copy(self):
        return copy.deepcopy(self)

    def write(self, fname=None):
        pass

    def get_caches(self):
        pass

    def clear_caches(self):
        pass

    def mpi_reduce(self):
        pass


class tsStripes(tsGeneric):
    """Destriper: one offset per detector per segment of about seg_len
    samples, segments also broken at time gaps > tthresh sample intervals
    (timestream.py:486-531)."""

    def __init__(self, tod, seg_len: int = 500, do_slope: bool = False, tthresh: float = 10):
        super().__init__(tod)
        dims = tod.get_data_dims()
        tvec = tod.get_tvec()
        tvec = tvec.detach().cpu().numpy() if isinstance(tvec, torch.Tensor) else np.asarray(tvec)
        dt = np.median(np.diff(tvec))
        splits = np.where(np.abs(np.diff(tvec)) > tthresh * dt)[0]
        inds = split_partitioned_vec(0, dims[1], splits, seg_len)
        self.inds = inds
        self.splits = splits
        self.nseg = len(inds) - 1
        dev = _device()
        self._lims = torch.from_numpy(np.asarray(inds, dtype=np.int64)).to(dev)
        self.params = torch.zeros((dims[0], self.nseg), dtype=torch.float64, device=dev)

    def tod2map(self, tod, dat=None, do_add: bool = True, do_omp: bool = False):
        if dat is None:
            print("need dat in tod2map destriper")
            return
        K.stripes_tod2map(self.params, _tod_dat(tod, dat, self.params.dtype).contiguous(), self._lims, do_add)

    def map2tod(self, tod, dat=None, do_add: bool = True, do_omp: bool = False):
        if dat is None:
            print("need dat in map2tod destriper")
            return
        K.stripes_map2tod(_tod_dat(tod, dat, self.params.dtype), self.params, self._lims, do_add)

    def set_prior_from_corr(self, corrvec, thresh: float = 0.5):
        """Inverse-spectrum prior from a correlation vector (timestream.py:516-526),
        with the DCT-I of libmkgpu."""
        corr = as_device(corrvec, torch.float64)
        assert corr.shape[0] == self.params.shape[0]
        n = self.params.shape[1]
        corr = corr[:, :n].contiguous()
        corrft = K.DCT1(corr.shape[0], n, torch.float64, corr.device)(corr)
        if thresh > 0:
            # numpy's median (the mean of the two middle values for even n)
            tt = thresh * torch.quantile(corrft, 0.5, dim=1, keepdim=True)
            corrft = torch.where(corrft < tt, tt.expand_as(corrft), corrft)
        self.params = 1.0 / corrft / (2 * (n - 1))

    def apply_prior(self, x, Ax):
        d = K.DCT1(x.params.shape[0], x.params.shape[1], torch.float64, x.params.device)
        Ax.params = Ax.params + d((d(x.params.contiguous()) * self.params).contiguous())


class tsBinnedAz(tsGeneric):
    """Per-detector offsets binned in azimuth, tod.info['az'] (timestream.py:533-560)."""

    def __init__(self, tod, lims=(0, 2 * np.pi), nbin: int = 360):
        self.fname = tod.info.get("fname")
        self.params = torch.zeros((tod.get_ndet(), nbin), dtype=torch.float64, device=_device())
        self.lims = (lims[0], lims[1])
        self.nbin = nbin

    def map2tod(self, tod, dat=None, do_add: bool = True, do_omp: bool = False):
        d = _tod_dat(tod, dat, self.params.dtype)
        K.binned_map2tod(d, self.params, as_device(tod.info["az"], torch.float64), self.lims, do_add)

    def tod2map(self, tod, dat=None, do_add: bool = True, do_omp: bool = False):
        d = _tod_dat(tod, dat, self.params.dtype)
        K.binned_tod2map(self.params, d.contiguous(), as_device(tod.info["az"], torch.float64), self.lims,
                         do_add)


class tsModel:
    """Per-TOD models keyed by tod.info['fname'] (timestream.py:842-928)."""

    def __init__(self, todvec=None, modelclass=None, *args, **kwargs):
        self.data: Dict[str, tsGeneric] = {}
        if todvec is None:
            return
        for tod in todvec.tods:
            self.data[tod.info["fname"]] = modelclass(tod, *args, **kwargs)

    @property
    def dtype(self) -> torch.dtype:
        return torch.float64

    def copy(self) -> "tsModel":
        new = tsModel()
        for nm, v in self.data.items():
            new.data[nm] = v.copy()
        return new

    def tod2map(self, tod, dat, do_add: bool = True, do_omp: bool = False):
        if not do_add:
            self.clear()
        self.data[tod.info["fname"]].tod2map(tod, dat, do_add, do_omp)

    def map2tod(self, tod, dat, do_add: bool = True, do_omp: bool = True):
        if not do_add:
            dat[:] = 0.0
        self.data[tod.info["fname"]].map2tod(tod, dat, do_add, do_omp)

    def apply_prior(self, x, Ax):
        for nm in self.data:
            self.data[nm].apply_prior(x.data[nm], Ax.data[nm])

    def dot(self, tsmodels: Optional["tsModel"] = None) -> float:
        tot = 0.0
        for nm, v in self.data.items():
            if tsmodels is None:
                tot += v.dot(v)
            else:
                if nm not in tsmodels.data:
                    raise KeyError(f"error in tsModel.dot - missing key {nm}")
                tot += v.dot(tsmodels.data[nm])
        return parallel.allreduce_scalar(tot)

    def clear(self):
        for v in self.data.values():
            v.clear()

    def axpy(self, tsmodel: "tsModel", a: float):
        for nm, v in self.data.items():
            v.axpy(tsmodel.data[nm], a)

    def __mul__(self, tsmodel: "tsModel") -> "tsModel":
        tt = self.copy()
        for nm in self.data:
            tt.data[nm] = self.data[nm] * tsmodel.data[nm]
        return tt

    def mpi_reduce(self):
        pass

    def get_caches(self):
        pass

    def clear_caches(self):
        pass
