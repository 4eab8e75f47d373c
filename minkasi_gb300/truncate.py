"""TOD length truncation to transform-friendly sizes (host side).

Restates find_good_fft_lens (minkasi/tools/py_fft.py:300-395) and
truncate_tod (minkasi/tods/processing.py:648-682): the TOD is cut to
m + 1 samples, m the largest {2,3,5,7,11}-smooth number the reference's
log-space enumeration finds below ndata - 1, so the DCT-I's FFT length
2(n-1) = 2m factors into small primes.
"""
from __future__ import annotations

from typing import Sequence

import numpy as np


def find_good_fft_lens(n: int, primes: Sequence[int] = (2, 3, 5, 7)) -> np.ndarray:
    lp = np.log2(np.asarray(primes, dtype=float))
    r = np.log2(n + 0.5)
    out = []

    def rec(level: int, lcur: float):
        if level == len(lp) - 1:
            out.extend(np.arange(lcur, r + 1e-3, lp[level]).tolist())
            return
        for fac in np.arange(lcur, r, lp[level]):
            rec(level + 1, fac)

    rec(0, 0.0)
    return np.sort(np.asarray(np.round(2 ** np.asarray(out)), dtype=int))


def truncated_length(ndata: int, primes: Sequence[int] = (2, 3, 5, 7, 11)) -> int:
    new = int(find_good_fft_lens(ndata - 1, primes).max()) + 1
    return new if new < ndata else ndata


def truncate_tod(tod_info: dict, primes: Sequence[int] = (2, 3, 5, 7, 11)) -> None:
    """Cut every array in tod_info whose axis matches ndata (in place on the dict)."""
    if "dat_calib" not in tod_info:
        return
    if len(tod_info["dat_calib"].shape) != 2:
        raise ValueError("dat_calib not 2d")
    ndata = tod_info["dat_calib"].shape[1]
    ndata_new = truncated_length(ndata, primes)
    if ndata_new >= ndata:
        return
    for key in list(tod_info.keys()):
        val = tod_info[key]
        if not hasattr(val, "shape") or len(val.shape) == 0:
            continue
        axes = [i for i, s in enumerate(val.shape) if s == ndata]
        if not axes:
            continue
        sl = [slice(None)] * len(val.shape)
        sl[axes[0]] = slice(0, ndata_new)
        tod_info[key] = val[tuple(sl)]
