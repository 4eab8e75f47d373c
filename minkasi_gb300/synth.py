"""Seeded synthetic TODs for the benchmark configurations (generated on the GPU).

The reference has no scan simulator; its configurations are described by
their shapes and physics, which this module turns into data:

* pointing: a daisy scan r = R sin(w1 t), theta = w2 t around a scan centre
  (or, for the sparse variant, raster sweeps along a few fixed rows),
  detectors on a square grid at ``det_pitch`` arcsec, flat-sky CAR pixels
  (ipix = x * ny + y, int32, the reference's layout);
* signal: a beta-model cluster amp (1 + r^2/theta_c^2)^(0.5 - 1.5 beta) at
  the map centre (the isothermal beta profile of minkasi/lib/minkasi.c:321-339);
* noise: white (sigma), 1/f with a knee frequency and PSD slope, and a
  common mode shared by all detectors (1/f spectrum, per-detector gains);
* lengths: nsamp drawn uniformly in a range, then truncated to an
  FFT-friendly length exactly as minkasi.tods.processing.truncate_tod does.

Choices the configurations leave open are fixed here and recorded in
``SynthConfig``: beta = 2/3, common-mode rms 3 mK, daisy periods 22 s and
22 * 1.618 s, detector gain scatter 2%.
"""
from __future__ import annotations

import math
from dataclasses import asdict, dataclass, field, replace
from typing import List, Optional, Sequence, Tuple

import numpy as np
import torch

from .truncate import truncated_length

ARCSEC = math.pi / 180 / 3600


@dataclass(frozen=True)
class SynthConfig:
    name: str = "custom"
    ntod: int = 1
    ndet_choices: Tuple[int, ...] = (64,)
    nsamp_range: Tuple[int, int] = (65536, 65536)
    nx: int = 256
    ny: int = 256
    pixsize_arcsec: float = 2.0
    det_pitch_arcsec: float = 10.0
    scan_radius_arcmin: float = 3.0
    centre_spread_arcmin: float = 0.0     # scan centres drawn uniformly in this radius
    fsamp: float = 180.0
    petal_period_s: float = 22.0
    beta: float = 2.0 / 3.0
    amp: float = -1e-3                    # K
    theta_c_arcsec: float = 30.0
    white: float = 1e-3                   # K rms per sample
    knee_hz: float = 1.0
    psd_slope: float = -2.0
    cm_rms: float = 3e-3                  # K
    gain_scatter: float = 0.02
    truncate: bool = True
    seed: int = 0
    # "daisy", or "raster": constant-declination sweeps x = L sin(w1 t) along
    # one of `tracks` fixed rows spread over +-centre_spread (every TOD
    # retraces one of them), so the hit pixels are a few narrow bands
    scan: str = "daisy"
    tracks: int = 0


CONFIGS = {
    # the reference's CPU-runnable configuration (1 TOD, 64 x 65536, 256^2 map at 2")
    "c1": SynthConfig(name="c1", ntod=1, ndet_choices=(64,), nsamp_range=(65536, 65536),
                      nx=256, ny=256, pixsize_arcsec=2.0),
    # plain method at GPU scale: 32 TODs x 256 det x U[2^17, 2^19], 1024^2 map at 1"
    "c2": SynthConfig(name="c2", ntod=32, ndet_choices=(256,), nsamp_range=(1 << 17, 1 << 19),
                      nx=1024, ny=1024, pixsize_arcsec=1.0),
    # batching: 200 TODs, ndet in {32,64,128,256}, nsamp U[5e4, 6e5], 2048^2 map,
    # scan centres spread over the field so the hit pattern is sparse
    "c4": SynthConfig(name="c4", ntod=200, ndet_choices=(32, 64, 128, 256),
                      nsamp_range=(50000, 600000), nx=2048, ny=2048, pixsize_arcsec=0.5,
                      scan_radius_arcmin=1.5, centre_spread_arcmin=4.5),
    # c4 with sparse hits: raster sweeps that retrace 3 narrow tracks, so
    # about 5% of the pixels inside the scan footprint are hit
    "c4sparse": SynthConfig(name="c4sparse", ntod=200, ndet_choices=(32, 64, 128, 256),
                            nsamp_range=(50000, 600000), nx=2048, ny=2048, pixsize_arcsec=0.5,
                            scan_radius_arcmin=6.0, centre_spread_arcmin=6.0, det_pitch_arcsec=5.0,
                            scan="raster", tracks=3),
    # a small case of c2 for profiler captures: 4 TODs x 256 x 2^17 (1.6 GB of inputs)
    "c2s": SynthConfig(name="c2s", ntod=4, ndet_choices=(256,), nsamp_range=(1 << 17, 1 << 17),
                       nx=1024, ny=1024, pixsize_arcsec=1.0),
    # small cases for tests
    "tiny": SynthConfig(name="tiny", ntod=2, ndet_choices=(8, 16), nsamp_range=(3000, 5000),
                        nx=64, ny=64, pixsize_arcsec=4.0, scan_radius_arcmin=1.5),
}


def tod_shapes(cfg: SynthConfig) -> List[Tuple[int, int]]:
    """(ndet, ndata) of every TOD, drawn from the config's seed (host side)."""
    rng = np.random.default_rng(cfg.seed)
    out = []
    for _ in range(cfg.ntod):
        ndet = int(rng.choice(cfg.ndet_choices))
        n = int(rng.integers(cfg.nsamp_range[0], cfg.nsamp_range[1] + 1))
        if cfg.truncate:
            n = truncated_length(n)
        out.append((ndet, n))
    return out


def det_offsets(ndet: int, pitch: float) -> np.ndarray:
    """(ndet, 2) offsets in arcsec on the most square grid with ndet cells."""
    nr = int(math.isqrt(ndet))
    while ndet % nr:
        nr -= 1
    nc = ndet // nr
    gx, gy = np.meshgrid((np.arange(nr) - (nr - 1) / 2) * pitch, (np.arange(nc) - (nc - 1) / 2) * pitch,
                         indexing="ij")
    return np.stack([gx.ravel(), gy.ravel()], axis=1)


def _one_over_f(gen: torch.Generator, nrow: int, n: int, cfg: SynthConfig, device) -> torch.Tensor:
    """Gaussian noise with PSD ~ 1 + (f_knee/f)^(-slope), unit white level."""
    w = torch.randn((nrow, n), generator=gen, dtype=torch.float64, device=device)
    f = torch.fft.rfftfreq(n, d=1.0 / cfg.fsamp, device=device, dtype=torch.float64)
    f[0] = f[1]
    amp = torch.sqrt(1.0 + (cfg.knee_hz / f) ** (-cfg.psd_slope))
    return torch.fft.irfft(torch.fft.rfft(w) * amp, n=n)


def make_tod_info(cfg: SynthConfig, k: int, ndet: int, ndata: int, device,
                  with_data: bool = True, with_radec: bool = True) -> dict:
    """info dict of TOD k: 'ipix' (int32, device), 'dat_calib' (float64,
    device) and the RA/dec offsets 'dx', 'dy' in radians."""
    gen = torch.Generator(device=device)
    gen.manual_seed(cfg.seed * 100003 + k)
    rng = np.random.default_rng(cfg.seed * 7919 + k)
    t = torch.arange(ndata, device=device, dtype=torch.float64) / cfg.fsamp
    R = cfg.scan_radius_arcmin * 60.0
    w1 = 2 * math.pi / cfg.petal_period_s
    w2 = w1 / 1.6180339887
    ph1, ph2 = rng.uniform(0, 2 * math.pi, size=2)
    off = torch.from_numpy(det_offsets(ndet, cfg.det_pitch_arcsec)).to(device)
    if cfg.scan == "raster":
        # sweep along x over +-R; the row is one of `tracks` fixed rows
        track = int(rng.integers(0, max(cfg.tracks, 1)))
        spread = cfg.centre_spread_arcmin * 60.0
        cy = -spread + 2 * spread * (track + 0.5) / max(cfg.tracks, 1)
        x = (R * torch.sin(w1 * t + ph1))[None, :] + off[:, :1]
        y = torch.full_like(t, cy)[None, :] + off[:, 1:]
    else:
        r = R * torch.sin(w1 * t + ph1)
        th = w2 * t + ph2
        if cfg.centre_spread_arcmin > 0:
            rr = cfg.centre_spread_arcmin * 60.0 * math.sqrt(rng.uniform())
            aa = rng.uniform(0, 2 * math.pi)
            cx, cy = rr * math.cos(aa), rr * math.sin(aa)
        else:
            cx = cy = 0.0
        x = (cx + r * torch.cos(th))[None, :] + off[:, :1]      # arcsec from map centre
        y = (cy + r * torch.sin(th))[None, :] + off[:, 1:]
    px = torch.round(x / cfg.pixsize_arcsec + cfg.nx / 2).clamp(0, cfg.nx - 1)
    py = torch.round(y / cfg.pixsize_arcsec + cfg.ny / 2).clamp(0, cfg.ny - 1)
    ipix = (px * cfg.ny + py).to(torch.int32).contiguous()
    info = {"ipix": ipix}
    if with_radec:  # 16 B per sample: skipped for the largest configurations
        info["dx"], info["dy"] = x * ARCSEC, y * ARCSEC
    if with_data:
        rad2 = x * x + y * y
        sig = cfg.amp * (1 + rad2 / cfg.theta_c_arcsec ** 2) ** (0.5 - 1.5 * cfg.beta)
        noise = cfg.white * _one_over_f(gen, ndet, ndata, cfg, device)
        cm = cfg.cm_rms * _one_over_f(gen, 1, ndata, cfg, device)
        cm = cm / cm.std()
        gains = 1 + cfg.gain_scatter * torch.randn((ndet, 1), generator=gen, dtype=torch.float64,
                                                   device=device)
        info["dat_calib"] = (sig + noise + gains * cm).contiguous()
    else:
        info["dat_calib"] = torch.empty((ndet, ndata), dtype=torch.float64, device="meta")
    return info


def make_todvec(cfg: SynthConfig, device=None, noise: bool = True, fwhm: float = 50.0,
                keep_data: bool = True, progress: bool = False):
    """Build (TodVec, SkyMap) for a configuration; noise models on the GPU."""
    from .maps import SkyMap
    from .noise import NoiseSmoothedSVD
    from .tods import Tod, TodVec

    device = device or torch.device("cuda", torch.cuda.current_device())
    tv = TodVec()
    for k, (ndet, n) in enumerate(tod_shapes(cfg)):
        info = make_tod_info(cfg, k, ndet, n, device)
        tod = Tod(info)
        if noise:
            tod.set_noise(NoiseSmoothedSVD, fwhm=fwhm)
        if not keep_data:
            tod.info["dat_calib"] = tod.info["dat_calib"].to("meta")
        tv.add_tod(tod)
        if progress and (k + 1) % 10 == 0:
            print(f"  generated {k + 1}/{cfg.ntod} TODs", flush=True)
    m = SkyMap(nx=cfg.nx, ny=cfg.ny, device=device)
    return tv, m


def config_dict(cfg: SynthConfig) -> dict:
    return asdict(cfg)
