"""Kernel micro-benchmarks on one synthetic TOD shape (CUDA events, best of N).

    python -m minkasi_gb300.kbench [--config c2s] [--only tod2map,map2tod,rot,noise,dct,conv,point,pol]
                                   [--shape NDET,NDATA]
    python -m minkasi_gb300.kbench --config c2 --only iter      # the whole operator (iter64: FP64 too)

Uses the first TOD shape and daisy pointing of a synthetic configuration
(default c2s: 256 detectors x 130978 samples onto a 1024x1024 map; --shape
overrides the TOD shape, e.g. 256,144278 for a length whose transform runs
Bluestein's algorithm) with random data, and reports per kernel the time and, for the projections, the
algorithmic GB/s (4 B pixel index + one sample per sample; the map is
L2-resident).  Rotations report their relative error against cuBLAS on the
FP64 / FP32 units and their TF/s counted as 2 ndet^2 ndata flops
(3 split products for the tensor-core 3xTF32 kernel are not counted).
Prints one JSON object.  This is also the command the ncu captures use.
"""
from __future__ import annotations

import argparse
import json

import torch

from . import kernels as K
from .synth import CONFIGS, make_tod_info, tod_shapes


def best_ms(fn, reps: int = 5, warm: int = 2) -> float:
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    best = float("inf")
    s = torch.cuda.current_stream()
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        fn()
        b.record(s)
        b.synchronize()
        best = min(best, a.elapsed_time(b))
    return best


def run(config: str = "c2s", only=None, shape=None) -> dict:
    dev = torch.device("cuda", torch.cuda.current_device())
    cfg = CONFIGS[config]
    ndet, n = shape if shape else tod_shapes(cfg)[0]
    info = make_tod_info(cfg, 0, ndet, n, dev, with_data=False)
    ipix = info["ipix"]
    npix = cfg.nx * cfg.ny
    N = ndet * n
    out = {"config": config, "ndet": ndet, "ndata": n, "npix": npix, "samples": N}
    want = set(only) if only else {"map2tod", "tod2map", "rot", "noise", "dct", "conv"}
    g = torch.Generator(device=dev).manual_seed(0)
    for dt, es in ((torch.float64, 8), (torch.float32, 4)):
        tag = "f64" if es == 8 else "f32"
        dat = torch.randn((ndet, n), generator=g, dtype=dt, device=dev)
        mp = torch.randn(npix, generator=g, dtype=dt, device=dev)
        if "map2tod" in want:
            d2 = torch.empty_like(dat)
            ms = best_ms(lambda: K.map2tod(d2, mp, ipix, False))
            out[f"map2tod_{tag}"] = {"ms": ms, "GBs": N * (4 + es) / ms / 1e6}
        if "tod2map" in want:
            acc = torch.zeros(npix, dtype=dt, device=dev)
            ms = best_ms(lambda: K.tod2map(acc, dat, ipix))
            out[f"tod2map_atomic_{tag}"] = {"ms": ms, "GBs": N * (4 + es) / ms / 1e6}
            ms = best_ms(lambda: K.tod2map_staged(acc, dat, ipix))
            out[f"tod2map_staged_{tag}"] = {"ms": ms, "GBs": N * (4 + es) / ms / 1e6}
            hits = torch.zeros(npix, dtype=torch.float64, device=dev)
            K.tod2map_rows(hits, ipix)
            hmax = int(hits.max().item())
            scr = K.FixedScratch(npix, dev)
            ms = best_ms(lambda: K.tod2map_fixed(acc, dat, ipix, hmax, scr))
            out[f"tod2map_fixed_{tag}"] = {"ms": ms, "GBs": N * (4 + es) / ms / 1e6}
            plan = K.PixPlan(ipix, npix)
            ms = best_ms(lambda: plan.tod2map(acc, dat))
            out[f"tod2map_sorted_{tag}"] = {"ms": ms, "GBs": N * (4 + es) / ms / 1e6}
            del plan
        plan = None
        if want & {"rot", "noise"}:
            plan = K.NoisePlan(ndet, n, dt, dev)
            A = torch.linalg.qr(torch.randn(ndet, ndet, dtype=torch.float64, device="cpu"))[0]
            A = A.to(dev).to(dt).contiguous()
        if "rot" in want:
            ref = plan.rotate(A, dat, rot_mode=1)
            for mode in ((1, 3, 4) if es == 8 else (1, 2, 3)):
                try:
                    y = plan.rotate(A, dat, rot_mode=mode)
                except K._lib.MkError as e:
                    out[f"rot{mode}_{tag}"] = {"error": str(e)[:120]}
                    continue
                err = float((y - ref).abs().max() / ref.abs().max())
                ms = best_ms(lambda m=mode: plan.rotate(A, dat, out=y, rot_mode=m))
                out[f"rot{mode}_{tag}"] = {"ms": ms, "TFs": 2 * ndet * ndet * n / ms / 1e9,
                                           "GBs": 2 * N * es / ms / 1e6, "rel_err_vs_blas": err}
        if "noise" in want:
            w = torch.rand((ndet, n), generator=g, dtype=dt, device=dev)
            o = torch.empty_like(dat)
            for mode in ((1, 4) if es == 8 else (1, 2)):
                try:
                    ms = best_ms(lambda m=mode: plan.apply(A, A.T.contiguous(), w, dat, out=o, rot_mode=m),
                                 reps=3)
                    out[f"apply_noise_rot{mode}_{tag}"] = {"ms": ms, "GBs_algorithmic": 3 * N * es / ms / 1e6}
                except K._lib.MkError as e:
                    out[f"apply_noise_rot{mode}_{tag}"] = {"error": str(e)[:120]}
        if "dct" in want:
            d = K.DCT1(ndet, n, dt, dev)
            o = torch.empty_like(dat)
            ms = best_ms(lambda: d(dat, out=o))
            out[f"dct1_{tag}"] = {"ms": ms}
            del d
        del plan
        torch.cuda.empty_cache()
    if "conv" in want:
        out.update(conv_bench(dev))
    if want & {"point", "pol"}:
        out.update(point_pol_bench(cfg, ndet, n, dev, want))
    return out


def iter_bench(config: str, dtypes=("f32",), reps: int = 3) -> dict:
    """The whole configuration's operator A x = P^T N P x, per precision:
    one application and its parts (map2tod over all TODs, the noise filter,
    tod2map), the filter both as the one-call group over all TODs and TOD by
    TOD, and the per-TOD filter time summed over TODs whose transform runs
    Bluestein's algorithm and over the others."""
    from . import synth
    dev = torch.device("cuda", torch.cuda.current_device())
    cfg = CONFIGS[config]
    tv, m = synth.make_todvec(cfg, dev)
    S = tv.get_nsamp()
    res = {"config": config, "samples": S, "ntod": len(tv.tods)}
    for tag in dtypes:
        dt = torch.float32 if tag == "f32" else torch.float64
        op = tv.engine(m, dt)
        op.prepare_noise()
        x = torch.randn(m.npix, dtype=dt, device=dev)
        y = torch.empty_like(x)
        r = {"rot_mode": op.rot_mode, "tod2map_kernel": op.method,
             "apply_ms": best_ms(lambda: op.apply(x, y), reps=reps, warm=1),
             "map2tod_ms": best_ms(lambda: K.map2tod(op.tmp, x, op.ipix, False), reps=reps, warm=1),
             "tod2map_ms": best_ms(lambda: op.project_out(y), reps=reps, warm=1)}
        grp = op._noise_group()
        if grp is not None:
            r["noise_group_ms"] = best_ms(grp.apply, reps=reps, warm=1)
        blue = smooth = 0.0
        nblue = 0
        for (v, vT, w), view, dims in zip(op.ops, op.views(op.tmp), op.dims):
            p = op.plans[dims]
            ms = best_ms(lambda: p.apply(v, vT, w, view, out=view, rot_mode=op.rot_mode), reps=2, warm=1)
            L1, L2 = p.split
            if L1 * L2 not in (0, 2 * (dims[1] - 1)):
                blue += ms
                nblue += 1
            else:
                smooth += ms
        r.update(noise_per_tod_ms=blue + smooth, noise_bluestein_ms=blue, noise_smooth_ms=smooth,
                 n_bluestein=nblue, dct_engines={f"{a}x{b}": e for (a, b), e in op.dct_engines.items()})
        # one more application inside an NVTX range, for a profiler's
        # launch list of exactly one operator application
        torch.cuda.synchronize()
        with torch.cuda.nvtx.range(f"apply_{tag}"):
            op.apply(x, y)
            torch.cuda.synchronize()
        res[tag] = r
        op.release()
        torch.cuda.empty_cache()
    return res


def point_pol_bench(cfg, ndet: int, n: int, dev, want) -> dict:
    """Pointing -> pixel (16 B of RA/dec read, 4 B written per sample) and
    the IQU projections with cached cos/sin 2gamma (4 B pixel + 16 B angle
    terms + 8 B sample per sample), FP64, on the configuration's first TOD."""
    info = make_tod_info(cfg, 0, ndet, n, dev, with_data=False, with_radec=True)
    ra, dec = info["dx"].contiguous(), info["dy"].contiguous()
    N = ndet * n
    res = {}
    if "point" in want:
        lims = [float(ra.min()), float(ra.max()), float(dec.min()), float(dec.max())]
        ps = cfg.pixsize_arcsec * torch.pi / 180 / 3600
        ny = int((lims[3] - lims[2]) / ps) + 3
        cosdec = float(torch.cos(torch.tensor(0.5 * (lims[2] + lims[3]), dtype=torch.float64)))
        out = torch.empty((ndet, n), dtype=torch.int32, device=dev)
        ms = best_ms(lambda: K.pix_car(ra, dec, lims[0], lims[2], ps, cosdec, ny, out=out))
        res["pix_car"] = {"ms": ms, "GBs": N * 20 / ms / 1e6}
        w6 = [lims[1] * 180 / torch.pi, lims[2] * 180 / torch.pi, 1.0, 1.0, -ps * 180 / torch.pi,
              ps * 180 / torch.pi]
        ms = best_ms(lambda: K.pix_wcs_car(ra, dec, w6, ny, out=out))
        res["pix_wcs_car"] = {"ms": ms, "GBs": N * 20 / ms / 1e6, "Gsamp_per_s": N / ms / 1e6}
    if "pol" in want:
        g = torch.Generator(device=dev).manual_seed(3)
        tg = torch.rand((ndet, n), generator=g, dtype=torch.float64, device=dev) * 6.283185307179586
        ms = best_ms(lambda: K.pol_sincos(tg))
        res["pol_sincos"] = {"ms": ms, "GBs": N * 24 / ms / 1e6}
        cs = K.pol_sincos(tg)
        ipix = info["ipix"]
        npix = cfg.nx * cfg.ny
        mp = torch.randn((npix, 3), generator=g, dtype=torch.float64, device=dev)
        dat = torch.empty((ndet, n), dtype=torch.float64, device=dev)
        ms = best_ms(lambda: K.polmap2tod(dat, mp, "IQU", cs, ipix, False))
        res["polmap2tod_iqu"] = {"ms": ms, "GBs": N * 28 / ms / 1e6}
        acc = torch.zeros((npix, 3), dtype=torch.float64, device=dev)
        ms = best_ms(lambda: K.tod2polmap(acc, dat, "IQU", cs, ipix))
        res["tod2polmap_iqu"] = {"ms": ms, "GBs": N * 28 / ms / 1e6}
        ms = best_ms(lambda: K.polmap2tod(dat, mp, "IQU", tg, ipix, False))
        res["polmap2tod_iqu_twogamma"] = {"ms": ms, "GBs": N * 20 / ms / 1e6}
    return res


def conv_bench(dev, hw: int = 2048, batch: int = 1, c: int = 16) -> dict:
    """The learned preconditioner's 3x3 convolutions on (batch, c, hw, hw)
    FP32 maps: fwd, adjoint and weight gradient of a c->c layer, counted as
    2 * 9 * c * c flops per pixel each."""
    from . import learned as L
    g = torch.Generator(device=dev).manual_seed(1)
    x = torch.randn((batch, c, hw, hw), generator=g, dtype=torch.float32, device=dev)
    w = torch.randn((c, c, 3, 3), generator=g, dtype=torch.float32, device=dev) * 0.1
    h = torch.randn_like(x)
    flops = 2 * 9 * c * c * batch * hw * hw
    res = {}
    for name, fn in (("conv_fwd", lambda: L.conv_fwd(x, w)), ("conv_adj", lambda: L.conv_adj(h, w)),
                     ("conv_wgrad", lambda: L.conv_wgrad(x, h))):
        ms = best_ms(fn)
        res[name] = {"ms": ms, "TFLOPs": flops / ms / 1e9, "shape": [batch, c, hw, hw]}
    res["precon_small"] = precon_bench(dev)
    res["precon_2048"] = precon_bench(dev, hw=2048)
    return res


def precon_bench(dev, hw: int = 256) -> dict:
    """z = M r of the learned preconditioner on an hw x hw FP64 map (the
    1 -> 16 -> 16 -> 16 -> 16 network, 8 convolutions), as the PCG runs it:
    replayed from a CUDA graph.  Also each convolution shape alone."""
    from . import learned as L
    net = L.ConvNet.init(seed=0, device=dev)
    hits = torch.rand((hw, hw), dtype=torch.float64, device=dev) * 100 + 1
    M = L.LearnedPrecon(hits, net, (hw, hw))
    r = torch.randn(hw * hw, dtype=torch.float64, device=dev)
    z = torch.empty_like(r)
    M.apply(r, z)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        M.apply(r, z)
    res = {"shape": [hw, hw], "apply_graph_ms": best_ms(g.replay, reps=20),
           "apply_eager_ms": best_ms(lambda: M.apply(r, z), reps=20)}
    x1 = torch.randn((1, 1, hw, hw), dtype=torch.float32, device=dev)
    x16 = torch.randn((1, 16, hw, hw), dtype=torch.float32, device=dev)
    w0, w1 = net.weights[0], net.weights[1]
    for name, fn in (("fwd_1_16", lambda: L.conv_fwd(x1, w0)), ("fwd_16_16", lambda: L.conv_fwd(x16, w1)),
                     ("adj_16_16", lambda: L.conv_adj(x16, w1)), ("adj_16_1", lambda: L.conv_adj(x16, w0))):
        res[name + "_ms"] = best_ms(fn, reps=20)
    return res


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="c2s")
    ap.add_argument("--only", default="")
    ap.add_argument("--shape", default="", help="NDET,NDATA instead of the configuration's first TOD")
    a = ap.parse_args()
    shape = tuple(int(v) for v in a.shape.split(",")) if a.shape else None
    only = [s for s in a.only.split(",") if s] or None
    if only and only[0] in ("iter", "iter64"):
        print(json.dumps(iter_bench(a.config, ("f32", "f64") if only[0] == "iter64" else ("f32",))))
    else:
        print(json.dumps(run(a.config, only, shape)))
