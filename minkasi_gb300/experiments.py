"""Solver experiments on the benchmark configurations (time to an FP64
residual, map error per refinement step, learned vs Jacobi).

    python -m minkasi_gb300.experiments --config c1 --tol 1e-6 [--no-learned] [--pairs 5000]
    python -m minkasi_gb300.experiments --config c4 --large [--no-learned] [--wall 600]

The --large form is the 200-TOD batching run (run_large): per-iteration
times of FP64 Jacobi PCG and of the mixed-precision PCG, the mixed solve to
tol, and (unless --no-learned) the learned preconditioner trained on pairs
from PCG runs on b = A s with known synthetic skies s, then the mixed solve
with it.

For one synthetic configuration this builds the TODs and noise models on the
GPU, the FP64 right-hand side b = sum P^T N d, the hit map and the Jacobi
preconditioner, a "truth" map (FP64 Jacobi PCG to 1e-10), and then times,
from x0 = 0 to ||b - A x||/||b|| <= tol with A the FP64 operator:

  jacobi_f64     : run_pcg, FP64 operator, Jacobi (the plain method)
  mixed_jacobi   : run_pcg_mixed: FP32 operator, FP64 vectors/dots, FP64 residual
                   replacement every 50 iterations (the refinement steps)
  refine20       : classic iterative refinement, FP32 inner PCG of 20 iterations
                   restarted from zero each outer step (bounded at 60 outer steps)
  mixed_learned  : the same with the learned SPD preconditioner in the inner solve
  learned_f64    : FP64 PCG with the learned preconditioner

Every wall time brackets the solve only (operators, autotuning and training
happen before), with torch.cuda.synchronize() on both sides; wall_s is the
second of two identical solves and cold_wall_s the first (graph captures,
lazy kernel loading).  inner_step_ms is one graph-replayed inner iteration.  Map errors are
against the truth map with the mean over hit pixels removed (A annihilates
a constant map, so that mean is undetermined).  Prints one JSON object.
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np
import torch

from . import learned as L
from .maps import Mapset
from .pcg import DevicePCG, MixedOp, run_pcg, run_pcg_mixed
from .projections import jacobi_precon, make_hits
from .synth import CONFIGS, make_todvec


def map_error(x: torch.Tensor, truth: torch.Tensor, hit: torch.Tensor) -> float:
    a = x.reshape(-1)[hit].double()
    b = truth.reshape(-1)[hit].double()
    a = a - a.mean()
    b = b - b.mean()
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))


def timed(fn):
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = fn()
    torch.cuda.synchronize()
    return out, time.perf_counter() - t0


def timed_warm(fn):
    """(result, warm seconds, cold seconds): the second of two identical
    calls, and the first (graph captures, lazy kernel loading, plans)."""
    _, cold = timed(fn)
    out, warm = timed(fn)
    return out, warm, cold


def inner_step_ms(op32, b: torch.Tensor, M, steps: int = 100) -> float:
    """Device time of one graph-replayed inner iteration of the mixed solver
    (FP32 operator, FP64 vectors) with preconditioner M."""
    st = DevicePCG(MixedOp(op32, b.numel(), b.device), b, torch.zeros_like(b), M, graph=True)
    st.start()
    for _ in range(5):
        st.step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        st.step()
    e1.record()
    e1.synchronize()
    return e0.elapsed_time(e1) / steps


def run(config: str = "c1", tol: float = 1e-6, learned: bool = True, pairs: int = 5000,
        epochs: int = 30, inner_iters: int = 20, seed_skies: int = 1000, log=print) -> dict:
    dev = torch.device("cuda", torch.cuda.current_device())
    cfg = CONFIGS[config]
    t0 = time.perf_counter()
    tv, m = make_todvec(cfg, dev)
    mapset = Mapset()
    mapset.add_map(m)
    rhs = mapset.copy()
    tv.make_rhs(rhs)
    hits = make_hits(tv, m)
    pre = jacobi_precon(hits)
    x0 = rhs.copy()
    x0.clear()
    op64 = tv.engine(m, torch.float64)
    op32 = tv.engine(m, torch.float32)
    setup_s = time.perf_counter() - t0
    hit = hits.map.reshape(-1) > 0
    out = {"config": config, "samples": tv.get_nsamp(), "npix": m.npix, "tol": tol,
           "hit_fraction": float(hit.double().mean()), "setup_s": setup_s,
           "tod2map_kernel": op64.method, "rot_mode_f64": op64.rot_mode, "rot_mode_f32": op32.rot_mode}
    xt, t_truth = timed(lambda: run_pcg(rhs, x0, tv, pre, maxiter=5000, tol=1e-10, verbose=False))
    truth = xt.maps[0].map.clone()
    out["truth"] = {"iters": xt.niter, "wall_s": t_truth}

    hist = []
    xj, tj, tjc = timed_warm(lambda: run_pcg(rhs, x0, tv, pre, maxiter=5000, tol=tol, verbose=False,
                                             history=None))
    out["jacobi_f64"] = {"iters": xj.niter, "wall_s": tj, "cold_wall_s": tjc,
                         "map_err": map_error(xj.maps[0].map, truth, hit)}

    steps = []
    cb = lambda k, xf, rel: steps.append({"outer": k, "true_rel_residual": rel,
                                          "map_err": map_error(xf, truth, hit)})
    xm, tm, tmc = timed_warm(lambda: run_pcg_mixed(rhs, x0, tv, pre, tol=tol))
    out["mixed_jacobi"] = {"iters": xm.niter, "fp64_residuals": xm.outer, "wall_s": tm, "cold_wall_s": tmc,
                           "inner_step_ms": inner_step_ms(op32, rhs.maps[0].map.reshape(-1),
                                                          pre.maps[0].map),
                           "true_rel_residual": xm.rel_residual,
                           "map_err": map_error(xm.maps[0].map, truth, hit)}
    run_pcg_mixed(rhs, x0, tv, pre, tol=tol, on_outer=cb)
    out["mixed_jacobi"]["per_refinement_step"] = steps
    steps_r = []
    cbr = lambda k, xf, rel: steps_r.append({"outer": k, "true_rel_residual": rel,
                                            "map_err": map_error(xf, truth, hit)})
    xr, trf = timed(lambda: run_pcg_mixed(rhs, x0, tv, pre, tol=tol, mode="refine",
                                          inner_iters=inner_iters, max_outer=60, on_outer=cbr))
    out["refine20"] = {"inner_iters": xr.niter, "outer": xr.outer, "wall_s": trf,
                       "true_rel_residual": xr.rel_residual, "per_refinement_step": steps_r[::5]}

    if learned:
        t1 = time.perf_counter()
        shape = (m.nx, m.ny)
        R, E, its = [], [], []
        seed = seed_skies
        # half the pairs from converged solves on seeded skies, half white
        n_solve = pairs // 2
        while sum(r.shape[0] for r in R) < n_solve:
            r, e, it = L.solve_pairs(op64, m, hits.map.reshape(-1), [seed], cfg.pixsize_arcsec)
            R.append(r)
            E.append(e)
            its += it
            seed += 1
        R = [torch.cat(R)[:n_solve]]
        E = [torch.cat(E)[:n_solve]]
        rw, ew = L.white_pairs(op32, hits.map, pairs - n_solve)
        R = torch.cat(R + [rw])
        E = torch.cat(E + [ew])
        del rw, ew
        t_pairs = time.perf_counter() - t1
        net = L.ConvNet.init(seed=0, device=dev)
        t2 = time.perf_counter()
        hist_loss = L.train(net, hits.map, shape, R, E, epochs=epochs)
        torch.cuda.synchronize()
        t_train = time.perf_counter() - t2
        del R, E
        Mlearn = L.LearnedPrecon(hits.map, net, shape)
        xl, tl, tlc = timed_warm(lambda: run_pcg_mixed(rhs, x0, tv, pre, tol=tol, inner_precon=Mlearn))
        xlf, tlf, tlfc = timed_warm(lambda: run_pcg(rhs, x0, tv, Mlearn, maxiter=5000, tol=tol,
                                                    verbose=False))
        # held-out skies: iterations to tol, learned vs Jacobi (FP64 PCG)
        held = []
        for s in range(5):
            b = L.sky_rhs(op64, m, 50_000 + s, cfg.pixsize_arcsec)
            kj, _ = L.iterations_to(op64, b, pre.maps[0].map, tol)
            kl, _ = L.iterations_to(op64, b, Mlearn, tol)
            held.append({"jacobi_iters": kj, "learned_iters": kl})
        out["learned"] = {"pairs": int(pairs), "solves": len(its), "pair_gen_s": t_pairs,
                          "train_s": t_train, "loss_first": hist_loss[0], "loss_last": hist_loss[-1],
                          "epochs": epochs, "held_out": held}
        out["mixed_learned"] = {"iters": xl.niter, "fp64_residuals": xl.outer, "wall_s": tl,
                                "cold_wall_s": tlc,
                                "inner_step_ms": inner_step_ms(op32, rhs.maps[0].map.reshape(-1), Mlearn),
                                "true_rel_residual": xl.rel_residual,
                                "map_err": map_error(xl.maps[0].map, truth, hit)}
        out["learned_f64"] = {"iters": xlf.niter, "wall_s": tlf, "cold_wall_s": tlfc,
                              "map_err": map_error(xlf.maps[0].map, truth, hit)}
        L.save(net, f"/tmp/mk_learned_{config}.npz")
    out["speedup_mixed_vs_jacobi_f64"] = tj / tm
    if learned:
        out["speedup_mixed_learned_vs_jacobi_f64"] = tj / out["mixed_learned"]["wall_s"]
    return out


def hit_density(hits: torch.Tensor) -> float:
    """Hit pixels / pixels inside the convex hull of the hit pixels."""
    from scipy.spatial import ConvexHull, Delaunay

    h = hits.detach().cpu().numpy()
    pts = np.argwhere(h > 0)
    if len(pts) < 3:
        return 1.0
    hull = pts[ConvexHull(pts).vertices]
    x0, y0 = pts.min(0)
    x1, y1 = pts.max(0)
    gx, gy = np.meshgrid(np.arange(x0, x1 + 1), np.arange(y0, y1 + 1), indexing="ij")
    inside = Delaunay(hull).find_simplex(np.stack([gx.ravel(), gy.ravel()], 1)) >= 0
    return float(len(pts) / max(int(inside.sum()), 1))


def _compact(hist: list) -> list:
    """(iteration, recursive residual, true FP64 residual, restarted) per replacement."""
    return [[h["iter"], h["recursive_rel"], h["true_rel_residual"], h.get("restart", False)] for h in hist]


def run_large(config: str = "c4", tol: float = 1e-6, max_iter: int = 3000, wall_limit_s: float = 900.0,
              learned: bool = False, pair_skies=(1000, 1001), pair_iters: int = 240, n_white: int = 64,
              epochs: int = 12, batch: int = 4, log=print) -> dict:
    """The batching configuration: TODs generated one at a time (each TOD's
    RHS contribution is accumulated and its timestream dropped), one pooled
    operator per precision over all TODs, per-iteration times of FP64 Jacobi
    PCG and of the mixed-precision PCG, and a mixed-precision solve to ``tol``
    (bounded by ``wall_limit_s``)."""
    from . import kernels as K
    from .maps import SkyMap
    from .noise import NoiseSmoothedSVD, clear_plan_cache
    from .pcg import DevicePCG, MixedOp
    from .synth import make_tod_info, tod_shapes
    from .tods import Tod, TodVec

    dev = torch.device("cuda", torch.cuda.current_device())
    cfg = CONFIGS[config]
    t0 = time.perf_counter()
    m = SkyMap(nx=cfg.nx, ny=cfg.ny, device=dev)
    rhs = torch.zeros(m.npix, dtype=torch.float64, device=dev)
    tv = TodVec()
    for k, (ndet, n) in enumerate(tod_shapes(cfg)):
        info = make_tod_info(cfg, k, ndet, n, dev, with_radec=False)
        tod = Tod(info)
        tod.set_noise(NoiseSmoothedSVD)
        dd = tod.noise.apply_noise(info["dat_calib"])
        K.tod2map(rhs, dd, info["ipix"])
        del dd
        tod.info["dat_calib"] = torch.empty((ndet, n), dtype=torch.float64, device="meta")
        tv.add_tod(tod)
        del tod, info
        if (k + 1) % 25 == 0:
            log(f"  {k + 1}/{cfg.ntod} TODs, {torch.cuda.memory_allocated() / 1e9:.1f} GB allocated")
    clear_plan_cache()
    torch.cuda.empty_cache()
    hits = make_hits(tv, m).map.reshape(-1)
    pre = torch.where(hits > 0, 1.0 / hits.clamp(min=1), torch.zeros_like(hits))
    op64 = tv.engine(m, torch.float64)
    op32 = tv.engine(m, torch.float32)
    torch.cuda.synchronize()
    out = {"config": config, "ntod": tv.ntod, "samples": tv.get_nsamp(), "npix": m.npix,
           "setup_s": time.perf_counter() - t0, "hit_density_in_footprint": hit_density(hits.view(m.nx, m.ny)),
           "tod2map_kernel_f64": op64.method, "tod2map_kernel_f32": op32.method,
           "rot_mode_f64": op64.rot_mode, "rot_mode_f32": op32.rot_mode,
           "gpu_mem_GB": torch.cuda.max_memory_allocated() / 1e9}

    def per_iter(op, b, M, n_it):
        x = torch.zeros_like(b)
        st = DevicePCG(op, b, x, M, graph=True)
        st.start()
        st.step()
        st.step()  # eager, then the captured graph
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(n_it):
            st.step()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n_it

    S = out["samples"]
    ms64 = per_iter(op64, rhs, pre, 2)
    out["jacobi_f64_iter"] = {"ms": ms64, "Msamp_per_s": S / ms64 / 1e3}
    msmx = per_iter(MixedOp(op32, m.npix, dev), rhs, pre, 5)
    out["mixed_iter"] = {"ms": msmx, "Msamp_per_s": S / msmx / 1e3}
    # mixed-precision solve to tol, bounded in wall time
    mp = m.copy()
    mp.map.copy_(rhs.view(m.nx, m.ny))
    b = Mapset()
    b.add_map(mp)
    x0 = b.copy()
    x0.clear()
    pre_ms = b.copy()
    pre_ms.maps[0].map.copy_(pre.view(m.nx, m.ny))
    hist = []
    t1 = time.perf_counter()
    budget = max(50, min(max_iter, int(wall_limit_s * 1e3 / max(msmx * 1.3, 1e-3))))
    xs, tm = timed(lambda: run_pcg_mixed(b, x0, tv, pre_ms, tol=tol, max_iter=budget, history=hist))
    out["mixed_solve"] = {"iters": xs.niter, "fp64_residuals": xs.outer, "restarts": xs.restarts,
                          "wall_s": tm, "true_rel_residual": xs.rel_residual, "reached_tol": xs.rel_residual <= tol,
                          "iteration_budget": budget, "replacements": _compact(hist)}
    out["jacobi_f64_projected_s"] = xs.niter * ms64 / 1e3
    out["projected_speedup_mixed_vs_jacobi_f64"] = out["jacobi_f64_projected_s"] / tm
    if learned:
        # training pairs: PCG iterates on b = A s for seeded skies s (known
        # solution), through the FP32 operator, plus white (A v, v) pairs
        del xs
        torch.cuda.empty_cache()
        t2 = time.perf_counter()
        mop = MixedOp(op32, m.npix, dev)
        R, E = L.known_solution_pairs(mop, m, hits, list(pair_skies), cfg.pixsize_arcsec,
                                      n_iter=pair_iters, every=3)
        rw, ew = L.white_pairs(op32, hits, n_white)
        R, E = torch.cat([R, rw]), torch.cat([E, ew])
        del rw, ew
        torch.cuda.synchronize()
        t_pairs = time.perf_counter() - t2
        net = L.ConvNet.init(seed=0, device=dev)
        t3 = time.perf_counter()
        hist_loss = L.train(net, hits, (m.nx, m.ny), R, E, epochs=epochs, batch=batch)
        torch.cuda.synchronize()
        t_train = time.perf_counter() - t3
        npairs = int(R.shape[0])
        del R, E
        torch.cuda.empty_cache()
        mlearn = L.LearnedPrecon(hits, net, (m.nx, m.ny))
        hist_l = []
        xl, tl = timed(lambda: run_pcg_mixed(b, x0, tv, pre_ms, tol=tol, max_iter=budget, history=hist_l,
                                             inner_precon=mlearn))
        out["learned"] = {"pairs": npairs, "pair_gen_s": t_pairs, "train_s": t_train, "epochs": epochs,
                          "loss_first": hist_loss[0], "loss_last": hist_loss[-1],
                          "weight_rms": [float(w.pow(2).mean().sqrt()) for w in net.weights]}
        out["mixed_learned_solve"] = {"iters": xl.niter, "fp64_residuals": xl.outer, "restarts": xl.restarts,
                                      "wall_s": tl, "true_rel_residual": xl.rel_residual,
                                      "reached_tol": xl.rel_residual <= tol, "replacements": _compact(hist_l)}
        out["projected_speedup_mixed_learned_vs_jacobi_f64"] = out["jacobi_f64_projected_s"] / tl
        L.save(net, f"/tmp/mk_learned_{config}.npz")
    return out


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="c1")
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--pairs", type=int, default=5000)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--inner", type=int, default=20)
    ap.add_argument("--large", action="store_true", help="the pooled large-configuration run")
    ap.add_argument("--wall", type=float, default=900.0)
    ap.add_argument("--large-epochs", type=int, default=12)
    a = ap.parse_args()
    if a.large:
        res = run_large(a.config, a.tol, wall_limit_s=a.wall, learned=not a.no_learned,
                        epochs=a.large_epochs)
    else:
        res = run(a.config, a.tol, not a.no_learned, a.pairs, a.epochs, a.inner)
    print(json.dumps(res))
