"""Solver experiments on the benchmark configurations (time to an FP64
residual, map error per refinement step, learned vs Jacobi).

    python -m minkasi_gb300.experiments --config c1 --tol 1e-6 [--learned] [--pairs 5000]

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
happen before), with torch.cuda.synchronize() on both sides.  Map errors are
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
from .pcg import run_pcg, run_pcg_mixed
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
    whits = make_hits(tv, m, do_weights=True)   # ~diag(A): the learned preconditioner's D
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
    xj, tj = timed(lambda: run_pcg(rhs, x0, tv, pre, maxiter=5000, tol=tol, verbose=False,
                                   history=None))
    out["jacobi_f64"] = {"iters": xj.niter, "wall_s": tj,
                         "map_err": map_error(xj.maps[0].map, truth, hit)}

    steps = []
    cb = lambda k, xf, rel: steps.append({"outer": k, "true_rel_residual": rel,
                                          "map_err": map_error(xf, truth, hit)})
    xm, tm = timed(lambda: run_pcg_mixed(rhs, x0, tv, pre, tol=tol))
    out["mixed_jacobi"] = {"iters": xm.niter, "fp64_residuals": xm.outer, "wall_s": tm,
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
        while sum(r.shape[0] for r in R) < pairs:
            r, e, it = L.solve_pairs(op64, m, hits.map.reshape(-1), [seed], cfg.pixsize_arcsec)
            R.append(r)
            E.append(e)
            its += it
            seed += 1
        R = torch.cat(R)[:pairs]
        E = torch.cat(E)[:pairs]
        t_pairs = time.perf_counter() - t1
        net = L.ConvNet.init(seed=0, device=dev)
        t2 = time.perf_counter()
        hist_loss = L.train(net, whits.map, shape, R, E, epochs=epochs)
        torch.cuda.synchronize()
        t_train = time.perf_counter() - t2
        del R, E
        Mlearn = L.LearnedPrecon(whits.map, net, shape)
        xl, tl = timed(lambda: run_pcg_mixed(rhs, x0, tv, pre, tol=tol, inner_precon=Mlearn))
        xlf, tlf = timed(lambda: run_pcg(rhs, x0, tv, Mlearn, maxiter=5000, tol=tol, verbose=False))
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
                                "true_rel_residual": xl.rel_residual,
                                "map_err": map_error(xl.maps[0].map, truth, hit)}
        out["learned_f64"] = {"iters": xlf.niter, "wall_s": tlf,
                              "map_err": map_error(xlf.maps[0].map, truth, hit)}
        L.save(net, f"/tmp/mk_learned_{config}.npz")
    out["speedup_mixed_vs_jacobi_f64"] = tj / tm
    if learned:
        out["speedup_mixed_learned_vs_jacobi_f64"] = tj / out["mixed_learned"]["wall_s"]
    return out


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="c1")
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--pairs", type=int, default=5000)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--inner", type=int, default=20)
    a = ap.parse_args()
    res = run(a.config, a.tol, not a.no_learned, a.pairs, a.epochs, a.inner)
    print(json.dumps(res))
