"""Converged maps against the FP64 oracle's solution, on the 1-TOD
configuration (64 detectors x 65,341 samples, 256 x 256 map at 2").

The oracle sets up the system: b = A s in FP64 on the CPU (minkasi's
TodVec.dot restated, minkasi/tods/core.py:967-1026) for a seeded synthetic
sky s on the hit pixels, so the exact solution of the oracle's system is s
itself, up to the constant on the hit region that A annihilates (the mean
over hit pixels is removed from both maps before comparing).  Each GPU solver
runs from x0 = 0 to an FP64 true residual of 1e-10, and its map must be
within the stated 1e-5 relative L2 of s:

* FP64 Jacobi PCG (the reference's method, run_pcg with a tolerance),
* mixed precision (FP32 operator, FP64 vectors and residual replacement),
* mixed precision with the learned preconditioner (committed weights).

The achieved residuals and map errors are printed.  GPU only."""
import os

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu
cuda = torch.device("cuda", 0)
TOL_MAP = 1e-5      # relative L2 on the converged map, hit-region mean removed
TOL_RES = 1e-10     # FP64 true residual each solve runs to


def _map_err(x, s, hit):
    a = x[hit] - x[hit].mean()
    b = s[hit] - s[hit].mean()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def system():
    import minkasi_gb300 as mk
    from minkasi_gb300 import learned as L
    from minkasi_gb300 import synth
    cfg = synth.CONFIGS["c1"]
    tv, m = synth.make_todvec(cfg, cuda)
    otods = []
    for t in tv.tods:
        v, vT, w = (a.cpu().numpy() for a in t.noise.operands(torch.float64))
        otods.append(oracle.OracleTod(ipix=t.info["ipix"].cpu().numpy(), v=v, vT=vT, mywt=w))
    hits = oracle.make_hits(otods, (m.nx, m.ny))
    hit = hits > 0
    s = np.where(hit, L.sky(m.nx, m.ny, cfg.pixsize_arcsec, 777, cuda).cpu().numpy(), 0.0)
    b = oracle.todvec_dot(otods, s, workers=os.cpu_count() or 1)
    mapset = mk.Mapset()
    mapset.add_map(m)
    rhs = mapset.copy()
    rhs.maps[0].assign(b)
    x0 = rhs.copy()
    x0.clear()
    ghits = mk.make_hits(tv, m)
    assert np.array_equal(ghits.to_numpy(), hits)
    pre = mk.jacobi_precon(ghits)
    return mk, L, tv, m, rhs, x0, pre, ghits, s, hit, otods, b


@pytest.mark.parametrize("solver", ["jacobi_f64", "mixed_jacobi", "mixed_learned"])
def test_converged_map_matches_the_oracle_solution(system, solver):
    mk, L, tv, m, rhs, x0, pre, ghits, s, hit, otods, b = system
    if solver == "jacobi_f64":
        x = mk.run_pcg(rhs, x0, tv, pre, maxiter=20000, tol=TOL_RES, verbose=False)
    elif solver == "mixed_jacobi":
        x = mk.run_pcg_mixed(rhs, x0, tv, pre, tol=TOL_RES, max_iter=20000)
    else:
        net = L.load(L.weights_path("c1"), cuda)
        ml = L.LearnedPrecon(ghits.map, net, (m.nx, m.ny))
        x = mk.run_pcg_mixed(rhs, x0, tv, pre, tol=TOL_RES, max_iter=20000, inner_precon=ml)
    xm = x.maps[0].to_numpy()
    # the residual as the oracle computes it, on the oracle's operator
    res = np.linalg.norm(b - oracle.todvec_dot(otods, xm, workers=os.cpu_count() or 1)) / np.linalg.norm(b)
    err = _map_err(xm, s, hit)
    print(f"{solver}: {x.niter} iterations, FP64 true residual {res:.3e} (oracle), "
          f"map error vs the oracle's solution {err:.3e}")
    assert res <= 1.05 * TOL_RES
    assert err <= TOL_MAP
