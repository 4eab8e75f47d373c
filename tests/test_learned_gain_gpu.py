"""What the trained network gains: the learned preconditioner is trained here,
on the GPU with the project's own forward, adjoint and weight-gradient
kernels, on the 1-TOD configuration (64 detectors x 65,341 samples, 256 x 256
map), and then compared with the Jacobi preconditioner of the reference's
scripts (precon = 1/hits, examples/minkasi_mpi_example.py:99-105) on skies it
has not seen: iterations and wall time of the mixed-precision PCG from
x0 = 0 to an FP64 true residual of 1e-6.

Training set: PCG iterates on b = A s for 4 seeded skies s with a known
solution (every 3rd of 300 iterates gives a pair (r_k, s - x_k)) plus 400
white pairs (A v, v); Adam, 10 epochs.  The held-out skies use other seeds.
GPU only."""
import time

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
cuda = torch.device("cuda", 0)


def _solve_time(mk, b, x0, tv, pre, **kw):
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    x = mk.run_pcg_mixed(b, x0, tv, pre, tol=1e-6, **kw)
    torch.cuda.synchronize()
    return x, time.perf_counter() - t0


def test_trained_preconditioner_beats_jacobi_on_held_out_skies():
    import minkasi_gb300 as mk
    from minkasi_gb300 import learned as L
    from minkasi_gb300 import synth
    from minkasi_gb300.pcg import MixedOp

    cfg = synth.CONFIGS["c1"]
    tv, m = synth.make_todvec(cfg, cuda)
    hits = mk.make_hits(tv, m)
    h = hits.map.reshape(-1)
    pre = mk.jacobi_precon(hits)
    op64 = tv.engine(m, torch.float64)
    op32 = tv.engine(m, torch.float32)
    t0 = time.perf_counter()
    R, E = L.known_solution_pairs(MixedOp(op32, m.npix, cuda), m, h, [1000, 1001, 1002, 1003],
                                  cfg.pixsize_arcsec, n_iter=300, every=3)
    rw, ew = L.white_pairs(op32, h, 400)
    R, E = torch.cat([R, rw]), torch.cat([E, ew])
    net = L.ConvNet.init(seed=0, device=cuda)
    hist = L.train(net, h, (m.nx, m.ny), R, E, epochs=10, batch=32)
    t_train = time.perf_counter() - t0
    assert hist[-1] < hist[0]
    ml = L.LearnedPrecon(h, net, (m.nx, m.ny))

    its_j, its_l, t_j, t_l = [], [], [], []
    for seed in (50_000, 50_001, 50_002):
        s = L.sky(m.nx, m.ny, cfg.pixsize_arcsec, seed, cuda).reshape(-1)
        s = torch.where(h > 0, s, torch.zeros_like(s))
        bm = mk.Mapset()
        bm.add_map(m.copy())
        op64.apply(s, bm.maps[0].map.reshape(-1))
        x0 = bm.copy()
        x0.clear()
        # warm both (graph capture, lazy loading), then time
        _solve_time(mk, bm, x0, tv, pre)
        _solve_time(mk, bm, x0, tv, pre, inner_precon=ml)
        xj, tj = _solve_time(mk, bm, x0, tv, pre)
        xl, tl = _solve_time(mk, bm, x0, tv, pre, inner_precon=ml)
        assert xj.rel_residual <= 1e-6 and xl.rel_residual <= 1e-6
        its_j.append(xj.niter)
        its_l.append(xl.niter)
        t_j.append(tj)
        t_l.append(tl)
    print(f"trained in {t_train:.1f} s on {R.shape[0]} pairs (loss {hist[0]:.3f} -> {hist[-1]:.3f}); "
          f"held-out iterations Jacobi {its_j} vs learned {its_l}; wall s Jacobi "
          f"{[round(t, 4) for t in t_j]} vs learned {[round(t, 4) for t in t_l]}")
    assert sum(its_l) < 0.9 * sum(its_j)
    assert sum(t_l) < sum(t_j)
