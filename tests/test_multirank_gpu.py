"""run_pcg and run_pcg_mixed over two ranks, each holding half of the TODs of
the tiny configuration, against the one-rank solve.

The ranks are two processes on cuda:0 joined by gloo.  Every operator
application inside the solvers is followed by the sum of the map over ranks
(RankSumOp), which gloo stages through host memory: the ranks wait for each
other only on the host, and no kernel of one process waits on the other's.
GPU only.
"""
import datetime
import os
import socket
import traceback

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

pytestmark = pytest.mark.gpu


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _solve(mk, tv, m):
    mapset = mk.Mapset()
    mapset.add_map(m)
    rhs = mapset.copy()
    tv.make_rhs(rhs)
    hits = mk.make_hits(tv, m)
    pre = mk.jacobi_precon(hits)
    x0 = rhs.copy()
    x0.clear()
    x12 = mk.run_pcg(rhs, x0, tv, pre, maxiter=12, graph=False, verbose=False)
    xm = mk.run_pcg_mixed(rhs, x0, tv, pre, tol=1e-6)
    return {"rhs": rhs.maps[0].to_numpy(), "hits": hits.to_numpy(), "x12": x12.maps[0].to_numpy(),
            "xm": xm.maps[0].to_numpy(), "xm_rel": xm.rel_residual, "xm_iters": xm.niter}


def _tiny(mk):
    from minkasi_gb300 import synth
    return synth.make_todvec(synth.CONFIGS["tiny"], torch.device("cuda", 0))


def _worker(rank, world, port, q):
    try:
        os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        torch.distributed.init_process_group("gloo", rank=rank, world_size=world,
                                             timeout=datetime.timedelta(seconds=120))
        torch.cuda.set_device(0)
        import minkasi_gb300 as mk
        from minkasi_gb300 import parallel
        full, m = _tiny(mk)
        mine = parallel.partition([float(t.get_nsamp()) for t in full.tods], world)[rank]
        tv = mk.TodVec()
        for i in mine:
            tv.add_tod(full.tods[i])
        tv.tod2map_method = "fixed"
        res = _solve(mk, tv, m)
        res["mine"] = mine
        q.put((rank, res))
        torch.distributed.destroy_process_group()
    except Exception:
        q.put((rank, traceback.format_exc()))


def test_two_ranks_solve_like_one():
    import minkasi_gb300 as mk
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=600) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        if p.is_alive():
            p.kill()
    for r in (0, 1):
        assert isinstance(out[r], dict), out[r]
    assert sorted(out[0]["mine"] + out[1]["mine"]) == [0, 1] and out[0]["mine"] and out[1]["mine"]

    full, m = _tiny(mk)
    full.tod2map_method = "fixed"
    one = _solve(mk, full, m)

    def rel(a, b):
        return float(np.abs(a - b).max() / np.abs(b).max())

    for r in (0, 1):
        got = out[r]
        assert np.array_equal(got["hits"], one["hits"])
        assert rel(got["rhs"], one["rhs"]) < 1e-12
        # FP64 PCG: only the order of the map sums differs from one rank
        assert rel(got["x12"], one["x12"]) < 1e-10
        assert got["xm_rel"] <= 1e-6
    # the ranks hold the same (replicated) solution
    assert np.array_equal(out[0]["x12"], out[1]["x12"])
    assert np.array_equal(out[0]["xm"], out[1]["xm"])
    # and it solves the full system: FP64 true residual with the one-rank operator
    mapset = mk.Mapset()
    mapset.add_map(m)
    rhs = mapset.copy()
    full.make_rhs(rhs)
    x = mapset.copy()
    x.maps[0].assign(out[0]["xm"])
    ax = full.dot(x).maps[0].to_numpy()
    b = rhs.maps[0].to_numpy()
    assert np.linalg.norm(b - ax) / np.linalg.norm(b) <= 1.05e-6
