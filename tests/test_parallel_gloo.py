"""Multi-rank host logic on CPU: two gloo ranks sum a map, reduce scalars,
and split TODs.  A failing rank is detected by the other through a short
process-group timeout (the failure is made on the host)."""
import os
import socket

import pytest
import torch
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q, fail_rank=-1):
    import datetime
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world,
                                         timeout=datetime.timedelta(seconds=20))
    from minkasi_gb300 import parallel
    try:
        assert parallel.have_mpi() and parallel.world() == world
        m = torch.full((4, 5), float(rank + 1), dtype=torch.float64)
        parallel.allreduce_(m)
        lo = parallel.allreduce_scalar(-float(rank), "min")
        tot = parallel.allreduce_scalar(10.0 * (rank + 1), "sum")
        parts = parallel.partition([5.0, 1.0, 3.0, 4.0, 2.0], world)
        if rank == fail_rank:
            raise RuntimeError("injected failure before the second reduction")
        m2 = torch.ones(3)
        parallel.allreduce_(m2)
        q.put((rank, float(m.sum()), lo, tot, parts, float(m2.sum())))
    except RuntimeError as e:
        q.put((rank, "error", str(e)))
    finally:
        if rank == fail_rank:
            os._exit(0)  # leave without joining the collective
        try:
            torch.distributed.destroy_process_group()
        except Exception:
            pass


def _hb_worker(rank, world, port, q, fail_rank):
    import datetime
    from minkasi_gb300 import parallel
    store = torch.distributed.TCPStore("127.0.0.1", port, world, rank == 0,
                                       timeout=datetime.timedelta(seconds=30))
    done = []
    try:
        for step in range(3):
            if rank == fail_rank and step == 1:
                q.put((rank, "left", done))
                q.close()
                q.join_thread()  # flush the message before the abrupt exit
                os._exit(0)  # the failure, made on the host between steps
            parallel.step_heartbeat(store, step, rank, world, timeout_s=3.0)
            done.append(step)
        q.put((rank, "ok", done))
    except parallel.PeerFailure as e:
        q.put((rank, "peer-failure", done))
    # keep the store server (rank 0) alive until the other rank has read it
    import time
    time.sleep(1.0)


class _DenseShare:
    """A rank's share of an operator, mocked on the CPU: A_r = B_r^T B_r over
    the rows of B this rank owns (the TODs of a rank, in miniature)."""

    def __init__(self, B):
        self.B = B

    def apply(self, x, out, accumulate=False):
        y = self.B.T @ (self.B @ x)
        if accumulate:
            out += y
        else:
            out.copy_(y)
        return out


def _ranksum_worker(rank, world, port, q, fail_rank):
    import datetime
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world,
                                         timeout=datetime.timedelta(seconds=20))
    from minkasi_gb300 import parallel
    from minkasi_gb300.pcg import RankSumOp, global_op
    try:
        g = torch.Generator().manual_seed(0)
        B = torch.randn(40, 12, generator=g, dtype=torch.float64)
        costs = [float(1 + (i % 7)) for i in range(B.shape[0])]
        mine = parallel.partition(costs, world)[rank]
        op = global_op(_DenseShare(B[mine]))
        assert isinstance(op, RankSumOp)
        x = torch.randn(12, generator=g, dtype=torch.float64)
        full = B.T @ (B @ x)
        y = op.apply(x, torch.empty(12, dtype=torch.float64))
        acc = torch.ones(12, dtype=torch.float64)
        op.apply(x, acc, accumulate=True)
        # a few CG steps on the summed operator: every rank must hold the
        # same iterates, equal to the one-rank solve
        A = B.T @ B + torch.eye(12, dtype=torch.float64)
        class Shifted:
            def apply(self_, v, out, accumulate=False):
                op.apply(v, out)
                out += v  # the identity, added after the sum (same on every rank)
                return out
        b = torch.randn(12, generator=g, dtype=torch.float64)
        xs, r = torch.zeros(12, dtype=torch.float64), b.clone()
        p, Ap = r.clone(), torch.empty(12, dtype=torch.float64)
        rr = float(r @ r)
        for _ in range(12):
            Shifted().apply(p, Ap)
            a = rr / float(p @ Ap)
            xs += a * p
            r -= a * Ap
            rr_new = float(r @ r)
            p = r + (rr_new / rr) * p
            rr = rr_new
        q.put((rank, float((y - full).abs().max() / full.abs().max()),
               float((acc - 1 - full).abs().max() / full.abs().max()),
               float((A @ xs - b).norm() / b.norm()), sorted(mine), xs.tolist()))
    finally:
        torch.distributed.destroy_process_group()


def _run(world, fail_rank=-1, target=None):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=target or _worker, args=(r, world, port, q, fail_rank))
             for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=90) for _ in range(world)]
    for p in procs:
        p.join(timeout=30)
        if p.is_alive():
            p.kill()
    return sorted(out, key=lambda t: t[0])


def test_two_rank_map_reduction_and_partition():
    out = _run(2)
    for rank, msum, lo, tot, parts, m2 in out:
        assert msum == 20 * 3.0        # (1 + 2) per pixel, 20 pixels
        assert lo == -1.0 and tot == 30.0
        assert sorted(sum(parts, [])) == [0, 1, 2, 3, 4]
        assert m2 == 6.0


def test_failed_rank_is_detected_by_heartbeat():
    out = _run(2, fail_rank=1, target=_hb_worker)
    assert out[1][1] == "left"
    assert out[0][1] == "peer-failure" and out[0][2] == [0]
    ok = _run(2, target=_hb_worker)
    assert all(o[1] == "ok" and o[2] == [0, 1, 2] for o in ok)


def test_rank_sum_operator_sums_the_shares():
    """Each rank applies the operator of the items it owns (a greedy
    partition), and RankSumOp sums the map over ranks after every
    application: both ranks see the full operator, and a CG run on it gives
    the same iterates on every rank, converged on the full system."""
    out = _run(2, target=_ranksum_worker)
    (_, e0, a0, res0, own0, x0), (_, e1, a1, res1, own1, x1) = out
    assert max(e0, e1, a0, a1) < 1e-13
    assert sorted(own0 + own1) == list(range(40)) and not set(own0) & set(own1)
    assert x0 == x1
    assert res0 < 1e-8
