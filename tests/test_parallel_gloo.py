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
