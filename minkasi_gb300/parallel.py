"""Multi-rank support, mirroring minkasi/parallel.py:1-79 on torch.distributed.

The reference shards TODs over MPI ranks (examples/minkasi_mpi_example.py:29)
and sums the map over ranks after every operator application
(minkasi/tods/core.py:1021-1022 -> minkasi/maps/skymap.py:742-783).  Here the
same single exchange is a sum all-reduce of the map through torch.distributed
(NCCL between GPUs, gloo on CPU); with one process everything is a no-op.
TOD sharding is a greedy longest-processing-time assignment on a per-TOD
cost (samples x log2 samples, the transform cost), which balances uneven
TODs better than the reference's round robin.
"""
from __future__ import annotations

import heapq
import math
from typing import List, Sequence

import torch


def have_dist() -> bool:
    return torch.distributed.is_available() and torch.distributed.is_initialized()


def rank() -> int:
    return torch.distributed.get_rank() if have_dist() else 0


def world() -> int:
    return torch.distributed.get_world_size() if have_dist() else 1


def have_mpi() -> bool:
    """True when more than one rank takes part (the reference's have_mpi)."""
    return world() > 1


def barrier() -> None:
    if have_mpi():
        torch.distributed.barrier()


def _backend_takes(t: torch.Tensor) -> bool:
    return not (t.is_cuda and torch.distributed.get_backend() == "gloo")


def allreduce_(t: torch.Tensor) -> torch.Tensor:
    """In-place sum over ranks (the map reduction of Mapset.mpi_reduce)."""
    if not have_mpi():
        return t
    if _backend_takes(t):
        torch.distributed.all_reduce(t)
    else:  # gloo with a CUDA tensor: stage through the host
        h = t.detach().cpu()
        torch.distributed.all_reduce(h)
        t.copy_(h)
    return t


def allreduce_scalar(x: float, op: str = "sum") -> float:
    """Scalar all-reduce for lims / nsamp (minkasi/tods/core.py:850-853,876)."""
    if not have_mpi():
        return x
    ops = {"sum": torch.distributed.ReduceOp.SUM, "min": torch.distributed.ReduceOp.MIN,
           "max": torch.distributed.ReduceOp.MAX}
    t = torch.tensor([float(x)], dtype=torch.float64)
    torch.distributed.all_reduce(t, op=ops[op])
    return float(t.item())


def tod_cost(ndet: int, ndata: int) -> float:
    return float(ndet) * ndata * math.log2(max(ndata, 2))


def partition(costs: Sequence[float], nproc: int) -> List[List[int]]:
    """Assign item indices to nproc ranks, largest first onto the least-loaded
    rank.  Deterministic: ties break on rank index, then item index."""
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    heap = [(0.0, r) for r in range(nproc)]
    out: List[List[int]] = [[] for _ in range(nproc)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + costs[i], r))
    return [sorted(o) for o in out]


class PeerFailure(RuntimeError):
    """A rank did not reach a step within the heartbeat timeout."""


def step_heartbeat(store, step: int, rank_: int, world_: int, timeout_s: float = 5.0,
                   poll_s: float = 0.02) -> None:
    """Host-side failure detection between steps: announce ``step`` in a
    key-value store (e.g. torch.distributed.TCPStore) and wait, at most
    ``timeout_s``, until every rank has announced it.  Raises PeerFailure
    naming the missing ranks, so survivors stop before their next launch
    instead of blocking in a collective with a dead peer."""
    import time

    store.set(f"mk/hb/{rank_}/{step}", "1")
    deadline = time.monotonic() + timeout_s
    missing = list(range(world_))
    while True:
        missing = [r for r in missing if not store.check([f"mk/hb/{r}/{step}"])]
        if not missing:
            return
        if time.monotonic() > deadline:
            raise PeerFailure(f"ranks {missing} did not reach step {step} within {timeout_s} s")
        time.sleep(poll_s)
