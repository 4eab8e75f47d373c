"""Project autotuner: picks the tod2map kernel and the rotation GEMM per
workload by timing the candidates on the actual device buffers, and caches
the choice in a JSON file keyed on (GPU, dtype, detector counts, samples,
map size, hit density).

Cache file: $MINKASI_GB300_AUTOTUNE, else ~/.cache/minkasi_gb300/autotune.json.
It also picks, per TOD shape, the DCT-I transform and the four-step split
L1 x L2 (the tile shape of the FFT passes).
Set MINKASI_GB300_TOD2MAP=atomic|staged|fixed|sorted (or ..._ROT=1|2|3, or
..._DCT=0|1|2, the kernels.set_dct_engine values) to force a choice.
"""
from __future__ import annotations

import json
import os
from typing import Dict, Iterable, Optional, Sequence, Tuple

import numpy as np
import torch

from . import kernels as K

_MEM: Dict[str, object] = {}


def cache_path() -> str:
    p = os.environ.get("MINKASI_GB300_AUTOTUNE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "minkasi_gb300", "autotune.json")


def _load() -> dict:
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(key: str, value) -> None:
    _MEM[key] = value
    d = _load()
    d[key] = value
    try:
        os.makedirs(os.path.dirname(cache_path()), exist_ok=True)
        tmp = cache_path() + ".tmp"
        with open(tmp, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
        os.replace(tmp, cache_path())
    except OSError:
        pass


def _lookup(key: str):
    if key in _MEM:
        return _MEM[key]
    return _load().get(key)


def workload_key(op, what: str) -> str:
    ndets = sorted(set(d[0] for d in op.dims))
    hits = op.hits()
    density = float((hits > 0).double().mean().item())
    gpu = torch.cuda.get_device_name(op.device)
    return (f"{what}|{gpu}|{str(op.dtype).split('.')[-1]}|ndet={ndets}|S={op.S}|npix={op.npix}"
            f"|density={density:.3f}")


def time_ms(fn, reps: int = 3, warm: int = 1) -> float:
    for _ in range(warm):
        fn()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = float("inf")
    for _ in range(reps):
        torch.cuda.synchronize()
        e0.record()
        fn()
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best


def choose_tod2map(op, candidates: Optional[Iterable[str]] = None) -> str:
    forced = os.environ.get("MINKASI_GB300_TOD2MAP")
    if forced:
        return forced
    if candidates is None:
        candidates = ["atomic", "staged", "fixed"]
        if op.S < (1 << 30) and max(op.sizes) < (1 << 31):
            candidates.append("sorted")  # plan memory 4 B/sample
    key = workload_key(op, "tod2map")
    hit = _lookup(key)
    if hit in candidates:
        return hit
    op.tmp.normal_()
    out = torch.zeros(op.npix, dtype=op.dtype, device=op.device)
    times = {m: time_ms(lambda m=m: op.project_out(out, m)) for m in candidates}
    best = min(times, key=times.get)
    if best != "sorted":
        op._pixplans = None
    _store(key, best)
    return best


def choose_rot_mode(op) -> int:
    """Fastest rotation GEMM that agrees with the FP64/FP32 cuBLAS result
    (rel. 1e-13 in FP64, 1e-5 in FP32) on the largest TOD shape: cuBLAS on
    the FP64/FP32 units (1), cuBLAS emulation (3), and this library's
    tensor-core kernels (2: FP32 3xTF32; 4: FP64 exact integer slices)."""
    forced = os.environ.get("MINKASI_GB300_ROT")
    if forced:
        return int(forced)
    key = workload_key(op, "rot")
    hit = _lookup(key)
    if hit is not None:
        return int(hit)
    i = int(np.argmax(op.sizes))
    nd, n = op.dims[i]
    v, vT, w = op.ops[i]
    plan = op.plans[(nd, n)]
    x = torch.randn((nd, n), dtype=op.dtype, device=op.device)
    ref = plan.apply(v, vT, w, x, rot_mode=1)
    tol = 1e-13 if op.dtype == torch.float64 else 1e-5
    tc_ok = op.dtype == torch.float32 and os.environ.get("MINKASI_GB300_TC", "1") != "0" and \
        nd in (32, 64, 128, 256)
    modes = [1, 3] + ([2] if tc_ok else []) + ([4] if op.dtype == torch.float64 else [])
    times = {}
    for m in modes:
        try:
            y = plan.apply(v, vT, w, x, rot_mode=m)
        except K._lib.MkError:
            continue
        err = float((y - ref).abs().max() / ref.abs().max())
        if err > tol:
            continue
        times[m] = time_ms(lambda m=m: plan.apply(v, vT, w, x, rot_mode=m))
    best = min(times, key=times.get)
    _store(key, best)
    return best


def with_dct_engine(engine, fn):
    """fn() with kernels.set_dct_engine in force (plans created in fn keep
    it), then the previous setting restored.  ``engine`` is an engine number
    or an (engine, split rank) pair: the rank also selects the four-step
    split L1 x L2 (kernels.set_fft4_split)."""
    e, rank = (engine, 0) if isinstance(engine, int) else (int(engine[0]), int(engine[1]))
    prev, prev_rank = K.dct_engine(), K.fft4_split()
    K.set_dct_engine(e)
    K.set_fft4_split(rank)
    try:
        return fn()
    finally:
        K.set_dct_engine(prev)
        K.set_fft4_split(prev_rank)


SPLIT_RANKS = 3  # four-step splits tried per TOD shape (closest to sqrt(L) first)


def choose_dct_engines(op, shapes: Sequence[Tuple[int, int]]) -> Dict[Tuple[int, int], Tuple[int, int]]:
    """Per TOD shape of an FP32 operator, the fastest noise filter among the
    four-step FFT (engine 0, Bluestein included) with each of its
    SPLIT_RANKS closest L1 x L2 splits (the tile shapes of its two passes)
    and cuFFT (engine 1), timed on the shape's first TOD with the rotation
    the shape will use.  Returns {shape: (engine, split rank)}; FP64
    operators keep the current engine (by default the four-step FFT in
    double precision)."""
    cur = K.dct_engine()
    if op.dtype != torch.float32:
        return {s: (cur, 0) for s in shapes}
    forced = os.environ.get("MINKASI_GB300_DCT")
    if forced:
        return {s: (int(forced), 0) for s in shapes}
    gpu = torch.cuda.get_device_name(op.device)
    out, todo = {}, []
    for s in shapes:
        hit = _lookup(f"dct2|{gpu}|{s[0]}x{s[1]}")
        if isinstance(hit, list) and len(hit) == 2:
            out[s] = (int(hit[0]), int(hit[1]))
        else:
            todo.append(s)
    if not todo:
        return out
    need = max(with_dct_engine(e, lambda s=s: K.noise_workspace_bytes(s[0], s[1], op.dtype))
               for s in todo for e in (0, 1))
    ws = torch.empty(need, dtype=torch.uint8, device=op.device)
    for s in todo:
        nd, n = s
        v, vT, w = op.ops[op.dims.index(s)]
        x = torch.randn((nd, n), dtype=op.dtype, device=op.device)
        y = torch.empty_like(x)
        mode = 2 if nd in (32, 64, 128, 256) else 1
        times, seen = {}, set()
        for cand in [(0, r) for r in range(SPLIT_RANKS)] + [(1, 0)]:
            plan = with_dct_engine(cand, lambda: K.NoisePlan(nd, n, op.dtype, op.device, workspace=ws))
            if cand[0] == 0 and (plan.engine == 1 or plan.split in seen):
                del plan
                continue  # no four-step transform, or the same split again
            seen.add(plan.split)
            times[cand] = time_ms(lambda: plan.apply(v, vT, w, x, out=y, rot_mode=mode))
            del plan
        best = min(times, key=times.get)
        out[s] = best
        _store(f"dct2|{gpu}|{nd}x{n}", list(best))
        del x, y
    del ws
    return out
