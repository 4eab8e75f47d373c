"""Benchmark: tod2map GB/s on the 32-TOD FP64 workload, plus the solver's
time to a 1e-6 FP64 residual (learned vs Jacobi PCG).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--no-pcg] [--no-solver] [--no-c4]

Workload (the reference's "plain method at GPU scale" configuration): 32
synthetic TODs, 256 detectors each, nsamp ~ U[2^17, 2^19] truncated to
FFT-friendly lengths, daisy-scan pointing onto a 1024x1024 map at 1",
FP64.  One step = one tod2map pass of every TOD's timestream into the map
(the projection of TodVec.make_rhs / TodVec.dot), inputs resident in HBM.
value = algorithmic bytes (4 B ipix + 8 B dat per sample) / step time.
The inputs (32 GB) exceed the 129 MB L2, so no flush is needed between steps.
With N ranks the TODs are split between them (largest first onto the least
loaded rank, minkasi's TOD sharding) and the map is summed over ranks every
step: the total work is fixed, so scaling is strong.

e2e: the same step through the public API (SkyMap.tod2map per TOD) with the
timestream in pinned host memory, copied to the device inside the timed
region (in chunks overlapped with the scatter), and the map read back to the
host every step; the pixel indices stay cached on the device as the API
caches them (tod.info[tag]).

Extra keys: map2tod GB/s on the same samples; per-iteration timings of the
full hot path (FP64 Jacobi PCG iteration = batched A-apply + update, and the
FP32 inner iteration of the mixed-precision solver) on the same TODs; and,
under "solver", the other half of the benchmark metric: wall time from x0 = 0
to an FP64 true residual ||b - A x||/||b|| <= 1e-6 for FP64 Jacobi PCG (the
plain method), the mixed-precision PCG with Jacobi, and the mixed-precision
PCG with the learned preconditioner (weights made by learned.train_recipe),
on the 1-TOD configuration (all three run to the end) and on the 200-TOD
configuration (the FP64 Jacobi solve, about two hours there, is its measured
iteration time times the mixed solve's iteration count, labelled projected).
The 200-TOD solves run first, in a child process with the whole GPU (they
peak near 240 GB of HBM).

CPU baselines run in a separate process with no GPU library loaded (this
script with --impl reference): the reference's tod2map, and its operator per
PCG iteration, on all host threads over a bounded sample of the workload.

--impl reference times the reference's CPU tod2map (its own C compiled from
source when available in oracle/_ref, else the C restatement in oracle/)
with all host threads on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

WORKLOAD = "c2: 32 TODs x 256 det x U[2^17,2^19] samples (truncated), 1024x1024 map at 1in, FP64"
METRIC = "tod2map GB/s"
BYTES_PER_SAMPLE = 12  # int32 pixel index + float64 sample
# measured DRAM bytes per sample (read + write) of each FP64 tod2map kernel:
# one ncu capture each (dram__bytes_read.sum + dram__bytes_write.sum) of a
# launch over the first c2 TOD shape, 256 x 130978 = 33,530,368 samples
NCU_DRAM_BYTES_PER_SAMPLE = {"atomic": (404.32e6 + 3.30e6) / 33530368,
                             "staged": (404.30e6 + 2.87e6) / 33530368}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c2")
    ap.add_argument("--no-pcg", action="store_true", help="skip the PCG-iteration extras")
    ap.add_argument("--no-solver", action="store_true", help="skip the time-to-residual solves")
    ap.add_argument("--no-c4", action="store_true", help="skip the 200-TOD solves")
    ap.add_argument("--cpu-pcg", action="store_true",
                    help="(reference arm) also time the reference CPU operator per PCG iteration")
    ap.add_argument("--method", default=None, help="force the tod2map kernel (atomic|staged|fixed|sorted)")
    ap.add_argument("--c4-only", action="store_true",
                    help="(internal) run only the 200-TOD solves and print their record")
    ap.add_argument("--sparse", action="store_true",
                    help="the 200-TOD workload with sparse hits instead: the autotuner's tod2map choice "
                         "and every scatter kernel's GB/s")
    return ap.parse_args()


def load_synth():
    """minkasi_gb300/synth.py and the truncate module it imports, loaded by
    file path under a stand-in package name, so that the CPU arm builds the
    same pointing without running the package __init__ (which loads the GPU
    library)."""
    import importlib.util
    import types

    name = "_mk_synth_only"
    if name + ".synth" in sys.modules:
        return sys.modules[name + ".synth"]
    pkg = types.ModuleType(name)
    pkg.__path__ = [os.path.join(REPO, "minkasi_gb300")]
    sys.modules[name] = pkg
    for mod in ("truncate", "synth"):
        spec = importlib.util.spec_from_file_location(f"{name}.{mod}",
                                                      os.path.join(REPO, "minkasi_gb300", f"{mod}.py"))
        m = importlib.util.module_from_spec(spec)
        sys.modules[spec.name] = m
        spec.loader.exec_module(m)
    return sys.modules[name + ".synth"]


def shard(shapes, rank, world):
    """The TOD indices this rank owns (greedy largest-first on the transform
    cost, the same rule as minkasi_gb300.parallel.partition)."""
    import math
    costs = [float(nd) * n * math.log2(max(n, 2)) for nd, n in shapes]
    if world == 1:
        return list(range(len(shapes)))
    from minkasi_gb300 import parallel
    return parallel.partition(costs, world)[rank]


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []          # (host time, csv line)
        self.window = None       # (t0, t1) of the timed region

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def mark(self, t0: float, t1: float) -> None:
        self.window = (t0, t1)

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        """Samples taken inside the timed window; if the window is shorter
        than the sampling period, the samples just before and after it."""
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self.lines
        scope = "timed region"
        if self.window is not None:
            t0, t1 = self.window
            inside = [l for t, l in lines if t0 <= t <= t1]
            if not inside:
                before = [l for t, l in lines if t < t0][-1:]
                after = [l for t, l in lines if t > t1][:1]
                inside = before + after
                scope = "nearest samples around the timed region"
            lines = inside
        else:
            lines = [l for _, l in lines]
        for ln in lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm), "scope": scope}


# ---------------------------------------------------------------- workload
def build_workload(cfg_name, device, with_noise, rank=0, world=1):
    import torch
    from minkasi_gb300 import synth
    from minkasi_gb300.maps import SkyMap
    from minkasi_gb300.tods import Tod, TodVec

    cfg = synth.CONFIGS[cfg_name]
    tv = TodVec()
    gen = torch.Generator(device=device)
    gen.manual_seed(1)
    shapes = synth.tod_shapes(cfg)
    mine = set(shard(shapes, rank, world))
    for k, (ndet, n) in enumerate(shapes):
        if k not in mine:
            continue
        if with_noise:
            info = synth.make_tod_info(cfg, k, ndet, n, device)
            tod = Tod(info)
            tod.set_noise()
        else:
            info = synth.make_tod_info(cfg, k, ndet, n, device, with_data=False)
            info["dat_calib"] = torch.randn((ndet, n), generator=gen, dtype=torch.float64, device=device)
            tod = Tod(info)
        tv.add_tod(tod)
    m = SkyMap(nx=cfg.nx, ny=cfg.ny, device=device)
    total = sum(nd * n for nd, n in shapes)
    return cfg, tv, m, total


def time_steps(fn, steps, warmup, stream, clk=None):
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    t0 = time.perf_counter()
    for a, b in ev:
        a.record(stream)
        fn()
        b.record(stream)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    if clk is not None:
        clk.mark(t0, t1)
    per = [a.elapsed_time(b) for a, b in ev]
    return sum(per), per, t1 - t0


# ---------------------------------------------------------------- CPU baseline
def cpu_tod2map_sample(tods_host, npix, seconds=12.0, prefer_ref=True):
    """Time the CPU tod2map over host copies of some TODs, all threads.
    Returns (GB/s, description, kind, cores)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle

    ref = oracle.ref_lib() if prefer_ref else None
    cores = os.cpu_count() or 1
    mp = np.zeros(npix)
    reps, nbytes, t_used = 0, 0, 0.0
    t_start = time.perf_counter()
    while time.perf_counter() - t_start < seconds:
        for ip, d in tods_host:
            t0 = time.perf_counter()
            if ref is not None:
                ref.tod2map_omp(mp.ctypes.data, d.ctypes.data, d.shape[0], d.shape[1], ip.ctypes.data,
                                npix)
            else:
                oracle.tod2map(mp, d, ip, nthread=cores)
            t_used += time.perf_counter() - t0
            nbytes += d.size * BYTES_PER_SAMPLE
        reps += 1
    kind = "reference" if ref is not None else "port"
    desc = (f"{len(tods_host)} of the workload's TODs ({sum(d.size for _, d in tods_host)} samples) "
            f"x {reps} passes, {cores} threads, {'reference tod2map_omp (minkasi.c) built from source' if ref is not None else 'oracle C restatement of tod2map_omp'}")
    return nbytes / t_used / 1e9, desc, kind, cores


def cpu_pcg_iter_sample(sample, npix, total_samples, seconds=20.0):
    """Seconds per PCG iteration of the reference's CPU operator (map2tod +
    NoiseSmoothedSVD.apply_noise with scipy's DCT-I, the shipped transform,
    on all host threads + tod2map), measured on the sample TODs and scaled
    to all of the workload's samples.  The noise operands are random arrays
    of the TODs' shapes: the time of these dense operations does not depend
    on their values."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle

    cores = os.cpu_count() or 1
    rng = np.random.default_rng(0)
    x = rng.standard_normal(npix)
    out = np.zeros(npix)
    used, samp, ntod = 0.0, 0, 0
    for ip, _ in sample:
        nd, n = ip.shape
        v = rng.standard_normal((nd, nd))
        vT = np.ascontiguousarray(v.T)
        w = rng.random((nd, n))
        d = np.zeros(ip.shape)
        t0 = time.perf_counter()
        oracle.map2tod(d, x, ip, False)
        d = oracle.apply_noise(v, vT, w, d, None, workers=cores)
        oracle.tod2map(out, np.ascontiguousarray(d), ip, nthread=cores)
        used += time.perf_counter() - t0
        samp += ip.size
        ntod += 1
        if used >= seconds:
            break
    return {"s_per_iter": used / samp * total_samples, "unit": "s", "cores": cores, "kind": "port",
            "sample": f"{ntod} of the workload's TODs ({samp} samples), scaled to {total_samples} samples; "
                      f"oracle C projections + numpy/scipy DCT-I apply_noise, {cores} threads"}


def cpu_sample(cfg_name, max_samples=3.5e8):
    """Host copies of the workload's first TODs: the same pointing as the GPU
    arm (synth on the CPU) and Gaussian timestreams."""
    import torch
    synth = load_synth()
    cfg = synth.CONFIGS[cfg_name]
    shapes = synth.tod_shapes(cfg)
    sample, tot = [], 0
    for k, (ndet, n) in enumerate(shapes):
        if tot >= max_samples:
            break
        info = synth.make_tod_info(cfg, k, ndet, n, torch.device("cpu"), with_data=False, with_radec=False)
        d = np.random.default_rng(k).standard_normal((ndet, n))
        sample.append((np.ascontiguousarray(info["ipix"].numpy()), d))
        tot += d.size
    return cfg, shapes, sample


def cpu_baseline_subprocess(args):
    """Run this script's reference arm in a fresh process (no torch CUDA
    context, no GPU library): the cpu_baseline and the CPU operator time."""
    cmd = [sys.executable, os.path.abspath(__file__), "--impl", "reference", "--steps", "3", "--warmup", "1",
           "--config", args.config, "--cpu-pcg"]
    env = dict(os.environ)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        env.pop(k, None)
    try:
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env)
        lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
        return json.loads(lines[-1]) if lines else {"error": r.stderr[-400:]}
    except (subprocess.TimeoutExpired, ValueError) as e:
        return {"error": str(e)}


# ---------------------------------------------------------------- arms
def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    cfg, shapes, sample = cpu_sample(args.config)
    npix = cfg.nx * cfg.ny
    vals = []
    desc = kind = None
    cores = os.cpu_count()
    for _ in range(args.warmup):
        cpu_tod2map_sample(sample, npix, seconds=0.5)
    for _ in range(args.steps):
        v, desc, kind, cores = cpu_tod2map_sample(sample, npix, seconds=4.0)
        vals.append(v)
    value = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "sample": desc},
            "cpu_baseline": {"value": value, "unit": "GB/s", "cores": cores, "kind": kind,
                             "sample": desc},
            "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "vs_baseline": None}
    if args.cpu_pcg:
        line["pcg_iter_cpu_reference"] = cpu_pcg_iter_sample(sample, npix, sum(nd * n for nd, n in shapes))
    print(json.dumps(line))


def c4_subprocess(args):
    """The 200-TOD solves in a fresh process on the whole GPU (they peak near
    240 GB, so they run before this process allocates anything)."""
    cmd = [sys.executable, os.path.abspath(__file__), "--c4-only"]
    env = dict(os.environ)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        env.pop(k, None)
    try:
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=3000, env=env)
        lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
        return json.loads(lines[-1]) if lines else {"error": r.stderr[-600:]}
    except (subprocess.TimeoutExpired, ValueError) as e:
        return {"error": str(e)}


def run_c4_only(args):
    import torch
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    import minkasi_gb300  # noqa: F401
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()
        rec = solve_c4(dev)
        clk.mark(t0, time.perf_counter())
    rec["clocks"] = clk.summary()
    print(json.dumps(rec))


def run_ours(args):
    rank, world, local = dist_env()
    c4 = None
    if world == 1 and not args.no_solver and not args.no_c4:
        c4 = c4_subprocess(args)
    import torch
    if world > 1:
        torch.distributed.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    import minkasi_gb300  # noqa: F401
    from minkasi_gb300 import kernels as K
    from minkasi_gb300 import parallel

    with_noise = not args.no_pcg
    cfg, tv, m, S_total = build_workload(args.config, dev, with_noise, rank, world)
    if args.method:
        tv.tod2map_method = args.method
    op = tv.engine(m)
    S = op.S
    for view, t in zip(op.views(op.tmp), tv.tods):
        view.copy_(t.info["dat_calib"])
    out = torch.zeros(op.npix, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream()

    def step():
        op.project_out(out)
        parallel.allreduce_(out)

    def max_over_ranks(x):
        t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
        if world > 1:
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        return float(t.item())

    # dominant-kernel timing: the scatter kernel alone, on the launching stream
    parallel.barrier()
    with ClockSampler(local) as clk:
        total_ms, per, wall = time_steps(step, args.steps, args.warmup, stream, clk)
    parallel.barrier()
    rank_ms_step = total_ms / args.steps
    ms_step = max_over_ranks(total_ms) / args.steps
    gbs = S_total * BYTES_PER_SAMPLE / (ms_step * 1e-3) / 1e9
    launches_per_step = {"atomic": 1, "staged": 1, "fixed": 4, "sorted": len(tv.tods)}[op.method]
    method, ntod_rank = op.method, len(tv.tods)

    # e2e through the public API with host buffers
    host = [t.info["dat_calib"].cpu().pin_memory() for t in tv.tods]
    h2d = sum(h.numel() * 8 for h in host)
    devbuf = [torch.empty_like(t.info["dat_calib"]) for t in tv.tods]

    def e2e_api():
        # SkyMap.tod2map on pinned host timestreams: the API copies them in
        # chunks on a copy stream, overlapped with the scatter of the
        # previous chunk (HostStager)
        m.clear()
        for t, h in zip(tv.tods, host):
            m.tod2map(t, h)
        m.mpi_reduce()
        return m.map.cpu()

    def e2e_copy():
        # the same with one blocking-order copy per TOD before its scatter
        m.clear()
        for t, h, d in zip(tv.tods, host, devbuf):
            d.copy_(h, non_blocking=True)
            m.tod2map(t, d)
        m.mpi_reduce()
        return m.map.cpu()

    def seconds_per_step(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        parallel.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            fn()
        torch.cuda.synchronize()
        return max_over_ranks((time.perf_counter() - t0) / args.steps)

    e2e_s = seconds_per_step(e2e_api)
    e2e_copy_s = seconds_per_step(e2e_copy)
    e2e_gbs = S_total * BYTES_PER_SAMPLE / e2e_s / 1e9
    e2e_copy_gbs = S_total * BYTES_PER_SAMPLE / e2e_copy_s / 1e9
    h2d_total = int(max_over_ranks(h2d)) * world if world > 1 else h2d
    del devbuf, host

    # extras: the other projection on the same samples (map2tod, FP64, set
    # mode: 4 B pixel index read + 8 B sample written), and the full hot path
    # per PCG iteration
    extras = {}
    src = torch.randn(op.npix, dtype=torch.float64, device=dev)
    m2t_ms, _, _ = time_steps(lambda: K.map2tod(op.tmp, src, op.ipix, False), args.steps, args.warmup, stream)
    m2t_gbs = S * BYTES_PER_SAMPLE / (m2t_ms / args.steps * 1e-3) / 1e9
    extras["map2tod"] = {"value": m2t_gbs, "unit": "GB/s", "ms_per_step": m2t_ms / args.steps,
                         "frac_of_hbm": None, "bytes_per_sample": BYTES_PER_SAMPLE,
                         "kernel": "k_map2tod_vec"}
    if with_noise and world == 1:
        extras.update(pcg_extras(tv, m, dev))

    peaks = {}
    try:
        peaks = json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    extras["map2tod"]["frac_of_hbm"] = extras["map2tod"]["value"] / peak
    clocks = clk.summary() if rank == 0 else None
    # DRAM bytes per sample of the scatter kernel from one ncu capture of the
    # small case (dram__bytes_read.sum + dram__bytes_write.sum), scaled to a
    # full launch by the sample count
    per_sample = NCU_DRAM_BYTES_PER_SAMPLE.get(op.method)
    traffic = None if per_sample is None else per_sample * S
    achieved = S * BYTES_PER_SAMPLE / (rank_ms_step * 1e-3) / 1e9
    nlaunch = launches_per_step * args.steps

    solver = None
    if world == 1 and not args.no_solver:
        # free the c2 workload before the solver configurations
        del op, out, src
        tv._engines.clear()
        tv._shared.clear()
        del tv, m
        import gc
        from minkasi_gb300.noise import clear_plan_cache
        clear_plan_cache()
        gc.collect()
        torch.cuda.empty_cache()
        solver = solver_extras(dev, c4)

    cpu = None
    if rank == 0 and world == 1:
        ref = cpu_baseline_subprocess(args)
        if "value" in ref:
            cpu = dict(ref["cpu_baseline"])
            if with_noise and "pcg_iter_cpu_reference" in ref:
                extras["pcg_iter_cpu_reference"] = ref["pcg_iter_cpu_reference"]
        else:
            cpu = {"value": None, "unit": "GB/s", "error": ref.get("error")}
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": gbs, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "strong" if world > 1 else "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "samples": S_total, "samples_rank0": S, "ntod_rank0": ntod_rank,
                   "npix": int(cfg.nx * cfg.ny), "tod2map_kernel": method,
                   "l2": "inputs (12 B x samples) larger than L2; no flush",
                   "parallelism": (f"TODs sharded over {world} ranks, map all-reduce per step" if world > 1
                                   else "1 GPU")},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "kernel": {"atomic": "k_tod2map_atomic8", "staged": "k_tod2map_staged",
                                "fixed": "k_scatter_fixed8", "sorted": "k_tod2map_sorted"}[method],
                     "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)"},
        "e2e": {"value": e2e_gbs, "unit": "GB/s", "h2d_bytes_per_step": h2d_total,
                "d2h_bytes_per_step": int(cfg.nx * cfg.ny) * 8,
                "mode": "SkyMap.tod2map per TOD on pinned host timestreams (chunked copies overlapped "
                        "with the scatter), map read back every step",
                "serial_copy_then_scatter": e2e_copy_gbs},
        "gpu_launches": nlaunch,
        "clocks": clocks,
        "cpu_baseline": cpu,
        "wall_s_timed": wall,
    }
    line.update(extras)
    if solver is not None:
        line["solver"] = solver
    print(json.dumps(line))


def pcg_extras(tv, m, dev):
    """Time FP64 Jacobi PCG iterations and FP32 inner iterations (graph replay)."""
    import torch
    import minkasi_gb300 as mk
    from minkasi_gb300.pcg import DevicePCG

    mapset = mk.Mapset()
    mapset.add_map(m)
    rhs = mapset.copy()
    tv.make_rhs(rhs)
    pre = mk.jacobi_precon(mk.make_hits(tv, m))
    S = tv.get_nsamp()
    res = {}
    for name, dtype in (("pcg_iter_f64", torch.float64), ("pcg_iter_f32_inner", torch.float32)):
        op = tv.engine(m, dtype)
        b = rhs.maps[0].map.reshape(-1).to(dtype)
        x = torch.zeros_like(b)
        st = DevicePCG(op, b, x, pre.maps[0].map, graph=True)
        st.start()
        st.step()  # eager first iteration, then captured
        st.step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n = 3
        e0.record()
        for _ in range(n):
            st.step()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / n
        res[name] = {"ms": ms, "Msamp_per_s": S / (ms * 1e-3) / 1e6, "tod2map_kernel": op.method,
                     "rot_mode": op.rot_mode}
        del st
    return res


# ---------------------------------------------------------------- solver
def _timed(fn, reps=1):
    """(result, wall seconds of the last of ``reps`` calls, of the first)."""
    import torch
    first = None
    out = None
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        first = dt if first is None else first
    return out, dt, first


def _true_rel(op64, b, x):
    """||b - A x|| / ||b|| with the FP64 operator (sum over ranks)."""
    import torch
    from minkasi_gb300.pcg import _true_residual, global_op
    return _true_residual(global_op(op64), b.reshape(-1), x.reshape(-1))


def solve_c1(dev, tol=1e-6):
    """The 1-TOD configuration (64 x 65,341 samples, 256^2 map): FP64 Jacobi
    PCG, mixed Jacobi and mixed learned to the FP64 tolerance.  Each wall time
    is the second of two identical solves (the first adds graph captures)."""
    import torch
    import minkasi_gb300 as mk
    from minkasi_gb300 import learned as L
    from minkasi_gb300 import synth

    t0 = time.perf_counter()
    cfg = synth.CONFIGS["c1"]
    tv, m = synth.make_todvec(cfg, dev)
    mapset = mk.Mapset()
    mapset.add_map(m)
    rhs = mapset.copy()
    tv.make_rhs(rhs)
    hits = mk.make_hits(tv, m)
    pre = mk.jacobi_precon(hits)
    x0 = rhs.copy()
    x0.clear()
    net = L.load(L.weights_path("c1"), dev)
    ml = L.LearnedPrecon(hits.map, net, (m.nx, m.ny))
    op64 = tv.engine(m, torch.float64)
    tv.engine(m, torch.float32)
    out = {"workload": "c1: 1 TOD x 64 det x 65,341 samples, 256x256 map at 2in", "tol": tol,
           "samples": tv.get_nsamp(), "setup_s": time.perf_counter() - t0,
           "learned_weights": os.path.relpath(L.weights_path("c1"), REPO)}
    runs = {
        "jacobi_f64": lambda: mk.run_pcg(rhs, x0, tv, pre, maxiter=5000, tol=tol, verbose=False),
        "mixed_jacobi": lambda: mk.run_pcg_mixed(rhs, x0, tv, pre, tol=tol),
        "mixed_learned": lambda: mk.run_pcg_mixed(rhs, x0, tv, pre, tol=tol, inner_precon=ml),
    }
    for name, fn in runs.items():
        x, wall, cold = _timed(fn, reps=2)
        rec = {"wall_s": wall, "cold_wall_s": cold, "iters": int(x.niter),
               "true_rel_residual": _true_rel(op64, rhs.maps[0].map, x.maps[0].map)}
        if hasattr(x, "outer"):
            rec["fp64_residuals"] = int(x.outer)
        out[name] = rec
    jf = out["jacobi_f64"]["wall_s"]
    out["speedup_mixed_jacobi_vs_jacobi_f64"] = jf / out["mixed_jacobi"]["wall_s"]
    out["speedup_mixed_learned_vs_jacobi_f64"] = jf / out["mixed_learned"]["wall_s"]
    out["speedup_learned_vs_jacobi_mixed"] = out["mixed_jacobi"]["wall_s"] / out["mixed_learned"]["wall_s"]
    out["precision"] = precision_c1(tv, m, hits, pre, ml, op64, dev)
    return out


def precision_c1(tv, m, hits, pre, ml, op64, dev):
    """The precision configuration on the 1-TOD inputs: a system with a known
    solution, b = A s (FP64 operator) for a seeded sky s on the hit pixels,
    solved from x0 = 0 by the mixed-precision PCG (FP32 operator with 3xTF32
    tensor-core rotations; FP64 dots and residual replacement) and by
    classic iterative refinement (FP64 residual, 20 FP32 inner PCG
    iterations per step).  At every FP64 residual evaluation: the true
    residual and the map error against s, hit-region mean removed (A
    annihilates a constant)."""
    import torch
    import minkasi_gb300 as mk
    from minkasi_gb300 import learned as L

    hit = hits.map.reshape(-1) > 0
    s = L.sky(m.nx, m.ny, 2.0, 4242, dev).reshape(-1)
    s = torch.where(hit, s, torch.zeros_like(s))
    bmap = mk.Mapset()
    bmap.add_map(m.copy())
    op64.apply(s, bmap.maps[0].map.reshape(-1))
    x0 = bmap.copy()
    x0.clear()
    sh = s[hit] - s[hit].mean()

    def err(xf):
        a = xf.reshape(-1)[hit]
        a = a - a.mean()
        return float(torch.linalg.norm(a - sh) / torch.linalg.norm(sh))

    out = {"system": "b = A s, s = seeded sky (GRF + clusters) on the hit pixels; errors vs s, "
                     "hit-region mean removed"}
    for name, kw in (("mixed_reliable", {"tol": 1e-10, "max_iter": 6000}),
                     ("mixed_reliable_learned", {"tol": 1e-10, "max_iter": 6000, "inner_precon": ml}),
                     ("classic_refine_20", {"tol": 1e-10, "mode": "refine", "inner_iters": 20,
                                            "max_outer": 60})):
        steps = []
        cb = lambda k, xf, rel: steps.append([int(k), float(rel), err(xf)])
        x = mk.run_pcg_mixed(bmap, x0, tv, pre, on_outer=cb, **kw)
        out[name] = {"iters": int(x.niter), "final_true_rel_residual": float(x.rel_residual),
                     "final_map_err": err(x.maps[0].map), "per_step": steps}
    return out


def solve_c4(dev, tol=1e-6, wall_limit_s=420.0):
    """The 200-TOD configuration (8.8e9 samples, 2048^2 map): setup, the FP32
    projections' GB/s, the FP64 Jacobi iteration time, and the mixed solves
    (Jacobi, learned) to the FP64 tolerance, each bounded in wall time."""
    import torch
    from minkasi_gb300 import kernels as K
    from minkasi_gb300 import learned as L
    from minkasi_gb300 import synth
    from minkasi_gb300.maps import Mapset
    from minkasi_gb300.pcg import DevicePCG, MixedOp, run_pcg_mixed
    from minkasi_gb300.projections import make_hits

    cfg = synth.CONFIGS["c4"]
    t0 = time.perf_counter()
    tv, m, rhs = L.build_large(cfg, dev, log=None)
    hits = make_hits(tv, m).map.reshape(-1)
    pre = torch.where(hits > 0, 1.0 / hits.clamp(min=1), torch.zeros_like(hits))
    op64 = tv.engine(m, torch.float64)
    op32 = tv.engine(m, torch.float32)
    torch.cuda.synchronize()
    S = tv.get_nsamp()
    out = {"workload": "c4: 200 TODs, ndet in {32,64,128,256}, nsamp U[5e4,6e5] (truncated), 2048x2048 map "
                       "at 0.5in", "tol": tol, "samples": S, "ntod": tv.ntod,
           "setup_s": time.perf_counter() - t0,
           "tod2map_kernel_f32": op32.method, "rot_mode_f32": op32.rot_mode, "rot_mode_f64": op64.rot_mode,
           "dct_engines_f32": sorted(set(int(v) for v in op32.dct_engines.values())),
           "gpu_mem_GB_peak": torch.cuda.max_memory_allocated() / 1e9,
           "learned_weights": os.path.relpath(L.weights_path("c4"), REPO)}
    stream = torch.cuda.current_stream()
    # FP32 projections at this scale (8 B per sample: 4 B index + 4 B sample)
    src = torch.randn(m.npix, dtype=torch.float32, device=dev)
    acc = torch.zeros(m.npix, dtype=torch.float32, device=dev)
    ms, _, _ = time_steps(lambda: K.map2tod(op32.tmp, src, op32.ipix, False), 5, 3, stream)
    out["map2tod_f32_GBps"] = S * 8 / (ms / 5 * 1e-3) / 1e9
    ms, _, _ = time_steps(lambda: op32.project_out(acc), 5, 3, stream)
    out["tod2map_f32_GBps"] = S * 8 / (ms / 5 * 1e-3) / 1e9
    del src, acc
    # one FP64 Jacobi PCG iteration (operator + fused update), eager
    st = DevicePCG(op64, rhs, torch.zeros_like(rhs), pre, graph=False)
    st.start(Ax=torch.zeros_like(rhs))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    st.step()
    e1.record()
    e1.synchronize()
    ms64 = e0.elapsed_time(e1)
    out["jacobi_f64_iter_ms"] = ms64
    del st
    mp = m.copy()
    mp.map.copy_(rhs.view(m.nx, m.ny))
    b = Mapset()
    b.add_map(mp)
    x0 = b.copy()
    x0.clear()
    pre_ms = b.copy()
    pre_ms.maps[0].map.copy_(pre.view(m.nx, m.ny))
    ml = L.LearnedPrecon(hits, L.load(L.weights_path("c4"), dev), (m.nx, m.ny))
    out["learned_pools"] = ml.pools
    budget = None
    for name, kw in (("mixed_jacobi", {}), ("mixed_learned", {"inner_precon": ml})):
        hist = []
        if budget is None:
            # iterations that fit the wall limit at the measured inner iteration
            stt = DevicePCG(MixedOp(op32, m.npix, dev), rhs, torch.zeros_like(rhs), pre, graph=True)
            stt.start()
            stt.step()
            stt.step()
            torch.cuda.synchronize()
            e0.record()
            for _ in range(3):
                stt.step()
            e1.record()
            e1.synchronize()
            inner_ms = e0.elapsed_time(e1) / 3
            out["mixed_inner_iter_ms"] = inner_ms
            del stt
            budget = max(100, int((wall_limit_s - 4 * ms64 / 1e3) * 1e3 / (inner_ms * 1.15)))
        x, wall, _ = _timed(lambda: run_pcg_mixed(b, x0, tv, pre_ms, tol=tol, max_iter=budget, history=hist, **kw))
        out[name] = {"wall_s": wall, "iters": int(x.niter), "fp64_residuals": int(x.outer),
                     "restarts": int(x.restarts), "true_rel_residual": float(x.rel_residual),
                     "reached_tol": bool(x.rel_residual <= tol), "iteration_budget": budget}
        del x
    it = out["mixed_jacobi"]["iters"]
    out["jacobi_f64_projected_s"] = it * ms64 / 1e3
    out["jacobi_f64_projected_note"] = ("measured FP64 Jacobi iteration x the mixed Jacobi solve's iteration "
                                        "count (the two counts agree on the 1-TOD configuration, where both run)")
    out["speedup_mixed_jacobi_vs_jacobi_f64_projected"] = out["jacobi_f64_projected_s"] / out["mixed_jacobi"]["wall_s"]
    out["speedup_mixed_learned_vs_jacobi_f64_projected"] = (out["jacobi_f64_projected_s"] /
                                                            out["mixed_learned"]["wall_s"])
    return out


def solver_extras(dev, c4=None):
    res = {"c1": solve_c1(dev)}
    if c4 is not None:
        res["c4"] = c4
    return res


def hit_density(hits) -> float:
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


def run_sparse(args):
    """c4sparse: 200 TODs of raster sweeps retracing 3 narrow tracks on the
    2048^2 map (about 5% of the footprint hit), FP64 timestreams: the
    autotuner's tod2map choice and the GB/s of each scatter kernel
    (12 B per sample), inputs resident in HBM."""
    import torch
    import minkasi_gb300  # noqa: F401
    from minkasi_gb300 import synth
    from minkasi_gb300.autotune import choose_tod2map
    from minkasi_gb300.maps import SkyMap
    from minkasi_gb300.tods import Tod, TodVec

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    cfg = synth.CONFIGS["c4sparse"]
    tv = TodVec()
    gen = torch.Generator(device=dev).manual_seed(1)
    for k, (nd, n) in enumerate(synth.tod_shapes(cfg)):
        info = synth.make_tod_info(cfg, k, nd, n, dev, with_data=False, with_radec=False)
        info["dat_calib"] = torch.randn((nd, n), generator=gen, dtype=torch.float64, device=dev)
        tv.add_tod(Tod(info))
    m = SkyMap(nx=cfg.nx, ny=cfg.ny, device=dev)
    op = tv.engine(m, torch.float64, tod2map="atomic")
    for view, t in zip(op.views(op.tmp), tv.tods):
        view.copy_(t.info["dat_calib"])
        t.info["dat_calib"] = t.info["dat_calib"].to("meta")
    torch.cuda.empty_cache()
    hits = op.hits()
    density = hit_density(hits.view(cfg.nx, cfg.ny))
    choice = choose_tod2map(op, ["atomic", "staged", "fixed"])
    for view in op.views(op.tmp):
        view.normal_()
    out = torch.zeros(op.npix, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream()
    res = {}
    for meth in ("atomic", "staged", "fixed"):
        ms, _, _ = time_steps(lambda: op.project_out(out, meth), args.steps, args.warmup, stream)
        res[meth] = op.S * BYTES_PER_SAMPLE / (ms / args.steps * 1e-3) / 1e9
    line = {"metric": "tod2map GB/s (sparse hits)", "value": res[choice], "unit": "GB/s",
            "workload": "c4sparse: 200 TODs, raster sweeps on 3 tracks, 2048x2048 map at 0.5in, FP64",
            "samples": op.S, "hit_pixels": int((hits > 0).sum().item()),
            "hit_density_in_footprint": density, "autotuner_choice": choice,
            "GBps_by_kernel": res, "note": "sorted not timed: its int32 sample plan needs S < 2^31"}
    print(json.dumps(line))


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    elif a.sparse:
        run_sparse(a)
    elif a.c4_only:
        run_c4_only(a)
    else:
        run_ours(a)
