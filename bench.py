"""Benchmark: tod2map GB/s on the 32-TOD FP64 workload (plus the PCG iteration).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (the reference's "plain method at GPU scale" configuration): 32
synthetic TODs, 256 detectors each, nsamp ~ U[2^17, 2^19] truncated to
FFT-friendly lengths, daisy-scan pointing onto a 1024x1024 map at 1",
FP64.  One step = one tod2map pass of every TOD's timestream into the map
(the projection of TodVec.make_rhs / TodVec.dot), inputs resident in HBM.
value = algorithmic bytes (4 B ipix + 8 B dat per sample) / step time.
The inputs (32 GB) exceed the 129 MB L2, so no flush is needed between steps.

e2e: the same step through the public API (SkyMap.tod2map per TOD) with the
timestream in pinned host memory, copied to the device inside the timed
region (in chunks overlapped with the scatter), and the map read back to the
host every step; the pixel indices stay cached on the device as the API
caches them (tod.info[tag]).

Extra keys: map2tod GB/s on the same samples; per-iteration timings of the
full hot path (FP64 Jacobi PCG iteration = batched A-apply + update, and the
FP32 inner iteration of the mixed-precision solver) on the same TODs, and
the reference's CPU operator per iteration (a bounded sample, scaled).

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
    ap.add_argument("--method", default=None, help="force the tod2map kernel (atomic|staged|fixed|sorted)")
    return ap.parse_args()


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
def build_workload(cfg_name, device, with_noise):
    import torch
    from minkasi_gb300 import synth
    from minkasi_gb300.maps import SkyMap
    from minkasi_gb300.tods import Tod, TodVec

    cfg = synth.CONFIGS[cfg_name]
    tv = TodVec()
    gen = torch.Generator(device=device)
    gen.manual_seed(1)
    for k, (ndet, n) in enumerate(synth.tod_shapes(cfg)):
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
    return cfg, tv, m


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


def cpu_pcg_iter_sample(tv, npix, seconds=20.0):
    """Seconds per PCG iteration of the reference's CPU operator (map2tod +
    NoiseSmoothedSVD.apply_noise with scipy's DCT-I, the shipped transform,
    on all host threads + tod2map), measured on the first TOD(s) of the
    workload and scaled to all of its samples."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle

    cores = os.cpu_count() or 1
    x = np.random.default_rng(0).standard_normal(npix)
    out = np.zeros(npix)
    used, samp, ntod = 0.0, 0, 0
    for t in tv.tods:
        nz = t.noise
        ip = np.ascontiguousarray(t.info["ipix"].cpu().numpy())
        v, vT, w = (a.detach().cpu().numpy() for a in (nz.v, nz.vT, nz.mywt))
        nv = None if nz.noisevec is None else nz.noisevec.detach().cpu().numpy()
        d = np.zeros(ip.shape)
        t0 = time.perf_counter()
        oracle.map2tod(d, x, ip, False)
        d = oracle.apply_noise(v, vT, w, d, nv, workers=cores)
        oracle.tod2map(out, d, ip, nthread=cores)
        used += time.perf_counter() - t0
        samp += ip.size
        ntod += 1
        if used >= seconds:
            break
    total = tv.get_nsamp()
    return {"s_per_iter": used / samp * total, "unit": "s", "cores": cores, "kind": "port",
            "sample": f"{ntod} of the workload's TODs ({samp} samples), scaled to {total} samples; "
                      f"oracle C projections + numpy/scipy DCT-I apply_noise, {cores} threads"}


def host_sample(tv, max_samples=3.5e8):
    out, tot = [], 0
    for t in tv.tods:
        if tot >= max_samples:
            break
        ip = t.info["ipix"].cpu().numpy()
        d = t.info["dat_calib"].cpu().numpy()
        out.append((np.ascontiguousarray(ip), np.ascontiguousarray(d)))
        tot += d.size
    return out


# ---------------------------------------------------------------- arms
def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    import torch
    from minkasi_gb300 import synth

    cfg = synth.CONFIGS[args.config]
    shapes = synth.tod_shapes(cfg)
    npix = cfg.nx * cfg.ny
    # the same pointing and the same kind of data as our arm, generated on
    # the CPU for a bounded sample of TODs
    dev = torch.device("cpu")
    sample = []
    tot = 0
    for k, (ndet, n) in enumerate(shapes):
        if tot >= 2.0e8:
            break
        info = synth.make_tod_info(cfg, k, ndet, n, dev, with_data=False)
        d = np.random.default_rng(k).standard_normal((ndet, n))
        sample.append((info["ipix"].numpy(), d))
        tot += d.size
    vals = []
    desc = kind = None
    cores = os.cpu_count()
    for _ in range(args.warmup):
        cpu_tod2map_sample(sample, npix, seconds=0.5)
    for _ in range(args.steps):
        v, desc, kind, cores = cpu_tod2map_sample(sample, npix, seconds=2.0)
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
    print(json.dumps(line))


def run_ours(args):
    import torch

    rank, world, local = dist_env()
    if world > 1:
        torch.distributed.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    import minkasi_gb300  # noqa: F401
    from minkasi_gb300 import kernels as K
    from minkasi_gb300 import parallel

    with_noise = not args.no_pcg
    cfg, tv, m = build_workload(args.config, dev, with_noise)
    # weak scaling: every rank runs the full workload on its own GPU and
    # the map is summed over ranks once per step (the reference's reduction)
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

    # dominant-kernel timing: the scatter kernel alone, on the launching stream
    parallel.barrier()
    with ClockSampler(local) as clk:
        total_ms, per, wall = time_steps(step, args.steps, args.warmup, stream, clk)
    parallel.barrier()
    tmax = torch.tensor([total_ms], dtype=torch.float64, device=dev)
    if world > 1:
        torch.distributed.all_reduce(tmax, op=torch.distributed.ReduceOp.MAX)
    total_ms = float(tmax.item())
    ms_step = total_ms / args.steps
    gbs = world * S * BYTES_PER_SAMPLE / (ms_step * 1e-3) / 1e9
    launches_per_step = {"atomic": 1, "staged": 1, "fixed": 4, "sorted": len(tv.tods)}[op.method]

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
        return m.map.cpu()

    def e2e_copy():
        # the same with one blocking-order copy per TOD before its scatter
        m.clear()
        for t, h, d in zip(tv.tods, host, devbuf):
            d.copy_(h, non_blocking=True)
            m.tod2map(t, d)
        return m.map.cpu()

    def seconds_per_step(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / args.steps

    e2e_s = seconds_per_step(e2e_api)
    e2e_copy_s = seconds_per_step(e2e_copy)
    e2e_gbs = world * S * BYTES_PER_SAMPLE / e2e_s / 1e9
    e2e_copy_gbs = world * S * BYTES_PER_SAMPLE / e2e_copy_s / 1e9
    del devbuf, host

    # extras: the other projection on the same samples (map2tod, FP64, set
    # mode: 4 B pixel index read + 8 B sample written), and the full hot path
    # per PCG iteration
    extras = {}
    src = torch.randn(op.npix, dtype=torch.float64, device=dev)
    m2t_ms, _, _ = time_steps(lambda: K.map2tod(op.tmp, src, op.ipix, False), args.steps, args.warmup, stream)
    m2t_gbs = S * BYTES_PER_SAMPLE / (m2t_ms / args.steps * 1e-3) / 1e9
    extras["map2tod"] = {"value": m2t_gbs, "unit": "GB/s", "ms_per_step": m2t_ms / args.steps,
                         "frac_of_hbm": None, "bytes_per_sample": BYTES_PER_SAMPLE}
    if with_noise and rank == 0:
        extras.update(pcg_extras(tv, m, dev))

    peaks = {}
    try:
        peaks = json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    extras["map2tod"]["frac_of_hbm"] = extras["map2tod"]["value"] / peak
    cpu = None
    if rank == 0 and world == 1:
        v, desc, kind, cores = cpu_tod2map_sample(host_sample(tv), op.npix, seconds=12.0)
        cpu = {"value": v, "unit": "GB/s", "cores": cores, "kind": kind, "sample": desc}
        if with_noise:
            extras["pcg_iter_cpu_reference"] = cpu_pcg_iter_sample(tv, op.npix)
    if rank != 0:
        return
    clocks = clk.summary()
    # DRAM bytes per sample of the scatter kernel from one ncu capture of the
    # small case (dram__bytes_read.sum + dram__bytes_write.sum), scaled to a
    # full launch by the sample count
    per_sample = NCU_DRAM_BYTES_PER_SAMPLE.get(op.method)
    traffic = None if per_sample is None else per_sample * S
    line = {
        "metric": METRIC, "value": gbs, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "samples": S, "ntod": len(tv.tods), "npix": op.npix,
                   "tod2map_kernel": op.method, "l2": "inputs (12 B x samples) larger than L2; no flush",
                   "parallelism": f"replicas x{world}, map all-reduce per step"},
        "roofline": {"bound": "hbm", "achieved": gbs / world, "peak": peak, "unit": "GB/s",
                     "frac": gbs / world / peak, "traffic": traffic,
                     "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)"},
        "e2e": {"value": e2e_gbs, "unit": "GB/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": op.npix * 8,
                "mode": "SkyMap.tod2map per TOD on pinned host timestreams (chunked copies overlapped "
                        "with the scatter), map read back every step",
                "serial_copy_then_scatter": e2e_copy_gbs},
        "gpu_launches": launches_per_step * args.steps,
        "clocks": clocks,
        "cpu_baseline": cpu,
        "wall_s_timed": wall,
    }
    line.update(extras)
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


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)
