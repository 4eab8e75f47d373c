"""Build libmkgpu.so in-tree for sm_103a (GB300).

    python minkasi_gb300/build.py          # incremental
    python minkasi_gb300/build.py --force

Each .cu under csrc/ is compiled by its own nvcc process (in parallel) into
_build/, then linked with cuFFT and cuBLAS into minkasi_gb300/libmkgpu.so.
No CMake, no torch extension machinery: the library is a plain C-ABI shared
object loaded with ctypes.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libmkgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmkgpu.so")


def _cuda_lib_dir(nvcc: str) -> str:
    root = os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    for sub in ("lib64", "lib", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib"):
        d = os.path.join(root, sub)
        if os.path.exists(os.path.join(d, "libcufft.so")):
            return d
    return os.path.join(root, "lib64")


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(REPO, "include", "*.h"))


def _stale(out: str, deps) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> str:
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdrs = _headers()
    flags = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3", "--expt-relaxed-constexpr",
             "-I", os.path.join(REPO, "include"), *ARCH, *extra_flags]
    jobs = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s)[:-3] + ".o")
        if force or _stale(o, [s, *hdrs]):
            jobs.append([nvcc, *flags, "-c", s, "-o", o])
    objs = [os.path.join(BUILD, os.path.basename(s)[:-3] + ".o") for s in srcs]

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {cmd[-3]}:\n{r.stdout}\n{r.stderr}")
        return r.stderr

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for err in ex.map(run, jobs):
                if verbose and err.strip():
                    print(err, file=sys.stderr)
    if force or jobs or _stale(LIB, objs):
        libdir = _cuda_lib_dir(nvcc)
        tmp = LIB + ".tmp"
        run([nvcc, "-shared", *ARCH, "-o", tmp, *objs, "-L", libdir, "-lcufft", "-lcublas",
             "-Xlinker", "-rpath," + libdir])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, verbose=a.verbose))
