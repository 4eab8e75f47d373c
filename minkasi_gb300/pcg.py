"""Preconditioned conjugate gradients (minkasi/mapmaking/pcg.py:22-255).

``run_pcg`` / ``run_pcg_wprior`` keep the reference's signatures and
recurrence (same order of updates, fixed ``maxiter`` unless the new ``tol``
keyword is given).  On the fast path (one SkyMap, SmoothedSVD noise, no
prior) an iteration is: one batched A-apply (map2tod, per-TOD noise filter,
tod2map) + three fused update kernels with every scalar on the device, and
from the second iteration on the whole iteration is replayed as one CUDA
graph -- no host round trip per iteration.

``run_pcg_mixed`` is the mixed-precision solver: FP64 vectors, dot products
and scalars around FP32 operator applications, refined by FP64 true
residuals (residual replacement) until ||b - A x|| / ||b|| reaches ``tol``.

With more than one rank (torch.distributed), each rank holds its own TODs
and every operator application inside these solvers is followed by a sum of
the map over ranks (``RankSumOp``), as the reference's TodVec.dot does
(minkasi/tods/core.py:1021-1022).  The maps, and so every PCG scalar, are
then identical on all ranks.  Iterations are not captured as CUDA graphs
in that case: the exchange runs on the host (gloo) or as a separate NCCL
call between the captured halves.
"""
from __future__ import annotations

import math
import sys
import time
from typing import List, Optional

import numpy as np
import torch

from . import kernels as K
from . import parallel
from ._lib import MK_S_FLAG, MK_S_ITER, MK_S_RR, MK_S_ZR
from .maps import Mapset, SkyMap, _reducer
from .tods import TodVec


class HasPrior:
    """Protocol of a prior: apply_prior(x, Ax) adds Q^-1 x to Ax (pcg.py:17-19)."""

    def apply_prior(self, x, Ax):  # pragma: no cover - protocol
        raise NotImplementedError


class null_precon:
    """A preconditioner that does nothing (pcg.py:241-255)."""

    def __init__(self):
        self.isnull = True

    def __add__(self, val):
        return val

    def __mul__(self, val):
        return val


class RankSumOp:
    """A rank's operator followed by the sum of the map over ranks: the one
    exchange per operator application of the reference's TodVec.dot
    (minkasi/tods/core.py:1021-1022 -> minkasi/maps/skymap.py:742-783).
    ``op`` applies this rank's share, A_r = sum over its TODs of P^T N P."""

    def __init__(self, op):
        self.op = op

    def __getattr__(self, name):
        return getattr(self.op, name)

    def apply(self, x: torch.Tensor, out: torch.Tensor, accumulate: bool = False) -> torch.Tensor:
        if not accumulate:
            self.op.apply(x, out)
            parallel.allreduce_(out)
            return out
        part = self.op.apply(x, torch.empty_like(out))
        parallel.allreduce_(part)
        out.add_(part)
        return out


def global_op(op):
    """The operator summed over ranks; the local operator itself on one rank."""
    return RankSumOp(op) if parallel.have_mpi() else op


def _is_map_precon(precon) -> bool:
    return (isinstance(precon, Mapset) and precon.nmap == 1 and isinstance(precon.maps[0], SkyMap)) \
        or hasattr(precon, "apply")


def _precon_arg(precon):
    if precon is None:
        return None
    return precon if hasattr(precon, "apply") else precon.maps[0].map


class DevicePCG:
    """Device-resident PCG state for one operator (flat maps of its dtype)."""

    def __init__(self, op, b: torch.Tensor, x: torch.Tensor, M: Optional[torch.Tensor],
                 graph: bool = True):
        self.op = op
        self.n = b.numel()
        dt, dev = b.dtype, b.device
        self.b = b.reshape(-1)
        self.x = x.reshape(-1)
        # a diagonal preconditioner (map) is fused into the update kernels; an
        # operator (anything with apply(r, z), e.g. LearnedPrecon) runs between
        # the two halves of the split update
        self.Mop = M if hasattr(M, "apply") else None
        self.M = None if (M is None or self.Mop is not None) else M.reshape(-1).to(dt).contiguous()
        self.r = torch.empty(self.n, dtype=dt, device=dev)
        self.z = torch.empty_like(self.r)
        self.p = torch.empty_like(self.r)
        self.Ap = torch.empty_like(self.r)
        self.s = torch.zeros(8, dtype=torch.float64, device=dev)
        self.red = _reducer(dev)
        self.graph_enabled = graph
        self._graph = None
        self.iters = 0

    def start(self, Ax: Optional[torch.Tensor] = None) -> None:
        if Ax is None:
            self.op.apply(self.x, self.Ap)
            Ax = self.Ap
        K.pcg_init(self.r, self.z, self.p, self.b, Ax.reshape(-1), self.M, self.s, self.red)
        if self.Mop is not None:
            self.Mop.apply(self.r, self.z)
            self.p.copy_(self.z)
            self.red.dot(self.r, self.z, out=self.s[MK_S_ZR])
        self.iters = 0

    def _step(self) -> None:
        self.op.apply(self.p, self.Ap)
        if self.Mop is None:
            K.pcg_update(self.x, self.r, self.z, self.p, self.Ap, self.M, self.s, self.red)
        else:
            K.pcg_step_xr(self.x, self.r, self.p, self.Ap, self.s, self.red)
            self.Mop.apply(self.r, self.z)
            K.pcg_step_zp(self.z, self.r, self.p, self.s, self.red)

    def step(self) -> None:
        if self.graph_enabled and self.iters >= 1:
            if self._graph is None:
                g = torch.cuda.CUDAGraph()
                with torch.cuda.graph(g):
                    self._step()
                self._graph = g
            self._graph.replay()
        else:
            self._step()
        self.iters += 1

    def scalars(self) -> np.ndarray:
        return self.s.cpu().numpy()


def _true_residual(op, b: torch.Tensor, x: torch.Tensor) -> float:
    ax = torch.empty_like(b)
    op.apply(x, ax)
    r = b.reshape(-1) - ax.reshape(-1)
    red = _reducer(b.device)
    return math.sqrt(red.dot(r, r).item()) / math.sqrt(red.dot(b.reshape(-1), b.reshape(-1)).item())


def run_pcg_wprior(b: Mapset, x0: Mapset, tods: TodVec, prior=None, precon=None,
                   mask: Optional[Mapset] = None, maxiter: int = 25, outroot: str = "map",
                   save_iters: List[int] = [-1], save_ind: int = 0, save_tail: str = ".fits",
                   plot_iters: List[int] = [], plot_info=None, plot_ind: int = 0, *,
                   tol: Optional[float] = None, check_every: int = 10, graph: bool = True,
                   verbose: bool = True, history: Optional[list] = None) -> Mapset:
    """PCG on A x = b (pcg.py:22-200).  With ``tol`` set, stops once the
    FP64 true residual ||b - A x||/||b|| <= tol (checked when the recursive
    residual says so, every ``check_every`` iterations)."""
    fast = (prior is None and mask is None and isinstance(tods, TodVec) and tods._fast(b)
            and (precon is None or _is_map_precon(precon)))
    if not fast:
        return _run_pcg_generic(b, x0, tods, prior, precon, mask, maxiter, outroot, save_iters,
                                save_ind, save_tail, verbose, history)
    t0 = time.time()
    op = global_op(tods.engine(b.maps[0]))
    x = x0.copy()
    st = DevicePCG(op, b.maps[0].map, x.maps[0].map, _precon_arg(precon),
                   graph=graph and not parallel.have_mpi())
    st.start()
    bnorm = math.sqrt(b.dot(b)) if tol is not None else None
    nsamp = tods.get_nsamp()
    torch.cuda.synchronize()
    tloop = time.time()
    i = -1
    for i in range(maxiter):
        st.step()
        need_check = tol is not None and ((i + 1) % check_every == 0 or i == maxiter - 1)
        if i in save_iters:
            x.maps[save_ind].write(outroot + "_" + str(i) + save_tail)
        if need_check or history is not None:
            s = st.scalars()
            if s[MK_S_FLAG]:
                raise FloatingPointError(f"PCG breakdown at iteration {i} (p.Ap <= 0 or non-finite)")
            rec = math.sqrt(max(s[MK_S_RR], 0.0)) / bnorm if bnorm else float("nan")
            if history is not None:
                history.append({"iter": i, "zr": float(s[MK_S_ZR]), "rel_rr": rec})
            if need_check and rec <= tol:
                tr = _true_residual(op, b.maps[0].map, x.maps[0].map)
                if history is not None:
                    history[-1]["true_rel_residual"] = tr
                if tr <= tol:
                    break
    torch.cuda.synchronize()
    niter = i + 1
    tave = (time.time() - tloop) / max(niter, 1)
    if verbose:
        print("average time per iteration was ", tave, " with effective throughput ",
              nsamp / tave / 1e6, " Msamp/s")
        sys.stdout.flush()
    x.niter = niter
    x.setup_s = tloop - t0
    return x


def run_pcg(b: Mapset, x0: Mapset, tods: TodVec, precon=None, mask: Optional[Mapset] = None,
            maxiter: int = 25, outroot: str = "map", save_iters: List[int] = [-1],
            save_ind: int = 0, save_tail: str = ".fits", plot_iters: List[int] = [],
            plot_info=None, plot_ind: int = 0, **kw) -> Mapset:
    """run_pcg_wprior without a prior (pcg.py:203-238)."""
    return run_pcg_wprior(b, x0, tods, None, precon, mask, maxiter, outroot, save_iters, save_ind,
                          save_tail, plot_iters, plot_info, plot_ind, **kw)


def _run_pcg_generic(b, x0, tods, prior, precon, mask, maxiter, outroot, save_iters, save_ind,
                     save_tail, verbose, history):
    """The reference recurrence on Mapset algebra (still GPU kernels): for
    priors, masks and multi-map Mapsets."""
    Ax = tods.dot(x0, mask=mask)
    r = b.copy()
    r.axpy(Ax, -1)
    z = precon * r if precon is not None else r.copy()
    p = z.copy()
    zr = r.dot(z)
    x = x0.copy()
    for i in range(maxiter):
        Ap = tods.dot(p, mask=mask)
        if prior is not None:
            prior.apply_prior(p, Ap)
        pAp = p.dot(Ap)
        alpha = zr / pAp
        x_new = x.copy()
        x_new.axpy(p, alpha)
        r_new = r.copy()
        r_new.axpy(Ap, -alpha)
        z_new = precon * r_new if precon is not None else r_new.copy()
        zr_new = r_new.dot(z_new)
        beta = zr_new / zr
        p_new = z_new.copy()
        p_new.axpy(p, beta)
        p, z, r, zr, x = p_new, z_new, r_new, zr_new, x_new
        if history is not None:
            history.append({"iter": i, "zr": zr, "alpha": alpha, "beta": beta})
        if i in save_iters:
            x.maps[save_ind].write(outroot + "_" + str(i) + save_tail)
    x.niter = maxiter
    return x


class MixedOp:
    """A in FP32 seen from FP64 vectors: p64 -> p32 -> A32 p32 -> Ap64."""

    def __init__(self, op32, n: int, device):
        self.op32 = op32
        self.p32 = torch.empty(n, dtype=torch.float32, device=device)
        self.a32 = torch.empty(n, dtype=torch.float32, device=device)

    def apply(self, x: torch.Tensor, out: torch.Tensor, accumulate: bool = False):
        self.p32.copy_(x.reshape(-1))
        self.op32.apply(self.p32, self.a32)
        if accumulate:
            out.reshape(-1).add_(self.a32)
        else:
            out.reshape(-1).copy_(self.a32)
        return out


def run_pcg_mixed(b: Mapset, x0: Mapset, tods: TodVec, precon=None, tol: float = 1e-6,
                  max_iter: int = 5000, replace_every: int = 200, graph: bool = True,
                  verbose: bool = False, history: Optional[list] = None,
                  inner_precon=None, on_outer=None, mode: str = "reliable",
                  inner_iters: int = 20, max_outer: int = 500,
                  restart_drift: float = 1.2) -> Mapset:
    """Mixed-precision PCG to an FP64 true residual ||b - A x||/||b|| <= tol.

    mode="reliable" (default): PCG whose vectors, dot products and scalars are
    FP64 but whose operator applications run in FP32 (FP32 projections, FP32
    DCT/filter, 3xTF32 tensor-core rotations); every ``replace_every``
    iterations, and whenever the recursive residual claims convergence, the
    residual is replaced by the FP64 true residual b - A64 x (an FP64
    operator application, as costly as 10-25 FP32 iterations on GB300; the
    recursive residual tracks the true one to ~6 digits over 200 iterations
    on the benchmark maps, hence the default).  Those replacements are the iterative-refinement
    steps: the FP64 residual corrects the drift of the FP32 operator while the
    Krylov space is kept.  When a replacement finds the recursive residual
    off from the true one by more than ``restart_drift`` (either way), the
    search direction restarts from z = M r: continuing with the old one
    after a large correction can diverge.

    mode="refine": classic iterative refinement -- each outer step solves
    A32 e = r64 with ``inner_iters`` FP32 PCG iterations from zero and updates
    x += e in FP64.  Restarting the Krylov space every ``inner_iters`` makes
    it stall on ill-conditioned maps; kept for comparison.

    ``inner_precon``/``precon`` may be a Mapset (diagonal) or any object with
    apply(r, z) (e.g. LearnedPrecon).  ``on_outer(k, x, rel)`` is called at
    every FP64 residual evaluation."""
    if mode == "refine":
        return _run_refine(b, x0, tods, precon, tol, inner_iters, max_outer, graph, verbose,
                           history, inner_precon, on_outer)
    m64 = b.maps[0]
    op64 = global_op(tods.engine(m64, torch.float64))
    op32 = global_op(tods.engine(m64, torch.float32))
    graph = graph and not parallel.have_mpi()
    x = x0.copy()
    xf = x.maps[0].map.reshape(-1)
    bf = m64.map.reshape(-1)
    red = _reducer(bf.device)
    bnorm = math.sqrt(red.dot(bf, bf).item())
    M = inner_precon if inner_precon is not None else _precon_arg(precon)
    st = DevicePCG(MixedOp(op32, bf.numel(), bf.device), bf, xf, M, graph=graph)
    ax = torch.empty_like(bf)
    ptmp = torch.empty_like(bf)

    def replace() -> float:
        # r = b - A64 x; z = M r; zr = r.z  (p kept; the caller restarts it
        # when the recursive residual had drifted)
        op64.apply(xf, ax)
        K.pcg_init(st.r, st.z, ptmp, bf, ax, st.M, st.s, st.red)
        if st.Mop is not None:
            st.Mop.apply(st.r, st.z)
            st.red.dot(st.r, st.z, out=st.s[MK_S_ZR])
        return math.sqrt(max(float(st.s[MK_S_RR]), 0.0)) / bnorm

    st.start()
    rel = math.sqrt(max(float(st.s[MK_S_RR]), 0.0)) / bnorm
    k = 0
    outer = 0
    restarts = 0
    since = 0
    while k < max_iter:
        st.step()
        k += 1
        since += 1
        check = since >= replace_every or k % 5 == 0
        if not check:
            continue
        s = st.scalars()
        if s[MK_S_FLAG]:
            raise FloatingPointError(f"mixed PCG breakdown at iteration {k}")
        rec = math.sqrt(max(s[MK_S_RR], 0.0)) / bnorm
        if since >= replace_every or rec <= tol:
            rel = replace()
            outer += 1
            since = 0
            # the recursive residual had drifted from the true one (the FP32
            # operator's rounding): the kept search direction no longer fits
            # the replaced residual, so restart it (p = z)
            restart = rel > restart_drift * rec or rec > restart_drift * rel
            if restart:
                st.p.copy_(st.z)
                restarts += 1
            if history is not None:
                history.append({"iter": k, "recursive_rel": rec, "true_rel_residual": rel,
                                "restart": restart})
            if verbose:
                print(f"iter {k}: true FP64 residual {rel:.3e} (recursive {rec:.3e})")
            if on_outer is not None:
                on_outer(outer, xf, rel)
            if rel <= tol:
                break
    x.niter = k
    x.outer = outer
    x.restarts = restarts
    x.rel_residual = rel
    return x


def _run_refine(b, x0, tods, precon, tol, inner_iters, max_outer, graph, verbose, history,
                inner_precon, on_outer) -> Mapset:
    m64 = b.maps[0]
    op64 = global_op(tods.engine(m64, torch.float64))
    op32 = global_op(tods.engine(m64, torch.float32))
    graph = graph and not parallel.have_mpi()
    x = x0.copy()
    xf = x.maps[0].map.reshape(-1)
    bf = m64.map.reshape(-1)
    red = _reducer(bf.device)
    bnorm = math.sqrt(red.dot(bf, bf).item())
    if inner_precon is not None:
        M32 = inner_precon
    elif precon is not None and hasattr(precon, "apply"):
        M32 = precon
    else:
        M32 = precon.maps[0].map.reshape(-1).float().contiguous() if precon is not None else None
    r32 = torch.empty(bf.numel(), dtype=torch.float32, device=bf.device)
    e32 = torch.zeros_like(r32)
    zero32 = torch.zeros_like(r32)
    inner = DevicePCG(op32, r32, e32, M32, graph=graph)
    ax = torch.empty_like(bf)
    total_inner = 0
    rel = float("inf")
    for outer in range(max_outer):
        op64.apply(xf, ax)
        r64 = bf - ax
        rel = math.sqrt(red.dot(r64, r64).item()) / bnorm
        if history is not None:
            history.append({"outer": outer, "inner_total": total_inner, "true_rel_residual": rel})
        if verbose:
            print(f"outer {outer}: true FP64 residual {rel:.3e} after {total_inner} inner iterations")
        if on_outer is not None:
            on_outer(outer, xf, rel)
        if rel <= tol:
            break
        r32.copy_(r64)
        e32.zero_()
        inner.start(zero32)
        for _ in range(inner_iters):
            inner.step()
        total_inner += inner_iters
        xf.add_(e32.to(torch.float64))
    x.niter = total_inner
    x.outer = outer
    x.rel_residual = rel
    return x
