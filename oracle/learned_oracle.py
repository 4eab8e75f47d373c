"""CPU oracle for the learned preconditioner's convolutions and training
gradient.  TEST INFRASTRUCTURE ONLY (imported by tests/ as the checker).

The reference has no learned preconditioner; this restates, in float64 numpy,
the math the CUDA kernels implement (libmkgpu mk_conv3x3_*):
  fwd  : y[b,co,p] = sum_{ci,d} w[co,ci,d] x[b,ci,p+d]
  adj  : x[b,ci,q] = sum_{co,d} w[co,ci,d] y[b,co,q-d]
  wgrad: g[co,ci,d] = sum_{b,p} h[b,co,p] x[b,ci,p+d]
(zero padding), and the loss of minkasi_gb300.learned.loss_and_grad:
  L = mean_b ||P(M r_b - e_b)||^2 / ||P e_b||^2,  M r = dsq (u + K^T K u), u = dsq r,
with P removing the mean over hit pixels.  ``loss_grad`` is analytic and is
itself pinned by finite differences in tests/test_learned_oracle.py.
"""
from __future__ import annotations

from typing import List, Sequence, Tuple

import numpy as np


def _pad(x):
    return np.pad(x, ((0, 0), (0, 0), (1, 1), (1, 1)))


def conv_fwd(x: np.ndarray, w: np.ndarray) -> np.ndarray:
    B, Cin, H, W = x.shape
    xp = _pad(x)
    y = np.zeros((B, w.shape[0], H, W))
    for dy in range(3):
        for dx in range(3):
            y += np.einsum("oc,bchw->bohw", w[:, :, dy, dx], xp[:, :, dy:dy + H, dx:dx + W])
    return y


def conv_adj(y: np.ndarray, w: np.ndarray) -> np.ndarray:
    B, Cout, H, W = y.shape
    yp = _pad(y)
    x = np.zeros((B, w.shape[1], H, W))
    for dy in range(3):
        for dx in range(3):
            x += np.einsum("oc,bohw->bchw", w[:, :, dy, dx],
                           yp[:, :, 2 - dy:2 - dy + H, 2 - dx:2 - dx + W])
    return x


def conv_wgrad(x: np.ndarray, h: np.ndarray) -> np.ndarray:
    B, Cin, H, W = x.shape
    xp = _pad(x)
    g = np.zeros((h.shape[1], Cin, 3, 3))
    for dy in range(3):
        for dx in range(3):
            g[:, :, dy, dx] = np.einsum("bohw,bchw->oc", h, xp[:, :, dy:dy + H, dx:dx + W])
    return g


def ktk(ws: Sequence[np.ndarray], u: np.ndarray) -> np.ndarray:
    a = u
    for w in ws:
        a = conv_fwd(a, w)
    for w in reversed(ws):
        a = conv_adj(a, w)
    return a


def _proj(v, mask):
    mean = (v * mask).sum(axis=1, keepdims=True) / mask.sum()
    return (v - mean) * mask


def loss(ws, dsq, mask, R, E, shape) -> float:
    """mean_b min_c ||c P(M r_b) - P e_b||^2 / ||P e_b||^2."""
    B = R.shape[0]
    u = R * dsq[None, :]
    z = ktk(ws, u.reshape(B, 1, *shape)).reshape(B, -1)
    mr = dsq[None, :] * (u + z)
    pe = _proj(E, mask)
    a = _proj(mr, mask)
    c = (a * pe).sum(axis=1) / (a * a).sum(axis=1)
    res = c[:, None] * a - pe
    return float(((res ** 2).sum(axis=1) / (pe ** 2).sum(axis=1)).mean())


def pool(x: np.ndarray, b: int) -> np.ndarray:
    """b x b block mean of [B, C, H, W] maps, pixels outside the map as 0."""
    B, C, H, W = x.shape
    Hc, Wc = -(-H // b), -(-W // b)
    xp = np.zeros((B, C, Hc * b, Wc * b))
    xp[:, :, :H, :W] = x
    return xp.reshape(B, C, Hc, b, Wc, b).sum(axis=(3, 5)) / (b * b)


def unpool(y: np.ndarray, b: int, H: int, W: int) -> np.ndarray:
    """The transpose of pool: each fine pixel gets its block's value / b^2."""
    up = np.repeat(np.repeat(y, b, axis=2), b, axis=3) / (b * b)
    return up[:, :, :H, :W]


def pooled_loss(ws, dsq, mask, R, E, shape, b: int) -> float:
    """The loss of the multi-scale form M r = dsq (u + P^T K^T K P u)."""
    B = R.shape[0]
    u = R * dsq[None, :]
    z = unpool(ktk(ws, pool(u.reshape(B, 1, *shape), b)), b, *shape).reshape(B, -1)
    mr = dsq[None, :] * (u + z)
    pe = _proj(E, mask)
    a = _proj(mr, mask)
    c = (a * pe).sum(axis=1) / (a * a).sum(axis=1)
    res = c[:, None] * a - pe
    return float(((res ** 2).sum(axis=1) / (pe ** 2).sum(axis=1)).mean())


def multilevel_loss(levels, dsq, mask, R, E, shape) -> float:
    """The loss of M r = dsq (u + sum_l P_l^T K_l^T K_l P_l u), levels a list
    of (weights, block size)."""
    B = R.shape[0]
    u = R * dsq[None, :]
    z = np.zeros_like(u)
    for ws, b in levels:
        z += unpool(ktk(ws, pool(u.reshape(B, 1, *shape), b)), b, *shape).reshape(B, -1)
    mr = dsq[None, :] * (u + z)
    pe = _proj(E, mask)
    a = _proj(mr, mask)
    c = (a * pe).sum(axis=1) / (a * a).sum(axis=1)
    res = c[:, None] * a - pe
    return float(((res ** 2).sum(axis=1) / (pe ** 2).sum(axis=1)).mean())


def loss_grad(ws, dsq, mask, R, E, shape) -> Tuple[float, List[np.ndarray]]:
    """Loss and its gradient w.r.t. every weight (backprop through K^T K)."""
    B = R.shape[0]
    n = len(ws)
    u = (R * dsq[None, :]).reshape(B, 1, *shape)
    acts = [u]
    for w in ws:
        acts.append(conv_fwd(acts[-1], w))
    bs = [acts[-1]]
    for w in reversed(ws):
        bs.append(conv_adj(bs[-1], w))
    z = bs[-1].reshape(B, -1)
    mr = dsq[None, :] * (u.reshape(B, -1) + z)
    pe = _proj(E, mask)
    a = _proj(mr, mask)
    den = (pe ** 2).sum(axis=1)
    c = (a * pe).sum(axis=1) / (a * a).sum(axis=1)
    res = c[:, None] * a - pe
    L = float(((res ** 2).sum(axis=1) / den).mean())
    # envelope theorem: at the optimal c the gradient is the partial at fixed c
    gmr = 2.0 * c[:, None] * _proj(res, mask) / den[:, None] / B
    g = (dsq[None, :] * gmr).reshape(B, 1, *shape)
    grads = [np.zeros_like(w) for w in ws]
    for l in range(1, n + 1):
        grads[l - 1] += conv_wgrad(g, bs[n - l])
        g = conv_fwd(g, ws[l - 1])
    h = g
    for l in range(n, 0, -1):
        grads[l - 1] += conv_wgrad(acts[l - 1], h)
        h = conv_adj(h, ws[l - 1])
    return L, grads
