"""GPU: the learned preconditioner's CUDA convolutions and training gradient
against the float64 CPU oracle, and the preconditioner's SPD property."""
import numpy as np
import pytest
import torch

import learned_oracle as lo

pytestmark = pytest.mark.gpu
cuda = torch.device("cuda", 0)


@pytest.fixture(scope="module")
def L():
    from minkasi_gb300 import learned
    return learned


def t(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(cuda)


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


# the last two are large enough (>= 4 x 152 tiles of 32 x 32 over the batch of
# 2) for the large-map tiling; the others use the small-map one
@pytest.mark.parametrize("cin,cout,H,W", [(1, 16, 33, 20), (16, 16, 16, 16), (16, 1, 40, 47), (5, 7, 3, 2),
                                         (16, 16, 70, 95), (16, 1, 65, 33), (7, 16, 521, 611),
                                         (16, 1, 530, 600)])
def test_conv_kernels_match_oracle(L, cin, cout, H, W):
    rng = np.random.default_rng(cin * 100 + cout)
    x = rng.standard_normal((2, cin, H, W))
    w = rng.standard_normal((cout, cin, 3, 3))
    y = rng.standard_normal((2, cout, H, W))
    assert rel(L.conv_fwd(t(x), t(w)).cpu().numpy(), lo.conv_fwd(x, w)) < 1e-5
    assert rel(L.conv_adj(t(y), t(w)).cpu().numpy(), lo.conv_adj(y, w)) < 1e-5
    assert rel(L.conv_wgrad(t(x), t(y)).cpu().numpy(), lo.conv_wgrad(x, y)) < 1e-5


def test_training_gradient_matches_oracle(L):
    rng = np.random.default_rng(7)
    shape = (24, 20)
    n = shape[0] * shape[1]
    ws = [rng.standard_normal((co, ci, 3, 3)) * 0.2
          for ci, co in zip(L.CHANNELS[:-1], L.CHANNELS[1:])]
    hits = rng.integers(0, 6, size=n).astype(float)
    mask = (hits > 0).astype(float)
    dsq = np.where(hits > 0, 1 / np.sqrt(np.maximum(hits, 1)), 0)
    R = rng.standard_normal((4, n))
    E = rng.standard_normal((4, n))
    Lref, gref = lo.loss_grad(ws, dsq, mask, R, E, shape)
    net = L.ConvNet([t(w) for w in ws])
    loss, grads = L.loss_and_grad(net, t(dsq), t(mask), t(R), t(E), shape)
    assert abs(loss - Lref) < 1e-4 * abs(Lref)
    for g, gr in zip(grads, gref):
        assert rel(g.cpu().numpy(), gr) < 1e-3


def test_learned_precon_is_spd_and_reduces_to_jacobi(L):
    rng = np.random.default_rng(3)
    shape = (32, 32)
    hits = torch.from_numpy(rng.integers(0, 4, size=shape[0] * shape[1]).astype(np.float64)).to(cuda)
    net = L.ConvNet.init(seed=1, scale=0.5, device=cuda)
    M = L.LearnedPrecon(hits, net, shape)
    a = torch.randn(shape[0] * shape[1], dtype=torch.float64, device=cuda)
    b = torch.randn_like(a)
    Ma, Mb = torch.empty_like(a), torch.empty_like(b)
    M.apply(a, Ma)
    M.apply(b, Mb)
    assert abs(float(b @ Ma) - float(a @ Mb)) < 1e-5 * float(a.abs().sum())
    assert float(a @ Ma) > 0
    zero = L.ConvNet([torch.zeros_like(w) for w in net.weights])
    Z = L.LearnedPrecon(hits, zero, shape)
    out = torch.empty_like(a)
    Z.apply(a, out)
    jac = torch.where(hits > 0, a / hits.clamp(min=1), torch.zeros_like(a))
    assert torch.allclose(out, jac, rtol=1e-6, atol=1e-12)
