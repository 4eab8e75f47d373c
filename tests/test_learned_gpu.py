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


# (400, 780) with a batch of 2 gives 650 tiles of 32 x 32, so the
# convolutions take the large-map tiling
@pytest.mark.parametrize("shape,B", [((24, 20), 4), ((400, 780), 2)])
def test_training_gradient_matches_oracle(L, shape, B):
    rng = np.random.default_rng(7)
    n = shape[0] * shape[1]
    ws = [rng.standard_normal((co, ci, 3, 3)) * 0.2
          for ci, co in zip(L.CHANNELS[:-1], L.CHANNELS[1:])]
    hits = rng.integers(0, 6, size=n).astype(float)
    mask = (hits > 0).astype(float)
    dsq = np.where(hits > 0, 1 / np.sqrt(np.maximum(hits, 1)), 0)
    R = rng.standard_normal((B, n))
    E = rng.standard_normal((B, n))
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


@pytest.mark.parametrize("shape", [(37, 53), (700, 900)])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_fused_precon_apply(L, shape, dtype):
    """mk_learned_precon_apply (first and last layers fused with the D^-1/2
    scalings) against the same operator built from the separate convolution
    calls (bit-exact), and against the float64 oracle on the small map.
    (700, 900) is large enough for the 32 x 32 tiling."""
    rng = np.random.default_rng(shape[0])
    n = shape[0] * shape[1]
    hits_np = rng.integers(0, 5, size=n).astype(np.float64)
    hits = torch.from_numpy(hits_np).to(cuda)
    net = L.ConvNet.init(seed=2, scale=0.3, device=cuda)
    M = L.LearnedPrecon(hits, net, shape, stencil=False)
    r = torch.from_numpy(rng.standard_normal(n)).to(cuda, dtype)
    z = torch.empty_like(r)
    M.apply(r, z)
    dsq = (M.dsq64 if dtype == torch.float64 else M.dsq32)
    u = dsq * r
    acts = u.float().view(1, 1, *shape)
    for w in net.weights:
        acts = L.conv_fwd(acts, w)
    for w in reversed(net.weights):
        acts = L.conv_adj(acts, w)
    want = dsq * (u + acts.reshape(-1).to(dtype))
    assert torch.equal(z, want)
    if shape[0] < 100:
        d = M.dsq64.cpu().numpy()
        u64 = d * r.double().cpu().numpy()
        a = u64.reshape(1, 1, *shape)
        ws = [w.double().cpu().numpy() for w in net.weights]
        for w in ws:
            a = lo.conv_fwd(a, w)
        for w in reversed(ws):
            a = lo.conv_adj(a, w)
        ref = d * (u64 + a.reshape(-1))
        assert rel(z.double().cpu().numpy(), ref) < 1e-5
    # z may alias r
    r2 = r.clone()
    M.apply(r2, r2)
    assert torch.equal(r2, z)


@pytest.mark.parametrize("shape", [(40, 36), (300, 517)])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_stencil_apply_equals_layered_inside_the_edge(L, shape, dtype):
    """K^T K as one 17 x 17 stencil (its impulse response) against the 8
    layered convolutions and the float64 oracle, with the hit pixels (and so
    u) at least 8 pixels from the map edge, where the two forms are the same
    operator; and the stencil form is symmetric positive definite."""
    rng = np.random.default_rng(shape[1])
    n = shape[0] * shape[1]
    hits_np = rng.integers(0, 5, size=shape).astype(np.float64)
    hits_np[:8], hits_np[-8:], hits_np[:, :8], hits_np[:, -8:] = 0, 0, 0, 0
    hits = torch.from_numpy(hits_np.ravel()).to(cuda)
    net = L.ConvNet.init(seed=4, scale=0.4, device=cuda)
    S = L.LearnedPrecon(hits, net, shape)
    assert S.stencil and tuple(S.kern.shape) == (17, 17)
    Lay = L.LearnedPrecon(hits, net, shape, stencil=False)
    r = torch.from_numpy(rng.standard_normal(n)).to(cuda, dtype)
    zs, zl = torch.empty_like(r), torch.empty_like(r)
    S.apply(r, zs)
    Lay.apply(r, zl)
    assert rel(zs.double().cpu().numpy(), zl.double().cpu().numpy()) < 1e-5
    d = S.dsq64.cpu().numpy()
    u64 = d * r.double().cpu().numpy()
    a = u64.reshape(1, 1, *shape)
    ws = [w.double().cpu().numpy() for w in net.weights]
    for w in ws:
        a = lo.conv_fwd(a, w)
    for w in reversed(ws):
        a = lo.conv_adj(a, w)
    ref = d * (u64 + a.reshape(-1))
    assert rel(zs.double().cpu().numpy(), ref) < 1e-5
    b = torch.from_numpy(rng.standard_normal(n)).to(cuda, torch.float64)
    a64 = r.double()
    Ma, Mb = torch.empty_like(a64), torch.empty_like(b)
    S.apply(a64, Ma)
    S.apply(b, Mb)
    assert abs(float(b @ Ma) - float(a64 @ Mb)) < 1e-5 * float((a64.abs() * b.abs()).sum())
    assert float(a64 @ Ma) > 0
    with pytest.raises(ValueError):
        S.apply(a64, a64)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_pooled_stencil_apply(L, dtype):
    """The multi-scale form z = D^-1/2 (u + P^T C * P u) with P the 8 x 8
    block mean: against the same operator built from pool_maps, the layered
    K^T K on the coarse grid and unpool_maps (hit pixels 64 fine pixels from
    the edge, so 8 coarse pixels: the layered and stencil forms agree), and
    symmetric positive definite."""
    rng = np.random.default_rng(11)
    shape, b = (256, 200), 8
    n = shape[0] * shape[1]
    hits_np = rng.integers(0, 5, size=shape).astype(np.float64)
    hits_np[:64], hits_np[-64:], hits_np[:, :64], hits_np[:, -64:] = 0, 0, 0, 0
    hits = torch.from_numpy(hits_np.ravel()).to(cuda)
    net = L.ConvNet.init(seed=5, scale=0.4, device=cuda, pool=b)
    S = L.LearnedPrecon(hits, net, shape)
    r = torch.from_numpy(rng.standard_normal(n)).to(cuda, dtype)
    z = torch.empty_like(r)
    S.apply(r, z)
    dsq = S.dsq64 if dtype == torch.float64 else S.dsq32
    u = dsq * r
    uc = L.pool_maps(u.float().view(1, 1, *shape), b).contiguous()
    want = dsq * (u + L.unpool_maps(net.ktk(uc), b, *shape).reshape(-1).to(dtype))
    assert rel(z.double().cpu().numpy(), want.double().cpu().numpy()) < 1e-5
    a64, b64 = r.double(), torch.from_numpy(rng.standard_normal(n)).to(cuda)
    Ma, Mb = torch.empty_like(a64), torch.empty_like(b64)
    S.apply(a64, Ma)
    S.apply(b64, Mb)
    assert abs(float(b64 @ Ma) - float(a64 @ Mb)) < 1e-5 * float((a64.abs() * b64.abs()).sum())
    assert float(a64 @ Ma) > 0
    with pytest.raises(ValueError):
        L.LearnedPrecon(hits, net, shape, stencil=False)


def test_pooled_training_gradient_directional(L):
    """The pooled loss gradient (P applied to the incoming gradient, then the
    network's own backward kernels, FP32) against a central finite
    difference, in float64, of the oracle's pooled loss along a random
    direction of the weights."""
    rng = np.random.default_rng(12)
    shape, b, B = (48, 40), 4, 3
    n = shape[0] * shape[1]
    hits = rng.integers(0, 6, size=n).astype(np.float64)
    mask = (hits > 0).astype(np.float64)
    dsq = np.where(hits > 0, 1 / np.sqrt(np.maximum(hits, 1)), 0.0)
    R = rng.standard_normal((B, n))
    E = rng.standard_normal((B, n))
    ws = [rng.standard_normal((co, ci, 3, 3)) * 0.2 for ci, co in zip(L.CHANNELS[:-1], L.CHANNELS[1:])]
    dirs = [rng.standard_normal(w.shape) * 0.2 for w in ws]
    net = L.ConvNet([t(w) for w in ws], pool=b)
    loss, grads = L.loss_and_grad(net, t(dsq), t(mask), t(R), t(E), shape)
    ana = float(sum((g.cpu().double().numpy() * d).sum() for g, d in zip(grads, dirs)))
    h = 1e-6
    lp = lo.pooled_loss([w + h * d for w, d in zip(ws, dirs)], dsq, mask, R, E, shape, b)
    lm = lo.pooled_loss([w - h * d for w, d in zip(ws, dirs)], dsq, mask, R, E, shape, b)
    num = (lp - lm) / (2 * h)
    assert abs(loss - lo.pooled_loss(ws, dsq, mask, R, E, shape, b)) < 1e-4 * abs(loss)
    assert abs(num - ana) < 1e-2 * abs(num), (num, ana)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_multilevel_apply_is_the_sum_of_levels(L, dtype):
    """Two levels (fine and 8 x 8 pooled): z = D^-1/2 (u + C1 * u + P^T C8 * P u),
    the sum of the single-level operators minus one identity term, and
    symmetric positive definite."""
    rng = np.random.default_rng(13)
    shape = (192, 160)
    n = shape[0] * shape[1]
    hits_np = rng.integers(0, 5, size=shape).astype(np.float64)
    hits_np[:64], hits_np[-64:], hits_np[:, :64], hits_np[:, -64:] = 0, 0, 0, 0
    hits = torch.from_numpy(hits_np.ravel()).to(cuda)
    n1 = L.ConvNet.init(seed=6, scale=0.4, device=cuda, pool=1)
    n8 = L.ConvNet.init(seed=7, scale=0.4, device=cuda, pool=8)
    M = L.LearnedPrecon(hits, [n1, n8], shape)
    assert M.pools == [1, 8]
    r = torch.from_numpy(rng.standard_normal(n)).to(cuda, dtype)
    z, z1, z8 = torch.empty_like(r), torch.empty_like(r), torch.empty_like(r)
    M.apply(r, z)
    L.LearnedPrecon(hits, n1, shape).apply(r, z1)
    L.LearnedPrecon(hits, n8, shape).apply(r, z8)
    dsq = M.dsq64 if dtype == torch.float64 else M.dsq32
    want = z1 + z8 - dsq * dsq * r
    assert rel(z.double().cpu().numpy(), want.double().cpu().numpy()) < 1e-5
    a64, b64 = r.double(), torch.from_numpy(rng.standard_normal(n)).to(cuda)
    Ma, Mb = torch.empty_like(a64), torch.empty_like(b64)
    M.apply(a64, Ma)
    M.apply(b64, Mb)
    assert abs(float(b64 @ Ma) - float(a64 @ Mb)) < 1e-5 * float((a64.abs() * b64.abs()).sum())
    assert float(a64 @ Ma) > 0


def test_multilevel_training_gradient_directional(L, tmp_path):
    """The two-level loss gradient (one list of gradients per level) against
    a central finite difference, in float64, of the oracle's multi-level loss
    along a random direction of all weights; save and load keep the levels."""
    rng = np.random.default_rng(14)
    shape, B = (48, 40), 3
    n = shape[0] * shape[1]
    hits = rng.integers(0, 6, size=n).astype(np.float64)
    mask = (hits > 0).astype(np.float64)
    dsq = np.where(hits > 0, 1 / np.sqrt(np.maximum(hits, 1)), 0.0)
    R = rng.standard_normal((B, n))
    E = rng.standard_normal((B, n))
    pools = (1, 4)
    wss = [[rng.standard_normal((co, ci, 3, 3)) * 0.2 for ci, co in zip(L.CHANNELS[:-1], L.CHANNELS[1:])]
           for _ in pools]
    dirs = [[rng.standard_normal(w.shape) * 0.2 for w in ws] for ws in wss]
    nets = [L.ConvNet([t(w) for w in ws], pool=b) for ws, b in zip(wss, pools)]
    loss, grads = L.loss_and_grad(nets, t(dsq), t(mask), t(R), t(E), shape)
    assert len(grads) == 2
    ana = float(sum((g.cpu().double().numpy() * d).sum()
                    for gl, dl in zip(grads, dirs) for g, d in zip(gl, dl)))
    h = 1e-6

    def shifted(sign):
        return [([w + sign * h * d for w, d in zip(ws, dl)], b) for ws, dl, b in zip(wss, dirs, pools)]

    num = (lo.multilevel_loss(shifted(1), dsq, mask, R, E, shape) -
           lo.multilevel_loss(shifted(-1), dsq, mask, R, E, shape)) / (2 * h)
    assert abs(loss - lo.multilevel_loss(list(zip(wss, pools)), dsq, mask, R, E, shape)) < 1e-4 * abs(loss)
    assert abs(num - ana) < 1e-2 * abs(num), (num, ana)
    path = str(tmp_path / "ml.npz")
    L.save(nets, path)
    back = L.load(path, cuda)
    assert [b.pool for b in back] == list(pools)
    assert all(torch.equal(x, y) for a, b in zip(nets, back) for x, y in zip(a.weights, b.weights))
