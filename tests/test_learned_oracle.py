"""CPU: the learned-preconditioner oracle is self-consistent -- the adjoint
convolution is the transpose of the forward one, and the analytic loss
gradient matches central finite differences."""
import numpy as np

import learned_oracle as lo


def _net(rng, chans=(1, 3, 2)):
    return [rng.standard_normal((co, ci, 3, 3)) * 0.3 for ci, co in zip(chans[:-1], chans[1:])]


def test_adjoint_is_transpose():
    rng = np.random.default_rng(0)
    w = rng.standard_normal((3, 2, 3, 3))
    x = rng.standard_normal((2, 2, 7, 9))
    y = rng.standard_normal((2, 3, 7, 9))
    assert abs(np.sum(lo.conv_fwd(x, w) * y) - np.sum(x * lo.conv_adj(y, w))) < 1e-10


def test_wgrad_is_gradient_of_inner_product():
    rng = np.random.default_rng(1)
    w = rng.standard_normal((3, 2, 3, 3))
    x = rng.standard_normal((2, 2, 6, 5))
    h = rng.standard_normal((2, 3, 6, 5))
    g = lo.conv_wgrad(x, h)
    eps = 1e-6
    for idx in [(0, 0, 0, 0), (2, 1, 1, 2), (1, 0, 2, 1)]:
        wp, wm = w.copy(), w.copy()
        wp[idx] += eps
        wm[idx] -= eps
        fd = (np.sum(lo.conv_fwd(x, wp) * h) - np.sum(lo.conv_fwd(x, wm) * h)) / (2 * eps)
        assert abs(fd - g[idx]) < 1e-6 * max(1, abs(fd))


def test_loss_gradient_matches_finite_differences():
    rng = np.random.default_rng(2)
    shape = (6, 7)
    n = shape[0] * shape[1]
    ws = _net(rng)
    hits = rng.integers(0, 5, size=n).astype(float)
    mask = (hits > 0).astype(float)
    dsq = np.where(hits > 0, 1 / np.sqrt(np.maximum(hits, 1)), 0)
    R = rng.standard_normal((3, n))
    E = rng.standard_normal((3, n))
    L, grads = lo.loss_grad(ws, dsq, mask, R, E, shape)
    assert abs(L - lo.loss(ws, dsq, mask, R, E, shape)) < 1e-12
    eps = 1e-6
    for li, w in enumerate(ws):
        for idx in [(0, 0, 1, 1), (w.shape[0] - 1, w.shape[1] - 1, 2, 0)]:
            wp = [x.copy() for x in ws]
            wm = [x.copy() for x in ws]
            wp[li][idx] += eps
            wm[li][idx] -= eps
            fd = (lo.loss(wp, dsq, mask, R, E, shape) - lo.loss(wm, dsq, mask, R, E, shape)) / (2 * eps)
            assert abs(fd - grads[li][idx]) < 1e-5 * max(1e-3, abs(fd)), (li, idx, fd, grads[li][idx])
