"""The FP64 student oracle's analytic gradients against central finite
differences (CPU), so that the oracle can check the GPU training kernels."""
import numpy as np

from oracle import distill_oracle as D


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    c_in, W, n3x3, H = 3, 4, 1, 3
    n = D.param_count(c_in, W, n3x3, H)
    p = rng.normal(0, 0.5, n)
    planes = (rng.random((2, c_in, 361)) < 0.3).astype(np.uint8)
    t = rng.random((2, 361))
    t /= t.sum(1, keepdims=True)
    vt = np.array([0.3, -0.6])
    (kl, lv), g = D.loss_and_grads(p, planes, t, vt, 0.7, c_in, W, n3x3, H)
    assert g.shape == (n,)
    idx = rng.choice(n, 60, replace=False)
    eps = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        (a1, b1), _ = D.loss_and_grads(pp, planes, t, vt, 0.7, c_in, W, n3x3, H)
        (a2, b2), _ = D.loss_and_grads(pm, planes, t, vt, 0.7, c_in, W, n3x3, H)
        fd = ((a1 + 0.7 * b1) - (a2 + 0.7 * b2)) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])


def test_im2col_col2im_are_adjoint():
    rng = np.random.default_rng(1)
    x = rng.normal(size=(2, 3, 19, 19))
    y = rng.normal(size=(2, 27, 361))
    lhs = (D.im2col(x, 3) * y).sum()
    rhs = (x * D.col2im(y, 3, 3)).sum()
    assert abs(lhs - rhs) < 1e-9 * abs(lhs)
