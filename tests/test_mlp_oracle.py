"""The MLP's CPU oracle (oracle/mlp_oracle.py) against finite differences,
so that it can in turn check the GPU kernels' gradients."""
import numpy as np

from oracle import mlp_oracle


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    dims = [5, 7, 6, 1]
    n = sum(o * (i + 1) for i, o in zip(dims[:-1], dims[1:]))
    w = rng.standard_normal(n) * 0.5
    x = rng.standard_normal((11, 5))
    y = rng.standard_normal(11)
    loss, g = mlp_oracle.loss_grad(w, dims, x, y)
    eps = 1e-6
    for k in rng.choice(n, 25, replace=False):
        wp, wm = w.copy(), w.copy()
        wp[k] += eps
        wm[k] -= eps
        fd = (mlp_oracle.loss_grad(wp, dims, x, y)[0] - mlp_oracle.loss_grad(wm, dims, x, y)[0]) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(fd)), (k, fd, g[k])
