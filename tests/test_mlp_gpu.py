"""The cost model's network on the GPU: forward pass and gradients from the
library's kernels against the CPU oracle (oracle/mlp_oracle.py), and training
that actually fits."""
import numpy as np
import pytest

from oracle import mlp_oracle
from uxxxxxxxxh_gb300.costmodel import MLP

pytestmark = pytest.mark.gpu


def _dims(m):
    return [m.in_dim] + [m.hidden] * m.layers + [1]


def test_forward_matches_oracle(cuda):
    m = MLP(19, 64, 3, seed=3)
    x = np.random.default_rng(1).standard_normal((300, 19)).astype(np.float32)
    got = m.forward(x)
    want = mlp_oracle.forward(m.get_params(), _dims(m), x)[-1][:, 0]
    assert np.allclose(got, want, rtol=1e-4, atol=1e-5)


def test_gradients_match_oracle(cuda):
    m = MLP(19, 64, 3, seed=4)
    rng = np.random.default_rng(2)
    x = rng.standard_normal((97, 19)).astype(np.float32)
    y = rng.standard_normal(97).astype(np.float32)
    loss, g = m.loss_grad(x, y)
    wl, wg = mlp_oracle.loss_grad(m.get_params().astype(np.float64), _dims(m), x.astype(np.float64),
                                  y.astype(np.float64))
    assert loss == pytest.approx(wl, rel=1e-4)
    assert np.linalg.norm(g - wg) <= 1e-4 * np.linalg.norm(wg)
    assert np.max(np.abs(g - wg)) <= 1e-4 * np.max(np.abs(wg))


def test_training_fits_a_smooth_function(cuda):
    rng = np.random.default_rng(5)
    x = rng.uniform(-1, 1, (4096, 19)).astype(np.float32)
    y = (np.sin(2 * x[:, 0]) + x[:, 1] * x[:, 2] - 0.5 * x[:, 3] ** 2).astype(np.float32)
    m = MLP(19, 64, 3, seed=6)
    before = float(np.mean((m.forward(x) - y) ** 2))
    m.train(x, y, epochs=60, batch=128, lr=2e-3, seed=1)
    after = float(np.mean((m.forward(x) - y) ** 2))
    assert after < 0.05 * before and after < 0.02, (before, after)


def test_params_round_trip(cuda):
    a, b = MLP(19, 64, 3, seed=7), MLP(19, 64, 3, seed=8)
    b.set_params(a.get_params())
    x = np.random.default_rng(3).standard_normal((10, 19)).astype(np.float32)
    assert np.array_equal(a.forward(x), b.forward(x))
