"""The warm-start MLP kernels against the FP64 CPU oracle (oracle/mlp_oracle.py):
forward outputs, the back-propagated gradient of every parameter group, one
Adam step with the device's own sample draw, determinism, and that training
fits a droplet-like profile."""
import numpy as np
import pytest

from sclbm.mlp import MLP
from oracle import mlp_oracle as orc

pytestmark = pytest.mark.gpu

GROUPS = {'W1': (orc.OFF_W1, orc.OFF_B1), 'b1': (orc.OFF_B1, orc.OFF_W2), 'W2': (orc.OFF_W2, orc.OFF_B2),
          'b2': (orc.OFF_B2, orc.OFF_W3), 'W3': (orc.OFF_W3, orc.OFF_B3), 'b3': (orc.OFF_B3, orc.OFF_W4),
          'W4': (orc.OFF_W4, orc.OFF_B4), 'b4': (orc.OFF_B4, orc.NP)}


def data(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1.5, 1.5, (n, 5)).astype(np.float32)
    t = np.tanh(2 * x[:, 4] - x[:, 2]) * 0.8 + 0.1 * x[:, 0]
    return x, t.astype(np.float32)


def test_forward_matches_oracle():
    m = MLP(seed=3)
    x, _ = data(1000, 1)
    y = m.predict(x)
    yo, _ = orc.forward(m.params(), x)
    assert np.abs(y - yo).max() < 2e-3 * max(1.0, np.abs(yo).max())
    assert np.median(np.abs(y - yo)) < 1e-5
    m.close()


@pytest.mark.parametrize('n', [64, 200, 1000])
def test_gradient_matches_oracle(n):
    m = MLP(seed=11)
    # larger weights than the default init, so every layer carries signal
    rng = np.random.default_rng(5)
    w = (m.params() * 2 + rng.normal(0, 0.05, m.n_params)).astype(np.float32)
    m.set_params(w)
    x, t = data(n, 2)
    g, loss = m.gradient(x, t)
    go, lo = orc.gradient(w, x, t)
    assert abs(loss - lo) <= 1e-5 * lo
    for name, (a, b) in GROUPS.items():
        err = np.linalg.norm(g[a:b] - go[a:b]) / max(np.linalg.norm(go[a:b]), 1e-30)
        assert err < 5e-3, (name, err)
    m.close()


def test_adam_step_matches_oracle():
    m = MLP(seed=21)
    w0 = m.params().astype(np.float64)
    x, t = data(300, 4)
    m.set_data(x, t)
    lr = 1e-3
    m.train(1, batch=128, lr=lr)
    w1 = m.params().astype(np.float64)
    idx = orc.sample_indices(21, 0, 128, 300)
    g, _ = orc.gradient(w0, x[idx], t[idx])
    wo, _, _ = orc.adam(w0, g, np.zeros_like(g), np.zeros_like(g), 1, lr)
    # the first Adam step moves each parameter by lr * g / (|g| + eps)
    assert np.abs(w1 - w0).max() <= lr * (1 + 1e-5)
    big = np.abs(g) > 1e-3 * np.abs(g).max()
    assert np.abs(w1 - wo)[big].max() < 1e-3 * lr + 1e-7
    m.close()


def test_training_is_deterministic_and_fits():
    x, t = data(20000, 7)
    out = []
    for _ in range(2):
        m = MLP(seed=5)
        m.set_data(x, t)
        loss = m.train(1200, batch=4096, lr=3e-3)
        out.append((loss, m.params()))
        m.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    loss = out[0][0]
    assert loss[-50:].mean() < 0.05 * loss[:10].mean()
