"""The MLP oracle's back-propagation against central finite differences of
its own loss (FP64, BF16 rounding off), and its BF16 rounding rule."""
import numpy as np

from oracle import mlp_oracle as orc


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.normal(0, 0.3, orc.NP)
    x = rng.uniform(-1, 1, (37, 5))
    t = rng.uniform(-1, 1, 37)
    g, _ = orc.gradient(p, x, t, exact=True)
    loss = lambda q: float(((orc.forward(q, x, exact=True)[0] - t) ** 2).mean())
    idx = np.concatenate([rng.choice(np.arange(a, b), size=min(6, b - a), replace=False) for a, b in
                          [(orc.OFF_W1, orc.OFF_B1), (orc.OFF_B1, orc.OFF_W2), (orc.OFF_W2, orc.OFF_B2),
                           (orc.OFF_B2, orc.OFF_W3), (orc.OFF_W3, orc.OFF_B3), (orc.OFF_B3, orc.OFF_W4),
                           (orc.OFF_W4, orc.OFF_B4), (orc.OFF_B4, orc.NP)]])
    h = 1e-6
    for i in idx:
        e = np.zeros(orc.NP)
        e[i] = h
        fd = (loss(p + e) - loss(p - e)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])


def test_bf16_rounding():
    # 1 + 2^-8 is halfway between 1 and 1 + 2^-7: ties to even -> 1
    assert orc.bf16(np.float32(1 + 2 ** -8)) == 1.0
    assert orc.bf16(np.float32(1 + 3 * 2 ** -8)) == 1 + 2 ** -6
    assert orc.bf16(np.float32(-2.5)) == -2.5
