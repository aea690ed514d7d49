"""Seeded synthetic initial densities (host side, numpy, FP64).

``droplet`` is the benchmark workload's initial state: a tanh droplet about the
box centre ``L//2`` (the reference's ``dim_center``, idpy/LBM/LBM.py:422),
rho = (rho_l+rho_g)/2 - (rho_l-rho_g)/2 * tanh((r-R)/width), multiplied by
(1 + noise*U(-1,1)) drawn from ``numpy.random.default_rng(seed)``.  Arrays are
shaped ``flip(dims)`` (x fastest), like the reference's ``GetDensityField``.
"""
import numpy as np


def radius_field(dims):
    grids = np.meshgrid(*[np.arange(L) for L in reversed(dims)], indexing='ij')
    r2 = np.zeros(grids[0].shape)
    for d, L in enumerate(dims):
        r2 += (grids[len(dims) - 1 - d] - L // 2) ** 2
    return np.sqrt(r2)


def droplet(dims, R, rho_l, rho_g, width=2.0, seed=1234, noise=1e-4):
    r = radius_field(dims)
    rho = 0.5 * (rho_l + rho_g) - 0.5 * (rho_l - rho_g) * np.tanh((r - R) / width)
    if noise:
        rng = np.random.default_rng(seed)
        rho = rho * (1.0 + noise * rng.uniform(-1.0, 1.0, rho.shape))
    return rho
