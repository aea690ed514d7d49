"""What the learned warm start gives: droplets started from the trained
network's profiles (radius set so that each carries the mass of its tanh
start) reach the same equilibrium Laplace pressure as droplets started from
the tanh profile, and start much closer to it (their density changes far less
over the first steps); a warm start far from equilibrium is caught by that
residual and restarted cold."""
import numpy as np
import pytest

from sclbm import sweep, warmstart
from sclbm.profiles import droplet

pytestmark = pytest.mark.gpu

RADII = [12.0, 18.0, 24.0, 15.0]
G = [-4.6, -4.75, -4.9, -4.55]


@pytest.fixture(scope='module')
def trained():
    prof, st = warmstart.equilibrium_profiles(n=96, seed=3, G_range=(-5.0, -4.5), R_range=(8.0, 30.0), taus=(1.0,),
                                              orders=(8,), max_steps=60000)
    ok = [p for p in prof if p['status'] == 'converged']
    assert len(ok) >= 80, st
    m, loss, _ = warmstart.train(ok, steps=6000, batch=4096, lr=2e-3, seed=1)
    assert loss[-100:].mean() < 1e-3 * loss[:10].mean()
    table = warmstart.ThermoTable((-5.0, -4.5), orders=(8,))
    rl, rg = map(list, zip(*[table(g, 8) for g in G]))
    masses = [droplet((warmstart.box_of(R),) * 2, R, a, b, 2.0, 0, 0.0).sum() for R, a, b in zip(RADII, rl, rg)]
    yield m, rl, rg, masses
    m.close()


def test_warm_start_reaches_the_same_equilibrium_from_closer(trained):
    m, rl, rg, masses = trained
    fields = warmstart.warm_fields(m, RADII, G, masses=masses)
    for f, M in zip(fields, masses):
        assert abs(f.sum() / M - 1) < 1e-3   # the radius carries the mass
    cold_fields = [droplet((warmstart.box_of(R),) * 2, R, a, b, 2.0, i, 0.0)
                   for i, (R, a, b) in enumerate(zip(RADII, rl, rg))]
    cold = sweep.ragged_sweep(RADII, G, rl, rg, max_steps=60000, init=cold_fields, residual_max=1e9)
    warm = sweep.ragged_sweep(RADII, G, rl, rg, max_steps=60000, init=fields, residual_max=0.1)
    assert (cold['status'] == 'converged').all() and (warm['status'] == 'converged').all()
    assert not warm['fallback'].any(), warm['residual']
    assert np.abs(warm['dp'] / cold['dp'] - 1).max() < 1e-4
    assert np.median(warm['residual']) < 0.5 * np.median(cold['residual']), (warm['residual'], cold['residual'])


def test_bad_warm_start_falls_back_to_cold(trained):
    m, rl, rg, masses = trained
    fields = warmstart.warm_fields(m, RADII, G, masses=masses)
    # a droplet far from coexistence: its liquid is 40% too light
    L = fields[1].shape[0]
    fields[1] = droplet((L, L), RADII[1], 0.6 * rl[1], rg[1], 2.0, 0, 0.0)
    warm = sweep.ragged_sweep(RADII, G, rl, rg, max_steps=60000, init=fields, residual_max=0.1)
    assert warm['fallback'][1] and warm['fallback'].sum() == 1
    cold = sweep.ragged_sweep(RADII[1:2], G[1:2], rl[1:2], rg[1:2], max_steps=60000)
    assert abs(warm['dp'][1] / cold['dp'][0] - 1) < 1e-4


def test_3d_warm_start_same_equilibrium_and_fallback():
    """The 3D batch (D3Q19, E6) started from a network trained on 3D
    equilibrium profiles: each warm field carries its tanh start's mass, the
    warm and cold batches reach the same Laplace pressure, the warm start's
    residual is lower, and a warm start far from coexistence falls back."""
    prof, st = warmstart.equilibrium_profiles_3d(n=24, seed=5, R_range=(11.0, 15.0), G_range=(-4.8, -4.5), L=48,
                                                 max_steps=20000)
    ok = [p for p in prof if p['status'] == 'converged']
    assert len(ok) >= 16, st
    m, loss, _ = warmstart.train(ok, steps=4000, batch=4096, lr=2e-3, seed=2)
    radii, G = [12.0, 13.5, 14.5], [-4.55, -4.7, -4.62]
    guess = [sweep.thermo_guess(g, 'D2E6') for g in G]
    rl, rg = [a for a, _ in guess], [b for _, b in guess]
    masses = [droplet((48,) * 3, R, a, b, 2.0, 0, 0.0).sum() for R, a, b in zip(radii, rl, rg)]
    fields = warmstart.warm_fields(m, radii, G, tau=1.0, order=6, masses=masses, dim=3, box=48)
    for f, M in zip(fields, masses):
        assert f.shape == (48, 48, 48) and abs(f.sum() / M - 1) < 1e-3
    kw = dict(stencil='D3E6', dim=3, boxes=[48] * 3, max_steps=20000)
    cold = sweep.ragged_sweep(radii, G, rl, rg, init=[droplet((48,) * 3, R, a, b, 2.0, i, 0.0)
                                                       for i, (R, a, b) in enumerate(zip(radii, rl, rg))],
                              residual_max=1e9, **kw)
    warm = sweep.ragged_sweep(radii, G, rl, rg, init=fields, residual_max=0.1, **kw)
    assert (cold['status'] == 'converged').all() and (warm['status'] == 'converged').all(), (cold, warm)
    assert not warm['fallback'].any(), warm['residual']
    assert np.abs(warm['dp'] / cold['dp'] - 1).max() < 1e-3, (warm['dp'], cold['dp'])
    assert np.median(warm['residual']) < np.median(cold['residual']), (warm['residual'], cold['residual'])
    fields[0] = droplet((48,) * 3, radii[0], 0.6 * rl[0], rg[0], 2.0, 0, 0.0)
    bad = sweep.ragged_sweep(radii, G, rl, rg, init=fields, residual_max=0.1, **kw)
    assert bad['fallback'][0] and bad['fallback'].sum() == 1
    m.close()
