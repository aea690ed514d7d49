"""Pin the CPU oracle to the reference: fixtures made by running the reference's
own CTypes FP64 path (tests/golden/make_golden.py).  CPU only."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from sclbm.LBM import XIStencils, FStencils

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')

BGK_CASES = ['d2e4_bgk_t1', 'd2e8_bgk_t08', 'd2e6_bgk_t12_psi1mexp', 'd3e6_bgk_t1',
             'd3e4_bgk_t09', 'd3e8_bgk_t1']
MRT_CASES = ['d2e4_mrt', 'd3e6_mrt_ones', 'd3e6_mrt_rates']


def load(name):
    p = os.path.join(GOLDEN, name + '.npz')
    if not os.path.exists(p):
        pytest.skip('fixture %s not generated' % name)
    z = np.load(p)
    return z, json.loads(str(z['config_json']))


def make(cfg, **kw):
    x, f = XIStencils[cfg['xi']], FStencils[cfg['fs']]
    return O.OracleSim(cfg['dims'], x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], cfg['G'],
                       tau=cfg['tau'], psi=cfg['psi'], rates=cfg.get('rates'), **kw)


def test_stencil_tables_are_the_references():
    t = json.loads(str(np.load(os.path.join(GOLDEN, 'mrt_basis.npz'))['tables_json']))
    for k, v in t['XIStencils'].items():
        assert [list(e) for e in XIStencils[k]['XIs']] == v['XIs']
        assert list(XIStencils[k]['Ws']) == v['Ws'] and XIStencils[k]['c2'] == v['c2']
    for k, v in t['FStencils'].items():
        assert [list(e) for e in FStencils[k]['Es']] == v['Es']
        assert list(FStencils[k]['Ws']) == v['Ws']


@pytest.mark.parametrize('lat', ['D2Q9', 'D3Q19'])
def test_hermite_bases_match_reference(lat):
    z = np.load(os.path.join(GOLDEN, 'mrt_basis.npz'))
    x = XIStencils[lat]
    M, Mw = O.hermite_bases(x['XIs'], x['Ws'], x['c2'])
    np.testing.assert_allclose(np.array(M, float), z['M_' + lat], rtol=0, atol=1e-14)
    np.testing.assert_allclose(np.array(Mw, float), z['MWOrth_' + lat], rtol=0, atol=1e-14)


@pytest.mark.parametrize('name', BGK_CASES)
def test_bgk_literals_match_reference(name):
    z, cfg = load(name)
    lit = json.loads(str(z['lit_json']))
    x = XIStencils[cfg['xi']]
    terms = O.bgk_terms(x['XIs'], x['Ws'], x['c2'], 1.0 / cfg['tau'])
    for q, tl in enumerate(terms):
        mine = [(n, '%.15g' % c) for c, n in tl]
        ref = [(k, '%.15g' % float(v)) for k, v in lit[str(q)].items()]
        assert mine == ref, (q, mine, ref)


@pytest.mark.parametrize('name', MRT_CASES)
def test_mrt_literals_close_to_reference(name):
    z, cfg = load(name)
    lit = json.loads(str(z['lit_json']))
    x = XIStencils[cfg['xi']]
    terms = O.mrt_terms(x['XIs'], x['Ws'], x['c2'], cfg['rates'], mode='exact')
    for q, tl in enumerate(terms):
        mine = {n: c for c, n in tl}
        ref = {k: float(v) for k, v in lit[str(q)].items()}
        for k in set(mine) | set(ref):
            assert abs(mine.get(k, 0.0) - ref.get(k, 0.0)) < 2e-14, (q, k)
        # same print order for the terms both keep
        common = [k for k in ref if k in mine]
        assert common == [k for k in mine if k in ref]


# Own exact MRT operator vs the reference's sympy-float literals: the reference's
# MRT literals carry float round-off (column sums off by up to ~7e-16, so its mass
# drifts by ~6e-16 per step); after 1000 steps the fields differ by ~2e-12 (n)
# and ~1.2e-11 (u) relative.  The same operator (its literals) is bit-identical.
MRT_OWN_TOL = dict(n=1e-11, u=5e-11, mass=1e-12)


def _run_case(z, cfg, sim, exact, tol=None):
    tol = tol or dict(n=1e-12, u=1e-12, mass=1e-13)
    sim.set_fields(z['n_init'])
    sim.init_populations()
    if exact:
        assert np.array_equal(sim.populations(), z['pop_init'])
    else:
        np.testing.assert_allclose(sim.populations(), z['pop_init'], rtol=1e-15, atol=0)
    prev = 0
    uconv, maxu = [], []
    for k in cfg['steps']:
        sim.run(k - prev)
        prev = k
        if k == 1:
            got = sim.populations()
            if exact:
                assert np.array_equal(got, z['pop_step1'])
            else:
                np.testing.assert_allclose(got, z['pop_step1'], rtol=1e-14, atol=1e-16)
        sim.compute_moments()
        n, u = sim.density(), sim.velocity()
        if exact:
            assert np.array_equal(n, z['n_%d' % k]), k
            assert np.array_equal(u, z['u_%d' % k]), k
            assert sim.mass() == float(z['mass_%d' % k])
        else:
            assert np.abs(n - z['n_%d' % k]).max() <= tol['n'] * np.abs(z['n_%d' % k]).max(), k
            assert np.abs(u - z['u_%d' % k]).max() <= tol['u'] * np.abs(z['u_%d' % k]).max() + 1e-15, k
            assert abs(sim.mass() - float(z['mass_%d' % k])) <= tol['mass'] * float(z['mass_%d' % k])
        a, b = sim.check_u()
        uconv.append(a)
        maxu.append(b)
    np.testing.assert_allclose(uconv, z['uconv'], rtol=1e-10)
    np.testing.assert_allclose(maxu, z['maxu'], rtol=1e-10)
    np.testing.assert_allclose(sim.delta_p(), z['dp'], rtol=1e-10, atol=1e-14)


@pytest.mark.parametrize('name', BGK_CASES)
def test_oracle_bitwise_equals_reference_bgk(name):
    """Own coefficients (15-digit literals): bit-identical fields and mass."""
    z, cfg = load(name)
    _run_case(z, cfg, make(cfg), exact=True)


@pytest.mark.parametrize('name', MRT_CASES)
def test_oracle_bitwise_equals_reference_mrt_literals(name):
    """The reference's own MRT literals driven through the oracle: bit-identical."""
    z, cfg = load(name)
    lit = json.loads(str(z['lit_json']))
    _run_case(z, cfg, make(cfg, literals=lit), exact=True)


@pytest.mark.parametrize('name', MRT_CASES)
def test_oracle_mrt_own_coefficients_close(name):
    """Own exact MRT operator (not sympy's float arithmetic): within MRT_OWN_TOL."""
    z, cfg = load(name)
    _run_case(z, cfg, make(cfg, mode='round15'), exact=False, tol=MRT_OWN_TOL)


def test_init_profiles_match_reference():
    z = np.load(os.path.join(GOLDEN, 'init_profiles.npz'))
    for tag, dims in [('2d', (40, 32)), ('3d', (12, 10, 8))]:
        R = dims[0] / 4.0
        np.testing.assert_allclose(O.init_radial(dims, 0.15, 2.2, R), z['radial_' + tag],
                                   rtol=0, atol=1e-15)
        np.testing.assert_allclose(O.init_radial(dims, 0.15, 2.2, R, full_flag=False),
                                   z['radial_inv_' + tag], rtol=0, atol=1e-15)
        np.testing.assert_allclose(O.init_flat(dims, 0.2, 4.5, dims[0] / 2.0, 0), z['flat_' + tag],
                                   rtol=1e-15, atol=1e-15)
        np.testing.assert_allclose(O.init_flat(dims, 0.2, 4.5, dims[1] / 3.0, 1),
                                   z['flat_d1_' + tag], rtol=1e-15, atol=1e-15)
        np.testing.assert_allclose(O.init_single_flat(dims, 0.2, 4.5, 0), z['single_flat_' + tag],
                                   rtol=1e-15, atol=1e-15)
    np.testing.assert_allclose(O.init_cylinder((12, 10, 8), 0.2, 4.5, 3.0, 2), z['cylinder_3d'],
                               rtol=0, atol=1e-15)


def test_divergence_onset_matches_reference():
    """The headline 2D configuration as written (G=-5, 2.2/0.15) blows up; the
    oracle reproduces the reference's per-step extrema while they are finite."""
    z, cfg = load('div_cfg1')
    stats = z['stats']
    sim = make(cfg)
    from sclbm.profiles import droplet   # the product's seeded droplet generator
    sim.set_fields(droplet(cfg['dims'], cfg['R'], cfg['rl'], cfg['rg'], cfg['width'], cfg['seed']))
    sim.init_populations()
    onset_ref = next(i for i, s in enumerate(stats) if not (s[2] and abs(s[0]) < 1e10))
    for k in range(len(stats)):
        sim.run(1)
        n = sim.populations().sum(axis=0)
        if k < onset_ref:
            np.testing.assert_allclose([n.max(), n.min()], stats[k][:2], rtol=1e-9)
        else:
            assert not (np.isfinite(n).all() and np.abs(n).max() < 1e10)
            break


def test_full_size_twin_1000_steps():
    """256^2, R=48, G=-4.5: the full-size stable twin after 1000 steps (bitwise)."""
    z, cfg = load('full_twin_256')
    sim = make(cfg)
    from sclbm.profiles import droplet
    sim.set_fields(droplet(cfg['dims'], cfg['R'], cfg['rl'], cfg['rg'], cfg['width'], cfg['seed']))
    sim.init_populations()
    assert sim.mass() == float(z['mass_0'])
    sim.run(1000)
    sim.compute_moments()
    n = sim.density()
    assert sim.mass() == float(z['mass_1000'])
    assert np.array_equal(n[128, :], z['row_1000'])
    assert np.array_equal(n[:, 128], z['col_1000'])
    u = sim.u.reshape(256, 256, 2)
    assert np.array_equal(u[148], z['urow_1000'])
