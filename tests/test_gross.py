"""Fluctuating Shan-Chen step (Gross et al. 2011, MainLoopGross2011SRT): the
oracle against the reference's own runs (tests/golden/gross_*.npz, made by
tests/golden/make_golden_gross.py: MMIX, MINSTD and NUMREC generators, one or
two generators per random moment, D2Q9 E4/E6/E8 and D3Q19 E4/E6, tau
0.8-1.2), the noise operator of the library (C++ rationals) against the
oracle's (Python fractions) and the reference's literals, and the seeding of
the drop-in against the reference's draws."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from sclbm import _lib, XIStencils, FStencils
from sclbm.MultiPhase import CRNGS

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
CASES = ['d2e4_mmix_t1', 'd2e8_minstd_indep_t08', 'd2e6_numrec_t12_psi1mexp', 'd3e4_mmix_t1',
         'd3e6_minstd_indep_t09']


def load(name):
    p = os.path.join(GOLDEN, 'gross_%s.npz' % name)
    if not os.path.exists(p):
        pytest.skip('fixture gross_%s not generated' % name)
    z = np.load(p)
    return z, json.loads(str(z['config_json'])), json.loads(str(z['noise_json']))


def oracle_case(z, c, literals):
    x, f = XIStencils[c['xi']], FStencils[c['fs']]
    s = O.OracleSim(c['dims'], x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], c['G'], tau=c['tau'], psi=c['psi'])
    s.set_fields(z['n_init'])
    s.init_populations()
    assert np.array_equal(s.populations(), z['pop_init'])
    s.set_fluctuations(c['kind'], c['indep'], c['kBT'], c['n0'], z['seeds_init'], c['tau'], literals)
    return s


def dense(terms, Q, nr):
    out = np.zeros((Q, nr))
    for q, tl in enumerate(terms):
        for cf, k in tl:
            out[q, k] = cf
    return out


@pytest.mark.parametrize('name', CASES)
def test_oracle_bitwise_equals_reference_with_its_literals(name):
    """Populations, density and generator states identical to the reference
    after every recorded step count."""
    z, c, nl = load(name)
    s = oracle_case(z, c, nl)
    done = 0
    for k in z['steps']:
        s.run(int(k) - done)
        done = int(k)
        assert np.array_equal(s.get_seeds(), z['seeds_%d' % k]), (name, k)
        assert np.array_equal(s.populations(), z['pop_%d' % k]), (name, k)
        assert np.array_equal(s.density(), z['n_%d' % k]), (name, k)


@pytest.mark.parametrize('name', CASES)
def test_oracle_own_operator(name):
    """With its own exact operator the oracle is bit-identical in 2D; in 3D the
    reference's sympy-float literals differ by <= 1e-15 (terms of 1e-17 where
    the exact coefficient is 0, last-digit differences), which after 20
    steps is < 1e-13 relative."""
    z, c, _ = load(name)
    s = oracle_case(z, c, None)
    done = 0
    for k in z['steps']:
        s.run(int(k) - done)
        done = int(k)
        assert np.array_equal(s.get_seeds(), z['seeds_%d' % k]), (name, k)
        got, want = s.populations(), z['pop_%d' % k]
        if c['xi'] == 'D2Q9':
            assert np.array_equal(got, want), (name, k)
        else:
            assert np.abs(got - want).max() / np.abs(want).max() < 1e-13, (name, k)


@pytest.mark.parametrize('name', CASES)
def test_noise_operators_agree(name):
    """The library's builder (sclbm_noise_operator, C++ rationals) equals the
    oracle's (Python fractions) bit for bit; both equal the reference's
    literals in 2D and are within 1e-15 (coefficients) / 1e-15 relative
    (variances) of them in 3D."""
    z, c, nl = load(name)
    x = XIStencils[c['xi']]
    D = len(c['dims'])
    Q = len(x['XIs'])
    mv, cf = _lib.noise_operator(D, x['XIs'], x['Ws'], x['c2'], c['tau'], c['kBT'], c['n0'])
    ot, norms = O.noise_terms([tuple(v) for v in x['XIs']], x['Ws'], x['c2'])
    om = np.array([-2.0 * O.noise_variance(nm, c['kBT'], 1.0 / (1.0 / c['tau']), c['n0']) for nm in norms])
    nr = Q - D - 1
    assert np.array_equal(cf, dense(ot, Q, nr))
    assert np.array_equal(mv, om)
    lt, lv = O.noise_from_literals(nl)
    ref = dense(lt, Q, nr)
    if D == 2:
        assert np.array_equal(cf, ref) and np.array_equal(mv, np.array(lv))
    else:
        assert np.abs(cf - ref).max() <= 1e-15
        assert np.abs(mv - lv).max() / np.abs(lv).max() <= 1e-15


def test_noise_term_order_is_the_printed_order():
    """Every population's terms come in the order of the moment names sorted
    as strings (Rm_0, Rm_1, Rm_10, ..., Rm_2, ...), as in the generated kernel."""
    _, _, nl = load('d3e4_mmix_t1')
    for tl in nl['terms']:
        names = ['Rm_%d' % k for k, _ in tl]
        assert names == sorted(names)


def test_noise_conserves_mass_and_momentum():
    """The noise populations of every random moment carry no mass and no
    momentum (exact operator: rows 0..D of the W-orthogonal basis)."""
    for lat in ('D2Q9', 'D3Q19'):
        x = XIStencils[lat]
        D = len(x['XIs'][0])
        _, cf = _lib.noise_operator(D, x['XIs'], x['Ws'], x['c2'], 1.0, 1e-4, 1.0, literals=_lib.LIT_EXACT)
        xi = np.array(x['XIs'], np.float64)
        assert np.abs(cf.sum(0)).max() < 1e-15
        assert np.abs(xi.T @ cf).max() < 1e-15


@pytest.mark.parametrize('name', CASES)
def test_dropin_seeding_matches_reference(name):
    """CRNGS seeding of the drop-in (numpy legacy generator, init_seed) draws the
    reference's initial generator states."""
    z, c, _ = load(name)
    want = z['seeds_init']
    got = CRNGS(c['kind'], want.size, 'numpy', c['init_seed'], owner=None)._cache
    assert got.dtype == want.dtype
    assert np.array_equal(got, want)


def test_generator_streams():
    """One step of each generator against its recurrence in Python integers;
    MINSTD stays in [1, 2^31 - 2]."""
    def step(kind, s):
        if kind == 'MMIX':
            return (s * 6364136223846793005 + 1442695040888963407) % 2 ** 64
        if kind == 'NUMREC':
            return (s * 1664525 + 1013904223) % 2 ** 32
        return (s * 16807) % (2 ** 31 - 1)
    for name in CASES:
        z, c, _ = load(name)
        s0, s1 = z['seeds_init'].astype(object), z['seeds_1'].astype(object)
        draws = 1 if c['indep'] else 2
        exp = s0.copy()
        for _ in range(draws):
            exp = np.array([step(c['kind'], int(v)) for v in exp], dtype=object)
        assert np.array_equal(exp, s1), name
        if c['kind'] == 'MINSTD':
            assert int(z['seeds_200' if 'seeds_200' in z else 'seeds_20'].max()) < 2 ** 31 - 1


def test_single_pass_noise_mask_matches_operator():
    """The compile-time nonzero pattern the single-pass kernel assumes
    (NoiseMask in noise.cuh) is the exact operator's."""
    import re
    src = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                            'idea.deploy_gb300', 'csrc', 'noise.cuh')).read()
    for lat in ('D2Q9', 'D3Q19'):
        m = re.search(r'struct NoiseMask<%s> \{.*?constexpr unsigned t\[\d+\] = \{([^}]*)\}' % lat, src, re.S)
        masks = [int(v, 16) for v in m.group(1).replace('\n', ' ').split(',')]
        x = XIStencils[lat]
        D = len(x['XIs'][0])
        for lit in (_lib.LIT_EXACT, _lib.LIT_ROUND15):
            _, cf = _lib.noise_operator(D, x['XIs'], x['Ws'], x['c2'], 1.0, 1e-4, 1.0, literals=lit)
            want = [sum(1 << k for k in range(cf.shape[1]) if cf[q, k] != 0) for q in range(cf.shape[0])]
            assert masks == want, lat
