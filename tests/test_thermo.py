"""The thermodynamic construction (sclbm.thermo) against the reference's own
SCThermo values (tests/golden/thermo.json, made by tests/golden/make_thermo.py):
critical point, flat-interface coexistence densities and pressure, surface
tension, for the E4/E6/E8 force stencils and both psi forms."""
import json
import os
from fractions import Fraction

import pytest

from sclbm import FStencils
from sclbm import thermo

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, 'golden', 'thermo.json')))['cases']
PSI = {'exp(-1/n)': 'exp', '1 - exp(-n)': '1mexp'}


@pytest.mark.parametrize('case', GOLD, ids=lambda c: '%s_%s_G%g' % (c['stencil'], PSI[c['psi']], c['G']))
def test_coexistence_matches_reference(case):
    assert 'error' not in case, case
    f = FStencils[case['stencil']]
    r = thermo.coexistence(case['G'], f['Es'], f['Ws'], psi=PSI[case['psi']])
    assert r['G_c'] == pytest.approx(case['G_c'], rel=1e-12)
    assert r['n_c'] == pytest.approx(case['n_c'], rel=1e-12)
    for k in ('n_l', 'n_g', 'p_0'):
        assert r[k] == pytest.approx(case[k], rel=1e-9), k
    assert r['sigma_f'] == pytest.approx(case['sigma_f'], rel=1e-7)


def test_stencil_constants():
    # eps = -2 alpha / beta and beta as the reference prints them
    want = {'D2E4': (0, 3), 'D2E6': (Fraction(2, 17), Fraction(17, 5)), 'D2E8': (Fraction(10, 31), Fraction(31, 7))}
    for st, (eps, beta) in want.items():
        k = thermo.stencil_constants(FStencils[st]['Es'], FStencils[st]['Ws'])
        assert k['eps'] == pytest.approx(float(eps), abs=1e-14)
        assert k['beta'] == pytest.approx(float(beta), rel=1e-14)
        assert k['e2'] == pytest.approx(1.0, rel=1e-14)


def test_no_phase_separation_above_critical_coupling():
    with pytest.raises(ValueError):
        thermo.ShanChen(-2.0, psi='exp')
