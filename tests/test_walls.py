"""Walls (GetWalls / MainLoopWalls): the oracle against the reference's own
runs (tests/golden/walls_*.npz, made by tests/golden/make_golden_walls.py):
bit-identical populations on every fluid cell after 1, 100 and 1000 steps of
a droplet resting on a wall (2D E4 and E8 channels, a 3D E4 slab)."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from sclbm.LBM import XIStencils, FStencils

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
CASES = ['d2e4_bgk_t1', 'd2e8_bgk_t08', 'd3e4_bgk_t1']


def load(name):
    p = os.path.join(GOLDEN, 'walls_%s.npz' % name)
    if not os.path.exists(p):
        pytest.skip('fixture walls_%s not generated' % name)
    z = np.load(p)
    return z, json.loads(str(z['config_json']))


def oracle_case(z, c):
    x, f = XIStencils[c['xi']], FStencils[c['fs']]
    s = O.OracleSim(c['dims'], x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], c['G'], tau=c['tau'], psi=c['psi'])
    s.set_fields(z['n_init'])
    s.init_populations()
    return s


@pytest.mark.parametrize('name', CASES)
def test_oracle_walls_bitwise_equals_reference(name):
    z, c = load(name)
    s = oracle_case(z, c)
    assert np.array_equal(s.populations(), z['pop_init'])
    s.set_walls(z['walls'], z['psi_w'])
    fluid = z['walls'] == 1
    done = 0
    for k in z['steps']:
        s.run(int(k) - done)
        done = int(k)
        got, want = s.populations(), z['pop_%d' % k]
        assert np.array_equal(got[:, fluid], want[:, fluid]), (name, k)
        assert np.array_equal(s.density()[fluid], z['n_%d' % k][fluid]), (name, k)
