"""The reference's "simple" step family (MainLoopSimple, MainLoopSimpleSC,
MainLoopSimpleWalls[SC], MainLoopSimpleWallsGravity,
MainLoopSimpleWallsInletOutletSC; idpy/LBM/MultiPhase.py:164-1014): the
oracle's restatement (OracleSimple) against the reference's own runs
(tests/golden/simple_*.npz, made by tests/golden/make_golden_simple.py):
populations, density, velocity and psi bit-identical on every cell, wall
cells included, after every recorded step count."""
import glob
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from sclbm import XIStencils, FStencils

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
CASES = sorted(os.path.basename(p)[7:-4] for p in glob.glob(os.path.join(GOLDEN, 'simple_*.npz')))


def load(name):
    p = os.path.join(GOLDEN, 'simple_%s.npz' % name)
    if not os.path.exists(p):
        pytest.skip('fixture simple_%s not generated' % name)
    z = np.load(p)
    return z, json.loads(str(z['config_json']))


def kind(c):
    """(forcing, gravity, u_in) of the case's loop."""
    loop = c['loop']
    return ('sc' if loop.endswith('SC') else 'guo', c.get('g') if 'Gravity' in loop else None,
            c.get('u_in') if 'InletOutlet' in loop else None)


def test_all_loops_have_fixtures():
    loops = {load(n)[1]['loop'] for n in CASES}
    assert loops == {'MainLoopSimple', 'MainLoopSimpleSC', 'MainLoopSimpleWalls', 'MainLoopSimpleWallsSC',
                     'MainLoopSimpleWallsGravity', 'MainLoopSimpleWallsInletOutletSC'}


@pytest.mark.parametrize('name', CASES)
def test_oracle_simple_bitwise_equals_reference(name):
    z, c = load(name)
    x, f = XIStencils[c['xi']], FStencils[c['fs']]
    forcing, g, u_in = kind(c)
    s = O.OracleSimple(c['dims'], x['XIs'], x['Ws'], f['Es'], f['Ws'], c['G'], tau=c['tau'],
                       walls=z['walls'] if 'walls' in z.files else None,
                       psi_w=z['psi_w'] if 'psi_w' in z.files else None, forcing=forcing, gravity=g, u_in=u_in)
    s.set_state(z['pop_init'], z['n_init'])
    done = 0
    for k in z['steps']:
        s.run(int(k) - done)
        done = int(k)
        assert np.array_equal(s.pop.reshape(z['pop_%d' % k].shape), z['pop_%d' % k]), (name, k)
        assert np.array_equal(s.n.reshape(z['n_%d' % k].shape), z['n_%d' % k]), (name, k)
        assert np.array_equal(s.u.reshape(z['u_%d' % k].shape), z['u_%d' % k]), (name, k)
        assert np.array_equal(s.psi.reshape(z['psi_%d' % k].shape), z['psi_%d' % k]), (name, k)
