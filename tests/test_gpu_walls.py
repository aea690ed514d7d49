"""Walls on the GPU (sclbm_set_walls, the drop-in GetWalls / MainLoopWalls)
against the reference's own runs (tests/golden/walls_*.npz): populations and
density on every fluid cell within 1e-12 of the reference after 1 .. 1000
steps (FP64, the reference's literals and arithmetic); mass conserved; the
FP32-shifted path close to FP64."""
import numpy as np
import pytest

from helpers import rel_err
from sclbm import _lib, XIStencils, FStencils
from test_walls import CASES, load

pytestmark = pytest.mark.gpu


def make(c, **kw):
    x, f = XIStencils[c['xi']], FStencils[c['fs']]
    return _lib.Sim(len(c['dims']), c['dims'], x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], c['G'], tau=c['tau'],
                    **kw)


def start(z, c, **kw):
    s = make(c, **kw)
    s.set_density(z['n_init'])
    s.set_velocity(np.zeros(len(c['dims']) * s.V))
    s.init_populations()
    s.set_walls(z['walls'], z['psi_w'])
    return s


@pytest.mark.parametrize('name', CASES)
def test_walls_match_reference(name):
    z, c = load(name)
    s = start(z, c)
    assert s.kernels_per_step() == 2
    fluid = (z['walls'] == 1).ravel()
    Q = z['pop_init'].shape[0]
    done = 0
    for k in z['steps']:
        s.step(int(k) - done)
        done = int(k)
        got = s.get_populations().reshape(Q, -1)[:, fluid]
        want = z['pop_%d' % k].reshape(Q, -1)[:, fluid]
        assert rel_err(got, want) < 1e-12, (name, k, rel_err(got, want))
        # the density of the current populations (the reference's n array
        # holds the density at the start of the last step instead)
        n = s.get_density()[fluid]
        assert rel_err(n, want.sum(0)) < 1e-12, (name, k)
    s.close()


def test_walls_conserve_mass_and_fp32_follows_fp64():
    z, c = load('d2e4_bgk_t1')
    s64 = start(z, c, literals=_lib.LIT_EXACT)
    m0, _ = s64.reductions()
    s64.step(1000)
    m1, _ = s64.reductions()
    assert abs(m1 - m0) / m0 < 1e-13
    s32 = start(z, c, precision=_lib.FP32_SHIFTED, rho0=0.2)
    s32.step(1000)
    fluid = (z['walls'] == 1).ravel()
    assert rel_err(s32.get_density()[fluid], s64.get_density()[fluid]) < 1e-3
    m32, _ = s32.reductions()
    assert abs(m32 - m0) / m0 < 1e-5
    s64.close()
    s32.close()


def test_dropin_getwalls_mainloopwalls():
    import sympy as sp
    from sclbm import ShanChenMultiPhase, CUDA_T
    z, c = load('d2e8_bgk_t08')
    ShanChenMultiPhase.verbose = False
    sc = ShanChenMultiPhase(lang=CUDA_T, dim_sizes=tuple(c['dims']), xi_stencil=XIStencils[c['xi']],
                            f_stencil=FStencils[c['fs']], psi_code='exp(-1./ln_0)', psi_sym=None, SC_G=c['G'],
                            tau=c['tau'])
    with pytest.raises(Exception):
        sc.MainLoopWalls([0, 1])   # no walls yet
    sc.sims_idpy_memory['n'].H2D(z['n_init'].ravel())
    sc.sims_idpy_memory['u'].SetConst(0.)
    sc.init_status['n'] = sc.init_status['u'] = True
    sc.InitPopulations()
    sc.GetWalls(z['walls'], z['psi_w'])
    sc.MainLoopWalls([0, 100])
    fluid = z['walls'] == 1
    Q = z['pop_init'].shape[0]
    pop = sc.GetPopulations().reshape((Q,) + z['walls'].shape) if hasattr(sc, 'GetPopulations') else None
    if pop is not None:
        assert rel_err(pop[:, fluid], z['pop_100'][:, fluid]) < 1e-12
    sc.End()
