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


@pytest.mark.parametrize('name', CASES)
def test_fp32_single_pass_with_walls(name):
    """FP32 walls in one pass (k_fused_walls: flags and the walls' psi in the
    halo reduction, bounce-back from a shared-memory flag ring) against the
    FP32 two-pass kernels (k_density_psi_walls + k_fcs_walls) and the FP64
    reference run: same populations to FP32 rounding of the two collision
    forms, mass conserved to FP32 rounding, FP64's density within 1e-3."""
    z, c = load(name)
    steps = int(z['steps'][-1])
    fluid = (z['walls'] == 1).ravel()
    out = []
    for path in (_lib.PATH_FUSED, _lib.PATH_TWO_PASS):
        s = start(z, c, precision=_lib.FP32_SHIFTED, rho0=0.2)
        s.set_tuning(path)
        assert s.kernels_per_step() == (1 if path == _lib.PATH_FUSED else 2)
        m0, _ = s.reductions()
        s.step(steps)
        m1, _ = s.reductions()
        assert abs(m1 - m0) / m0 < 1e-5, (name, path)
        out.append((s.get_populations().reshape(z['pop_init'].shape[0], -1)[:, fluid], s.get_density()[fluid]))
        s.close()
    assert rel_err(out[0][0], out[1][0]) < 1e-4, rel_err(out[0][0], out[1][0])
    want = z['pop_%d' % steps].reshape(z['pop_init'].shape[0], -1)[:, fluid].sum(0)
    assert rel_err(out[0][1], want) < 1e-3
