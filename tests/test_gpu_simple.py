"""The simple step family on the GPU (sclbm_set_simple, the drop-in
MainLoopSimple* loops) against the reference's own runs
(tests/golden/simple_*.npz): FP64 in the reference's operation order;
populations, density, velocity and psi on every non-wall cell within 1e-12
(relative, max-norm; psi uses CUDA's exp, which may differ from glibc's by an
ulp) after every recorded step count.  FP32-shifted within 1e-3 of the
reference, mass-conserving."""
import numpy as np
import pytest

from helpers import rel_err
from sclbm import _lib, XIStencils, FStencils
from sclbm.MultiPhase import ShanChenMultiPhase
from test_simple import CASES, load, kind

pytestmark = pytest.mark.gpu


def start(z, c):
    x, f = XIStencils[c['xi']], FStencils[c['fs']]
    D = len(c['dims'])
    s = _lib.Sim(D, c['dims'], x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], c['G'], tau=c['tau'])
    has_walls = 'walls' in z.files
    if has_walls:
        s.set_walls(z['walls'], z['psi_w'])
    s.set_populations(z['pop_init'])
    s.set_density(z['n_init'])
    s.set_velocity(np.zeros(D * s.V))
    forcing, g, u_in = kind(c)
    s.set_simple(_lib.SIMPLE_SC if forcing == 'sc' else _lib.SIMPLE_GUO, use_walls=has_walls, gravity=g,
                 inlet_outlet=u_in is not None, u_in=u_in or 0.0)
    return s


@pytest.mark.parametrize('name', CASES)
def test_simple_step_matches_reference(name):
    z, c = load(name)
    s = start(z, c)
    D, Q = len(c['dims']), z['pop_init'].shape[0]
    live = (z['walls'] != 0).ravel() if 'walls' in z.files else np.ones(s.V, bool)
    done = 0
    for k in z['steps']:
        s.step(int(k) - done)
        done = int(k)
        pop = s.get_populations().reshape(Q, -1)[:, live]
        assert rel_err(pop, z['pop_%d' % k].reshape(Q, -1)[:, live]) < 1e-12, (name, k)
        assert rel_err(s.get_density()[live], z['n_%d' % k].ravel()[live]) < 1e-12, (name, k)
        u = s.get_velocity().reshape(D, -1)[:, live]
        ref_u = z['u_%d' % k].reshape(D, -1)[:, live]
        assert np.abs(u - ref_u).max() < 1e-12 * max(np.abs(ref_u).max(), 1e-3), (name, k)
    s.close()


@pytest.mark.parametrize('name', ['walls_guo_d2e4', 'inout_sc_d2e4_t09', 'periodic_sc_d2e6_t12'])
def test_dropin_simple_loops(name):
    sp = pytest.importorskip('sympy')
    z, c = load(name)
    n = sp.Symbol('n')
    sc = ShanChenMultiPhase(lang='cuda', dim_sizes=tuple(c['dims']), xi_stencil=XIStencils[c['xi']],
                            f_stencil=FStencils[c['fs']], psi_code='exp(-1./ln)', psi_sym=sp.exp(-1 / n),
                            SC_G=c['G'], tau=c['tau'])
    sc.verbose = False
    sc.sims_idpy_memory['n'].H2D(z['n_init'].ravel())
    sc.sims_idpy_memory['u'].SetConst(0.0)
    sc.init_status['n'] = sc.init_status['u'] = True
    sc.InitPopulations()
    if 'walls' in z.files:
        sc.GetWalls(z['walls'], z['psi_w'])
    sc.sims_idpy_memory['n'].H2D(z['n_init'].ravel())
    live = (z['walls'] != 0) if 'walls' in z.files else np.ones(z['n_init'].shape, bool)
    kw = {'u_in': c['u_in']} if 'InletOutlet' in c['loop'] else {}
    done = 0
    for k in z['steps']:
        getattr(sc, c['loop'])([0, int(k) - done], **kw)
        done = int(k)
        assert rel_err(sc.GetPopulations()[:, live], z['pop_%d' % k][:, live]) < 1e-12, (name, k)
        assert rel_err(sc.GetDensityField()[live], z['n_%d' % k][live]) < 1e-12, (name, k)
    # the generated-kernel step takes over again
    sc.MainLoop([0, 2])
    assert np.isfinite(sc.GetDensityField()).all()
    sc.End()


def test_simple_refusals():
    z, c = load('walls_guo_d2e4')
    x, f = XIStencils[c['xi']], FStencils[c['fs']]
    s = _lib.Sim(2, c['dims'], x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], c['G'])
    with pytest.raises(_lib.SclbmError):
        s.set_simple(_lib.SIMPLE_GUO, use_walls=True)   # no walls yet
    with pytest.raises(_lib.SclbmError):
        s.set_simple(_lib.SIMPLE_SC, gravity=1e-5)      # gravity goes with Guo
    s.close()


@pytest.mark.parametrize('name', CASES)
def test_simple_fp32_follows_reference(name):
    """The FP32-shifted simple kernels (the same formulas on g = f - w rho0,
    rest population from mass conservation): density within 1e-3 of the
    reference's FP64 run on every non-wall cell at the last checkpoint; total
    mass conserved to FP32 rounding where the loop has no inlet/outlet."""
    z, c = load(name)
    x, f = XIStencils[c['xi']], FStencils[c['fs']]
    D = len(c['dims'])
    s = _lib.Sim(D, c['dims'], x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], c['G'], tau=c['tau'],
                 precision=_lib.FP32_SHIFTED, rho0=float(z['n_init'].min()))
    has_walls = 'walls' in z.files
    if has_walls:
        s.set_walls(z['walls'], z['psi_w'])
    s.set_populations(z['pop_init'])
    s.set_density(z['n_init'])
    s.set_velocity(np.zeros(D * s.V))
    forcing, g, u_in = kind(c)
    s.set_simple(_lib.SIMPLE_SC if forcing == 'sc' else _lib.SIMPLE_GUO, use_walls=has_walls, gravity=g,
                 inlet_outlet=u_in is not None, u_in=u_in or 0.0)
    m0, _ = s.reductions()
    k = int(z['steps'][-1])
    s.step(k)
    live = (z['walls'] != 0).ravel() if has_walls else np.ones(s.V, bool)
    assert rel_err(s.get_density()[live], z['n_%d' % k].ravel()[live]) < 1e-3, name
    if u_in is None:
        m1, _ = s.reductions()
        assert abs(m1 - m0) / m0 < 1e-5, name
    s.close()
