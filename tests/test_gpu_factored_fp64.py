"""The factored FP64 BGK operator (SCLBM_LIT_FACTORED): the same step as the
expanded operator with exact coefficients up to rounding, and as close to the
oracle (the reference's arithmetic restated) as the expanded form is."""
import numpy as np
import pytest

from helpers import rel_err
from oracle import oracle as O
from sclbm import _lib, XIStencils, FStencils, ShanChenMultiPhase, CUDA_T
from sclbm.profiles import droplet

pytestmark = pytest.mark.gpu

CASES = [('D2Q9', 'D2E4', (64, 48), 1.0), ('D2Q9', 'D2E8', (96, 80), 0.8), ('D3Q19', 'D3E6', (32, 24, 20), 1.0),
         ('D3Q19', 'D3E8', (24, 24, 24), 1.2)]


def run(lat, st, dims, tau, lit, steps):
    x, f = XIStencils[lat], FStencils[st]
    s = _lib.Sim(len(dims), dims, x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], -4.6, tau=tau, literals=lit)
    s.set_density(droplet(dims, min(dims) / 4, 4.6, 0.2, 2.0, 3))
    s.set_velocity(np.zeros(len(dims) * s.V))
    s.init_populations()
    s.step(steps)
    s.compute_moments()
    out = s.get_density(), s.get_velocity(), s.get_populations(), s.reductions()[0]
    s.close()
    return out


@pytest.mark.parametrize('lat,st,dims,tau', CASES)
def test_factored_fp64_equals_expanded_up_to_rounding(lat, st, dims, tau):
    ne, ue, pe, me = run(lat, st, dims, tau, _lib.LIT_EXACT, 200)
    nf, uf, pf, mf = run(lat, st, dims, tau, _lib.LIT_FACTORED, 200)
    # one rounding per operation apart, grown by the droplet's own dynamics over
    # 200 steps (the expanded form and the oracle differ by 1e-12 on these boxes)
    assert rel_err(nf, ne) < 1e-12 and rel_err(pf, pe) < 1e-12, (rel_err(nf, ne), rel_err(pf, pe))
    assert rel_err(uf, ue) < 1e-11, rel_err(uf, ue)
    assert abs(mf / me - 1) < 1e-13


@pytest.mark.parametrize('lat,st,dims,tau', CASES[1:3])
def test_factored_fp64_as_close_to_oracle_as_expanded(lat, st, dims, tau):
    x, f = XIStencils[lat], FStencils[st]
    n0 = droplet(dims, min(dims) / 4, 4.6, 0.2, 2.0, 3)
    ora = O.OracleSim(dims, x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], -4.6, tau=tau)
    ora.set_fields(n0)
    ora.init_populations()
    ora.run(200)
    ora.compute_moments()
    ne = run(lat, st, dims, tau, _lib.LIT_EXACT, 200)[0]
    nf = run(lat, st, dims, tau, _lib.LIT_FACTORED, 200)[0]
    ee, ef = rel_err(ne, ora.n), rel_err(nf, ora.n)
    assert ef < 1e-11 and ef < 2 * ee + 1e-14, (ef, ee)


def test_dropin_keyword_factored():
    sc = ShanChenMultiPhase(lang=CUDA_T, dim_sizes=(64, 48), xi_stencil=XIStencils['D2Q9'],
                            f_stencil=FStencils['D2E4'], psi_code='exp(-1./ln_0)', psi_sym=None, SC_G=-4.5,
                            tau=1.0, literals='factored')
    sc.InitRadialInterface(n_g=0.2086, n_l=4.5625, R=12)
    sc.MainLoop([0, 100])
    sc.ComputeMomentsMeta()
    assert np.isfinite(sc.GetDensityField()).all()
    sc.End()
