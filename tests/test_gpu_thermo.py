"""Coexistence on the GPU: a flat-interface run against the reference's own run
and against the thermodynamic construction.

The reference's ShanChenMultiPhase settles a liquid slab at D2Q9, E4, G = -4.5
(tests/golden/flat_e4_g45.npz, made by tests/golden/make_golden.py from the
reference's InitFlatInterface and MainLoop, idpy/LBM/MultiPhase.py:1855-1895):
the GPU FP64 path in the reference's arithmetic follows its whole density
field to 1e-12 through the first 1000 steps, and settles (70,000 steps,
max|u| below 1e-11) at the reference's bulk densities to 1e-9.  In between,
the slab may drift along x: every position is an equilibrium, and round-off
(CUDA's exp against glibc's) breaks the symmetry of the start, so positions
are not compared once the transient has grown.  The settled bulk
densities are then compared with the thermodynamic flat-interface construction
of the reference (SCThermo.ShanChen, idpy/LBM/SCThermo.py:157-186,346), which
sclbm.thermo restates: the discrete lattice run and the continuum construction
differ by -0.10 % (liquid) and -1.4 % (gas) in the reference itself, and by
the same amounts here.
"""
import numpy as np
import pytest

from helpers import load, rel_err
from sclbm import ShanChenMultiPhase, XIStencils, FStencils, CUDA_T, thermo

pytestmark = pytest.mark.gpu

ShanChenMultiPhase.verbose = False


def test_flat_interface_follows_reference_and_thermodynamics():
    z, cfg = load('flat_e4_g45')
    sc = ShanChenMultiPhase(lang=CUDA_T, dim_sizes=tuple(cfg['dims']), xi_stencil=XIStencils['D2Q9'],
                            f_stencil=FStencils['D2E4'], psi_code='exp(-1./ln_0)', psi_sym=None, SC_G=cfg['G'],
                            tau=cfg['tau'])
    sc.InitFlatInterface(n_g=cfg['n_g'], n_l=cfg['n_l'], width=cfg['width'], direction=0)
    assert rel_err(sc.GetDensityField(), z['n_init']) <= 1e-15
    sc.MainLoop([0, 1000])
    sc.ComputeMomentsMeta()
    n = sc.GetDensityField()
    assert rel_err(n, z['n_1000']) <= 1e-12, rel_err(n, z['n_1000'])
    sc.MainLoop([0, 69000])
    sc.ComputeMomentsMeta()
    n = sc.GetDensityField()
    u = sc.GetVelocityField()
    assert np.abs(u).max() < 1e-11                      # settled
    n_l, n_g = float(n.max()), float(n.min())
    assert abs(n_l / float(z['n_70000'].max()) - 1) < 1e-9 and abs(n_g / float(z['n_70000'].min()) - 1) < 1e-9
    f = FStencils['D2E4']
    th = thermo.coexistence(cfg['G'], f['Es'], f['Ws'])
    dl, dg = n_l / th['n_l'] - 1, n_g / th['n_g'] - 1
    print('flat E4 G=-4.5: n_l %.10f n_g %.10f; thermodynamics %.10f %.10f; rel %.3e %.3e'
          % (n_l, n_g, th['n_l'], th['n_g'], dl, dg))
    # the reference's own settled slab differs from the construction by these amounts
    ref_l, ref_g = float(z['n_70000'].max()), float(z['n_70000'].min())
    assert abs(dl - (ref_l / th["n_l"] - 1)) < 2e-9 and abs(dg - (ref_g / th["n_g"] - 1)) < 2e-9
    assert -2e-3 < dl < 0 and -2e-2 < dg < 0
    sc.End()
