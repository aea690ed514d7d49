"""Generate the golden fixtures for the Shan-Chen step from the reference itself.

This script imports the reference implementation (lullimat/idea.deploy, package
``idpy``) from a checkout given by ``--reference`` and runs its CTypes FP64 path
(``ShanChenMultiPhase(lang=CTYPES_T)``, gcc ``-std=c99 -O3``, serial loop) on
small seeded cases.  It writes one ``<case>.npz`` per case into this directory.
The fixtures pin the CPU oracle under ``oracle/`` and, through it, the CUDA
path; nothing at test time imports the reference.

What is recorded per case (all FP64):
  * ``n_init``          initial density field (tanh droplet x seeded noise)
  * ``pop_init``        populations after ``InitPopulations`` (SoA, (Q, *flip(dims)))
  * ``pop_step1``       populations after one ``MainLoop`` step (SoA)
  * ``n_<k>``, ``u_<k>`` density and Guo-shifted velocity after ``k`` steps
                        (``ComputeMomentsMeta``; u as (D, *flip(dims)))
  * ``mass_<k>``        sum of all populations after ``k`` steps
  * ``uconv``, ``maxu`` ``CheckUConvergenceSCMP`` values at each checkpoint
  * ``dp``              ``DeltaPLaplace()`` after the last checkpoint
  * ``lit_json``        the coefficient literals of the generated collision
                        kernel, one dict per population: monomial -> literal

The reference needs five modules that are absent here and unused on this path
(h5py, matplotlib, IPython, dill, multiprocess); empty stand-ins are written to
a temporary directory and put on ``sys.path`` first.

Usage:
    python tests/golden/make_golden.py --reference /path/to/idea.deploy [case ...]
"""
import argparse
import contextlib
import glob
import io
import json
import os
import re
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

STUBS = {
    'h5py.py': '',
    'dill.py': '',
    'multiprocess.py': '',
    'matplotlib/__init__.py': '',
    'matplotlib/pyplot.py': 'def figure(*a, **k):\n    pass\n',
    'IPython/__init__.py': '',
    'IPython/display.py': 'def display(*a, **k):\n    pass\nMath = Latex = display\n',
}

# Each case: lattice, force stencil, collision, tau, G, psi, dims (x first),
# droplet radius, rho_l, rho_g, tanh width, checkpoints, MRT rates (or None)
CASES = {
    'd2e4_bgk_t1': dict(xi='D2Q9', fs='D2E4', tau=1.0, G=-4.5, psi='exp', dims=(40, 32),
                        R=10.0, rl=4.5625, rg=0.2086, width=2.0, steps=[1, 10, 100, 1000]),
    'd2e8_bgk_t08': dict(xi='D2Q9', fs='D2E8', tau=0.8, G=-4.5, psi='exp', dims=(36, 44),
                         R=9.0, rl=4.646, rg=0.204, width=2.0, steps=[1, 100, 1000]),
    'd2e6_bgk_t12_psi1mexp': dict(xi='D2Q9', fs='D2E6', tau=1.2, G=-1.6, psi='1mexp',
                                  dims=(32, 32), R=8.0, rl=1.736, rg=0.1595, width=2.0,
                                  steps=[1, 100, 1000]),
    'd2e4_mrt': dict(xi='D2Q9', fs='D2E4', tau=1.0, G=-4.5, psi='exp', dims=(40, 32),
                     R=10.0, rl=4.5625, rg=0.2086, width=2.0, steps=[1, 100, 1000],
                     rates=[1.0, 1.0, 1.0, 1.2, 1.25, 1.3, 1.1, 0.9, 1.4]),
    'd3e6_bgk_t1': dict(xi='D3Q19', fs='D3E6', tau=1.0, G=-4.5, psi='exp', dims=(20, 18, 16),
                        R=5.0, rl=4.636, rg=0.147, width=2.0, steps=[1, 100, 1000]),
    'd3e4_bgk_t09': dict(xi='D3Q19', fs='D3E4', tau=0.9, G=-4.5, psi='exp', dims=(16, 16, 16),
                         R=5.0, rl=4.5, rg=0.21, width=2.0, steps=[1, 100]),
    'd3e8_bgk_t1': dict(xi='D3Q19', fs='D3E8', tau=1.0, G=-4.5, psi='exp', dims=(16, 14, 18),
                        R=4.0, rl=4.6, rg=0.16, width=2.0, steps=[1, 50]),
    'd3e6_mrt_ones': dict(xi='D3Q19', fs='D3E6', tau=1.0, G=-4.5, psi='exp', dims=(16, 16, 16),
                          R=5.0, rl=4.636, rg=0.147, width=2.0, steps=[1, 100],
                          rates=[1.0] * 19),
    'd3e6_mrt_rates': dict(xi='D3Q19', fs='D3E6', tau=1.0, G=-4.5, psi='exp', dims=(12, 14, 16),
                           R=4.0, rl=4.636, rg=0.147, width=2.0, steps=[1, 50],
                           rates=[1.0, 1.0, 1.0, 1.0, 1.1, 1.2, 1.15, 1.25, 1.3, 1.05,
                                  1.4, 1.35, 1.3, 1.45, 1.5, 1.2, 1.1, 1.6, 1.7]),
}

# The configuration the reference's 2D headline is quoted on, as written
# (G=-5, rho_l=2.2, rho_g=0.15): it diverges; record per-step extrema.
DIVERGENCE = dict(xi='D2Q9', fs='D2E4', tau=1.0, G=-5.0, psi='exp', dims=(256, 256),
                  R=48.0, rl=2.2, rg=0.15, width=2.0, nsteps=40)

# Its stable twin at full size (G=-4.5): scalar summaries only.
FULL_TWIN = dict(xi='D2Q9', fs='D2E4', tau=1.0, G=-4.5, psi='exp', dims=(256, 256),
                 R=48.0, rl=4.5625, rg=0.2086, width=2.0, steps=[1000, 10000])

# The 3D headline's shape at a size the reference runs in minutes: D3Q19, E6,
# MRT with every rate 1.0, a droplet in a 64^3 box at the stable coupling
# G = -4.5 with the 3D E6 flat-interface densities; 1000 steps.  The radius is
# 16: a droplet of the headline's proportion (R = 10 here for R = 40 in 256^3)
# evaporates completely into the small box within 1000 steps (the gas has to
# take up the Laplace excess, and a small box has too little of it), which
# would leave a uniform gas to compare.  Compact records (summaries, per-plane
# sums, two central planes of n and u) keep the fixture small.
CFG2_64 = dict(xi='D3Q19', fs='D3E6', tau=1.0, G=-4.5, psi='exp', dims=(64, 64, 64),
               R=16.0, rl=4.636, rg=0.147, width=2.0, steps=[100, 1000], rates=[1.0] * 19)

# A flat-interface (slab) run of the reference at a coupling where it settles:
# D2Q9, E4, G = -4.5, tau = 1, a 64 x 4 periodic box with a liquid slab of
# width 32 from the reference's own InitFlatInterface (n_g = 0.2, n_l = 4.55);
# the run reaches u_conv < 1e-12 by about 70,000 steps.  During the transient
# the slab may drift along x (any position is an equilibrium; round-off
# breaks the symmetry), so only the early checkpoint pins the whole profile
# and the settled one pins the bulk densities.
FLAT_E4 = dict(xi='D2Q9', fs='D2E4', tau=1.0, G=-4.5, psi='exp', dims=(64, 4), n_g=0.2, n_l=4.55, width=32.0,
               steps=[1000, 10000, 40000, 70000])

SEED = 1234


def setup_reference(ref):
    tmp = tempfile.mkdtemp(prefix='idpy_stubs_')
    for rel, body in STUBS.items():
        p = os.path.join(tmp, rel)
        os.makedirs(os.path.dirname(p), exist_ok=True)
        with open(p, 'w') as f:
            f.write(body)
    sys.path.insert(0, ref)
    sys.path.insert(0, tmp)
    sys.dont_write_bytecode = True
    import warnings
    warnings.filterwarnings('ignore')


def droplet(dims, R, rl, rg, width, seed=SEED, noise=1e-4):
    """tanh droplet about L//2 with multiplicative seeded noise (x fastest)."""
    grids = np.meshgrid(*[np.arange(L) for L in reversed(dims)], indexing='ij')
    # grids[-1] is x, grids[-2] is y, ...
    r2 = np.zeros(grids[0].shape)
    for d, L in enumerate(dims):
        r2 += (grids[len(dims) - 1 - d] - L // 2) ** 2
    r = np.sqrt(r2)
    rho = 0.5 * (rl + rg) - 0.5 * (rl - rg) * np.tanh((r - R) / width)
    rng = np.random.default_rng(seed)
    rho = rho * (1.0 + noise * rng.uniform(-1.0, 1.0, rho.shape))
    return rho


def make_sim(c):
    import sympy as sp
    from idpy.IdpyCode import CTYPES_T
    from idpy.LBM.MultiPhase import ShanChenMultiPhase
    from idpy.LBM.LBM import XIStencils, FStencils
    n = sp.Symbol('n')
    if c['psi'] == 'exp':
        psi_code, psi_sym = 'exp(-1./ln_0)', sp.exp(-1 / n)
    else:
        psi_code, psi_sym = '(1. - exp(-ln_0))', 1 - sp.exp(-n)
    with contextlib.redirect_stdout(io.StringIO()):
        sc = ShanChenMultiPhase(lang=CTYPES_T, dim_sizes=tuple(c['dims']),
                                xi_stencil=XIStencils[c['xi']], f_stencil=FStencils[c['fs']],
                                psi_code=psi_code, psi_sym=psi_sym, SC_G=c['G'], tau=c['tau'])
    return sc


def set_fields(sc, rho):
    sc.sims_idpy_memory['n'].H2D(np.ascontiguousarray(rho.ravel()))
    sc.sims_idpy_memory['u'].SetConst(0.)
    sc.init_status['n'] = sc.init_status['u'] = True
    sc.InitPopulations()


def aos_to_soa(pop, Q, dims):
    return pop.reshape(-1, Q).T.reshape((Q,) + tuple(reversed(dims))).copy()


def mrt_args(c):
    import sympy as sp
    from idpy.LBM.LBM import XIStencils
    from idpy.LBM.Collisions import RelaxationMatrix
    from idpy.LBM.Equilibria import HermiteEquilibria
    eq = HermiteEquilibria(XIStencils[c['xi']])
    rm = RelaxationMatrix(eq)
    Q = len(c['rates'])
    syms = [sp.Symbol('\\omega_%d' % i) for i in range(Q)]
    S = rm.GetDiagonalMatrix(syms)
    return dict(relaxation_matrix=S, omega_syms_vals=list(zip(syms, c['rates'])))


def run_loop(sc, c, steps, fn):
    with contextlib.redirect_stdout(io.StringIO()):
        if c.get('rates') is None:
            sc.MainLoop([0] + list(steps), convergence_functions=[fn])
        else:
            sc.MainLoopMRT([0] + list(steps), convergence_functions=[fn], **mrt_args(c))


def parse_literals(kernel_name, c):
    """Coefficient literals of the generated kernel called kernel_name whose
    macros match this case (several cases may share the kernel cache)."""
    V = int(np.prod(c['dims']))
    want = ['#define V %d\n' % V, '#define L_0 %d\n' % c['dims'][0],
            '#define OMEGA %r\n' % (1. / c['tau']), '#define SC_G %r\n' % c['G']]
    files = sorted(glob.glob('/tmp/idpy_ctypes_kernels/*.c'), key=os.path.getmtime)
    src = None
    for f in reversed(files):
        s = open(f).read()
        if ('int ' + kernel_name + '(') in s and all(w in s for w in want):
            src = s
            break
    if src is None:
        raise RuntimeError('generated kernel not found for ' + kernel_name)
    out = {}
    for m in re.finditer(r'\(\*\(pop_swap \+ (\d+) \+ x_dst \* Q\)\) = (.*?);', src):
        q, expr = int(m.group(1)), m.group(2)
        terms = {}
        for tm in re.finditer(r'([+-]?)\s*(\d[0-9.eE+-]*)\*([A-Za-z_][A-Za-z0-9_*]*)', expr):
            sign, lit, mono = tm.groups()
            terms[mono] = ('-' if sign == '-' else '') + lit
        out[q] = terms
    return out


def gen_case(name, c):
    t0 = time.time()
    sc = make_sim(c)
    Q = 9 if c['xi'] == 'D2Q9' else 19
    D = len(c['dims'])
    rho = droplet(c['dims'], c['R'], c['rl'], c['rg'], c['width'])
    set_fields(sc, rho)
    rec = dict(n_init=rho.copy(),
               pop_init=aos_to_soa(sc.sims_idpy_memory['pop'].D2H(), Q, c['dims']))
    from idpy.LBM.MultiPhaseLoopChecks import CheckUConvergenceSCMP
    state = dict(k=0, uconv=[], maxu=[])
    steps = list(c['steps'])

    def recorder(lbm):
        k = steps[state['k']]
        state['k'] += 1
        lbm.ComputeMomentsMeta()
        rec['n_%d' % k] = lbm.GetDensityField().copy()
        u = lbm.sims_idpy_memory['u'].D2H().reshape(-1, D)
        rec['u_%d' % k] = u.T.reshape((D,) + tuple(reversed(c['dims']))).copy()
        rec['mass_%d' % k] = float(lbm.sims_idpy_memory['pop'].D2H().sum())
        if k == 1:
            rec['pop_step1'] = aos_to_soa(lbm.sims_idpy_memory['pop'].D2H(), Q, c['dims'])
        with contextlib.redirect_stdout(io.StringIO()):
            CheckUConvergenceSCMP(lbm)
        state['uconv'].append(lbm.sims_vars['u_conv'][-1])
        state['maxu'].append(lbm.sims_vars['max_u'][-1])
        return False

    run_loop(sc, c, steps, recorder)
    with contextlib.redirect_stdout(io.StringIO()):
        sc.ComputeMomentsMeta()
        dp = sc.DeltaPLaplace()
    rec['dp'] = np.array(dp, dtype=np.float64)
    rec['uconv'] = np.array(state['uconv'])
    rec['maxu'] = np.array(state['maxu'])
    kname = 'K_ForceCollideStreamSCMPMeta' if c.get('rates') is None else \
        'K_ForceCollideStreamSCMP_MRTMeta'
    rec['lit_json'] = np.array(json.dumps(parse_literals(kname, c)))
    rec['config_json'] = np.array(json.dumps(dict(c, seed=SEED)))
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **rec)
    print(name, 'done in %.1f s' % (time.time() - t0), flush=True)


def gen_divergence():
    c = DIVERGENCE
    t0 = time.time()
    sc = make_sim(c)
    rho = droplet(c['dims'], c['R'], c['rl'], c['rg'], c['width'])
    set_fields(sc, rho)
    Q = 9
    stats = []

    def rec(lbm):
        pop = lbm.sims_idpy_memory['pop'].D2H().reshape(-1, Q)
        nn = pop.sum(axis=1)
        with np.errstate(all='ignore'):
            stats.append([np.nanmax(nn), np.nanmin(nn), float(np.isfinite(nn).all())])
        return False

    run_loop(sc, c, list(range(1, c['nsteps'] + 1)), rec)
    np.savez_compressed(os.path.join(HERE, 'div_cfg1.npz'), stats=np.array(stats),
                        config_json=np.array(json.dumps(dict(c, seed=SEED))))
    print('div_cfg1 done in %.1f s' % (time.time() - t0), flush=True)


def gen_full_twin():
    c = FULL_TWIN
    t0 = time.time()
    sc = make_sim(c)
    rho = droplet(c['dims'], c['R'], c['rl'], c['rg'], c['width'])
    set_fields(sc, rho)
    rec = {'mass_0': float(sc.sims_idpy_memory['pop'].D2H().sum())}
    steps = list(c['steps'])
    state = dict(k=0)
    L = c['dims'][0]

    def recorder(lbm):
        k = steps[state['k']]
        state['k'] += 1
        lbm.ComputeMomentsMeta()
        n = lbm.GetDensityField()
        u = lbm.sims_idpy_memory['u'].D2H().reshape(-1, 2)
        rec['mass_%d' % k] = float(lbm.sims_idpy_memory['pop'].D2H().sum())
        rec['nsum_%d' % k] = float(n.sum())
        rec['nmax_%d' % k] = float(n.max())
        rec['nmin_%d' % k] = float(n.min())
        rec['umax_%d' % k] = float(np.abs(u).max())
        rec['row_%d' % k] = n[L // 2, :].copy()
        rec['col_%d' % k] = n[:, L // 2].copy()
        rec['urow_%d' % k] = u.reshape(L, L, 2)[L // 2 + 20, :, :].copy()
        return False

    run_loop(sc, c, steps, recorder)
    np.savez_compressed(os.path.join(HERE, 'full_twin_256.npz'), **rec,
                        config_json=np.array(json.dumps(dict(c, seed=SEED))))
    print('full_twin done in %.1f s' % (time.time() - t0), flush=True)


def gen_cfg2_64():
    c = CFG2_64
    t0 = time.time()
    sc = make_sim(c)
    rho = droplet(c['dims'], c['R'], c['rl'], c['rg'], c['width'])
    set_fields(sc, rho)
    rec = {'mass_0': float(sc.sims_idpy_memory['pop'].D2H().sum())}
    steps = list(c['steps'])
    state = dict(k=0)
    L = c['dims'][0]
    from idpy.LBM.MultiPhaseLoopChecks import CheckUConvergenceSCMP

    def recorder(lbm):
        k = steps[state['k']]
        state['k'] += 1
        lbm.ComputeMomentsMeta()
        n = lbm.GetDensityField()                                  # (z, y, x)
        u = lbm.sims_idpy_memory['u'].D2H().reshape(L, L, L, 3)    # (z, y, x, d)
        rec['mass_%d' % k] = float(lbm.sims_idpy_memory['pop'].D2H().sum())
        rec['nsum_%d' % k] = float(n.sum())
        rec['nmax_%d' % k] = float(n.max())
        rec['nmin_%d' % k] = float(n.min())
        rec['umax_%d' % k] = float(np.abs(u).max())
        rec['nplane_%d' % k] = n.sum(axis=(1, 2)).copy()          # per z plane
        rec['nz_%d' % k] = n[L // 2].copy()                        # plane z = L/2
        rec['nx_%d' % k] = n[:, :, L // 2 + 3].copy()              # plane x = L/2 + 3
        rec['uz_%d' % k] = u[L // 2].copy()
        rec['ux_%d' % k] = u[:, :, L // 2 + 3].copy()
        with contextlib.redirect_stdout(io.StringIO()):
            CheckUConvergenceSCMP(lbm)
        rec['uconv_%d' % k] = float(lbm.sims_vars['u_conv'][-1])
        rec['maxu_%d' % k] = float(lbm.sims_vars['max_u'][-1])
        return False

    run_loop(sc, c, steps, recorder)
    with contextlib.redirect_stdout(io.StringIO()):
        sc.ComputeMomentsMeta()
        dp = sc.DeltaPLaplace()
    rec['dp'] = np.array(dp, dtype=np.float64)
    rec['seconds'] = time.time() - t0
    rec['lit_json'] = np.array(json.dumps(parse_literals('K_ForceCollideStreamSCMP_MRTMeta', c)))
    np.savez_compressed(os.path.join(HERE, 'cfg2_64.npz'), **rec,
                        config_json=np.array(json.dumps(dict(c, seed=SEED))))
    print('cfg2_64 done in %.1f s' % (time.time() - t0), flush=True)


def gen_flat_e4():
    c = FLAT_E4
    t0 = time.time()
    sc = make_sim(c)
    with contextlib.redirect_stdout(io.StringIO()):
        sc.InitFlatInterface(n_g=c['n_g'], n_l=c['n_l'], width=c['width'], direction=0)
    rec = {'n_init': sc.GetDensityField().copy()}
    steps = list(c['steps'])
    state = dict(k=0)
    from idpy.LBM.MultiPhaseLoopChecks import CheckUConvergenceSCMP

    def recorder(lbm):
        k = steps[state['k']]
        state['k'] += 1
        lbm.ComputeMomentsMeta()
        n = lbm.GetDensityField()
        rec['n_%d' % k] = n.copy()
        rec['umax_%d' % k] = float(np.abs(lbm.sims_idpy_memory['u'].D2H()).max())
        with contextlib.redirect_stdout(io.StringIO()):
            CheckUConvergenceSCMP(lbm)
        rec['uconv_%d' % k] = float(lbm.sims_vars['u_conv'][-1])
        return False

    with contextlib.redirect_stdout(io.StringIO()):
        sc.MainLoop([0] + steps, convergence_functions=[recorder])
    np.savez_compressed(os.path.join(HERE, 'flat_e4_g45.npz'), **rec,
                        config_json=np.array(json.dumps(c)))
    print('flat_e4_g45 done in %.1f s' % (time.time() - t0), flush=True)


def gen_init_profiles():
    """The reference's own interface-initialisation kernels (width 1)."""
    rec = {}
    for tag, xi, fs, dims in [('2d', 'D2Q9', 'D2E4', (40, 32)), ('3d', 'D3Q19', 'D3E4', (12, 10, 8))]:
        c = dict(xi=xi, fs=fs, tau=1.0, G=-4.5, psi='exp', dims=dims)
        sc = make_sim(c)
        with contextlib.redirect_stdout(io.StringIO()):
            sc.InitRadialInterface(n_g=0.15, n_l=2.2, R=dims[0] / 4.0, full_flag=True)
        rec['radial_' + tag] = sc.GetDensityField().copy()
        rec['radial_pop_' + tag] = sc.sims_idpy_memory['pop'].D2H().copy()
        with contextlib.redirect_stdout(io.StringIO()):
            sc.InitRadialInterface(n_g=0.15, n_l=2.2, R=dims[0] / 4.0, full_flag=False)
        rec['radial_inv_' + tag] = sc.GetDensityField().copy()
        with contextlib.redirect_stdout(io.StringIO()):
            sc.InitFlatInterface(n_g=0.2, n_l=4.5, width=dims[0] / 2.0, direction=0)
        rec['flat_' + tag] = sc.GetDensityField().copy()
        with contextlib.redirect_stdout(io.StringIO()):
            sc.InitFlatInterface(n_g=0.2, n_l=4.5, width=dims[1] / 3.0, direction=1)
        rec['flat_d1_' + tag] = sc.GetDensityField().copy()
        with contextlib.redirect_stdout(io.StringIO()):
            sc.InitSingleFlatInterface(n_g=0.2, n_l=4.5, direction=0)
        rec['single_flat_' + tag] = sc.GetDensityField().copy()
        if tag == '3d':
            with contextlib.redirect_stdout(io.StringIO()):
                sc.InitCylinderInterface(n_g=0.2, n_l=4.5, R=3.0, direction=2)
            rec['cylinder_' + tag] = sc.GetDensityField().copy()
    np.savez_compressed(os.path.join(HERE, 'init_profiles.npz'), **rec)
    print('init_profiles done', flush=True)


def gen_mrt_basis():
    """The reference's Hermite moment bases (invertible set and its W-orthogonal form)."""
    from idpy.LBM.LBM import XIStencils
    from idpy.LBM.Equilibria import HermiteEquilibria
    rec = {}
    for xi in ['D2Q9', 'D3Q19']:
        eq = HermiteEquilibria(XIStencils[xi])
        st = eq.idpy_stencil
        Mw = st.GetWOrthInvertibleHermiteSet(search_depth=6)['MWOrth']
        Mn = st.GetInvertibleHermiteSet(search_depth=6)['M']
        rec['MWOrth_' + xi] = np.array(Mw.evalf(), dtype=np.float64)
        rec['M_' + xi] = np.array(Mn.evalf(), dtype=np.float64)
        rec['tuples_' + xi] = np.array(json.dumps([str(t) for t in st.MTaylorTuples]))
    from idpy.LBM.LBM import FStencils
    tables = {'XIStencils': {k: {kk: list(vv) if isinstance(vv, tuple) else vv
                                 for kk, vv in XIStencils[k].items()} for k in ['D2Q9', 'D3Q19']},
              'FStencils': {k: {kk: list(vv) for kk, vv in FStencils[k].items()}
                            for k in ['D2E4', 'D2E6', 'D2E8', 'D3E4', 'D3E6', 'D3E8']}}
    rec['tables_json'] = np.array(json.dumps(tables))
    np.savez_compressed(os.path.join(HERE, 'mrt_basis.npz'), **rec)
    print('mrt_basis done', flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--reference', required=True)
    ap.add_argument('cases', nargs='*')
    a = ap.parse_args()
    setup_reference(os.path.abspath(a.reference))
    todo = a.cases or (list(CASES) + ['div_cfg1', 'full_twin_256', 'cfg2_64', 'flat_e4_g45', 'init_profiles',
                                       'mrt_basis'])
    for name in todo:
        if name in CASES:
            gen_case(name, CASES[name])
        elif name == 'div_cfg1':
            gen_divergence()
        elif name == 'full_twin_256':
            gen_full_twin()
        elif name == 'cfg2_64':
            gen_cfg2_64()
        elif name == 'flat_e4_g45':
            gen_flat_e4()
        elif name == 'init_profiles':
            gen_init_profiles()
        elif name == 'mrt_basis':
            gen_mrt_basis()
        else:
            raise SystemExit('unknown case ' + name)


if __name__ == '__main__':
    main()
