"""Generate fixtures of the reference's "simple" step family from the reference itself.

The loops MainLoopSimple, MainLoopSimpleSC, MainLoopSimpleWalls,
MainLoopSimpleWallsSC, MainLoopSimpleWallsGravity,
MainLoopSimpleWallsInletOutlet and MainLoopSimpleWallsInletOutletSC
(idpy/LBM/MultiPhase.py:164-1014) run hand-written kernels
(idpy/LBM/MultiPhaseKernels.py:132-604, idpy/LBM/LBMKernels.py:117-258,299-456):
inlet / outlet setters, moments and psi on flagged cells, an in-place
collision (Guo forcing, the original Shan-Chen velocity shift, or Guo forcing
with gravity along y), a periodic pull stream and halfway bounce-back out of
the wall cells.  Those kernels index every array q-major (g + q*V), so the
runs here use the CTypes backend with ``set_ordering='gpu'``; psi is given on
``ln`` as those kernels name the density.

Writes ``simple_<case>.npz`` into this directory:
  * ``walls``, ``psi_w``  flags (1 fluid, 0 wall, 2 inlet, 3 outlet) and the
                          psi given to GetWalls (absent for the periodic loops)
  * ``n_init``, ``pop_init``  initial density and populations (SoA)
  * ``pop_<k>``, ``n_<k>``, ``u_<k>``, ``psi_<k>``  the reference's arrays after
                          k steps ((Q | D, *flip(dims)))
  * ``config_json``       the case

Nothing at test time imports the reference.

Usage:
    python tests/golden/make_golden_simple.py --reference /path/to/idea.deploy [case ...]
"""
import argparse
import contextlib
import io
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as mg  # noqa: E402

CASES = {
    # periodic droplet, Guo forcing / Shan-Chen velocity shift
    'periodic_guo_d3e4': dict(loop='MainLoopSimple', xi='D3Q19', fs='D3E4', tau=1.0, G=-4.5, dims=(14, 12, 10),
                              R=3.5, rl=4.5, rg=0.21, geometry=None, steps=[1, 40]),
    'periodic_sc_d2e6_t12': dict(loop='MainLoopSimpleSC', xi='D2Q9', fs='D2E6', tau=1.2, G=-4.5, dims=(32, 28),
                                 R=7.0, rl=4.6, rg=0.2, geometry=None, steps=[1, 100, 500]),
    # droplet resting on the lower wall of a channel
    'walls_guo_d2e4': dict(loop='MainLoopSimpleWalls', xi='D2Q9', fs='D2E4', tau=1.0, G=-4.5, dims=(40, 28),
                           R=7.0, rl=4.5625, rg=0.2086, geometry='channel', centre_y=7.0, n_wall=2.0,
                           steps=[1, 100, 500]),
    'walls_sc_d2e8_t08': dict(loop='MainLoopSimpleWallsSC', xi='D2Q9', fs='D2E8', tau=0.8, G=-4.5, dims=(36, 30),
                              R=6.0, rl=4.646, rg=0.204, geometry='channel2', centre_y=8.0, n_wall=1.5,
                              steps=[1, 100, 500]),
    # MainLoopSimpleWallsGravity runs its loop on a merged copy of the memory
    # dicts (to add g, MultiPhase.py:937-947): the buffer swap stays in the copy,
    # so after an odd number of steps the next call starts from the stale
    # populations.  Its checkpoints here are even.
    'gravity_d2e6': dict(loop='MainLoopSimpleWallsGravity', xi='D2Q9', fs='D2E6', tau=1.0, G=-4.5, dims=(32, 36),
                         R=6.0, rl=4.6, rg=0.2, geometry='channel', centre_y=14.0, n_wall=1.0, g=-2e-5,
                         steps=[2, 100, 300]),
    'walls_guo_d3e6': dict(loop='MainLoopSimpleWalls', xi='D3Q19', fs='D3E6', tau=0.9, G=-4.5, dims=(14, 12, 12),
                           R=3.5, rl=4.636, rg=0.147, geometry='channel', centre_y=4.0, n_wall=2.0, steps=[1, 30]),
    # channel with an inlet column at x = 0 and an outlet column at x = Lx - 1.
    # Only the Shan-Chen-forcing loop runs: MainLoopSimpleWallsInletOutlet builds
    # its inlet kernel without the position helpers it calls (MultiPhase.py:600-604),
    # so the reference cannot load it (undefined symbol F_PosFromIndex).  Both
    # loops pass 'idloop_k' to the inlet kernel without putting it in the memory
    # dict (IdpyLoop only updates an existing key, IdpyCode.py:1731): the run
    # here adds sims_idpy_memory['idloop_k'] = 0 first (the kernel does not read it).
    'inout_sc_d2e4_t09': dict(loop='MainLoopSimpleWallsInletOutletSC', xi='D2Q9', fs='D2E4', tau=0.9, G=-3.5,
                              dims=(40, 18), R=0.0, rl=2.0, rg=2.0, geometry='inout', n_wall=2.0, u_in=0.015,
                              steps=[1, 100, 500]),
}


def make_sim(c):
    import sympy as sp
    from idpy.IdpyCode import CTYPES_T
    from idpy.LBM.MultiPhase import ShanChenMultiPhase
    from idpy.LBM.LBM import XIStencils, FStencils
    n = sp.Symbol('n')
    with contextlib.redirect_stdout(io.StringIO()):
        sc = ShanChenMultiPhase(lang=CTYPES_T, dim_sizes=tuple(c['dims']), xi_stencil=XIStencils[c['xi']],
                                f_stencil=FStencils[c['fs']], psi_code='exp(-1./ln)', psi_sym=sp.exp(-1 / n),
                                SC_G=c['G'], tau=c['tau'], set_ordering='gpu')
    return sc


def fields(c):
    dims = c['dims']
    D = len(dims)
    shape = tuple(reversed(dims))
    grids = np.meshgrid(*[np.arange(L) for L in reversed(dims)], indexing='ij')
    rng = np.random.default_rng(mg.SEED)
    if c['R'] > 0:
        centre = [L // 2 for L in dims]
        if c['geometry'] is not None:
            centre[1] = c['centre_y']
        r2 = np.zeros(shape)
        for d in range(D):
            r2 += (grids[D - 1 - d] - centre[d]) ** 2
        r = np.sqrt(r2)
        rho = 0.5 * (c['rl'] + c['rg']) - 0.5 * (c['rl'] - c['rg']) * np.tanh((r - c['R']) / 2.0)
    else:
        rho = np.full(shape, c['rl'])
    rho = rho * (1.0 + 1e-4 * rng.uniform(-1.0, 1.0, shape))
    walls = np.ones(shape, np.int32)
    yax = D - 2      # array axis of y
    if c['geometry'] in ('channel', 'inout', 'channel2'):
        w = 2 if c['geometry'] == 'channel2' else 1
        sl = [slice(None)] * D
        sl[yax] = slice(0, w)
        walls[tuple(sl)] = 0
        sl[yax] = slice(-w, None)
        walls[tuple(sl)] = 0
    if c['geometry'] == 'inout':
        fluid_rows = walls[..., 0] != 0
        walls[..., 0][fluid_rows] = 2
        walls[..., -1][fluid_rows] = 3
    psi_w = np.full(shape, np.exp(-1.0 / c.get('n_wall', 1.0)))
    return rho, walls, psi_w


def run(sc, c, k):
    kw = {}
    if 'InletOutlet' in c['loop'] and 'idloop_k' not in sc.sims_idpy_memory:
        sc.sims_idpy_memory['idloop_k'] = np.int32(0)
    if 'Gravity' in c['loop']:
        kw['g'] = c['g']
    if 'InletOutlet' in c['loop']:
        kw['u_in'] = c['u_in']
    with contextlib.redirect_stdout(io.StringIO()):
        getattr(sc, c['loop'])([0, k], **kw)


def gen_case(name, c):
    t0 = time.time()
    sc = make_sim(c)
    Q = 9 if c['xi'] == 'D2Q9' else 19
    D = len(c['dims'])
    shape = tuple(reversed(c['dims']))
    rho, walls, psi_w = fields(c)
    mg.set_fields(sc, rho)
    out = dict(n_init=rho, pop_init=sc.sims_idpy_memory['pop'].D2H().reshape((Q,) + shape))
    if c['geometry'] is not None:
        with contextlib.redirect_stdout(io.StringIO()):
            sc.GetWalls(walls, psi_w)
        out.update(walls=walls, psi_w=psi_w)
    done = 0
    for k in c['steps']:
        run(sc, c, k - done)
        done = k
        out['pop_%d' % k] = sc.sims_idpy_memory['pop'].D2H().reshape((Q,) + shape)
        out['n_%d' % k] = sc.sims_idpy_memory['n'].D2H().reshape(shape)
        out['u_%d' % k] = sc.sims_idpy_memory['u'].D2H().reshape((D,) + shape)
        out['psi_%d' % k] = sc.sims_idpy_memory['psi'].D2H().reshape(shape)
    out['steps'] = np.array(c['steps'])
    out['config_json'] = json.dumps(dict(c, seed=mg.SEED))
    np.savez_compressed(os.path.join(HERE, 'simple_%s.npz' % name), **out)
    print(name, '%.1fs' % (time.time() - t0), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--reference', required=True)
    ap.add_argument('cases', nargs='*')
    a = ap.parse_args()
    mg.setup_reference(os.path.abspath(a.reference))
    for name in (a.cases or list(CASES)):
        gen_case(name, CASES[name])


if __name__ == '__main__':
    main()
