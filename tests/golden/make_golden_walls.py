"""Generate the wall fixtures from the reference itself.

Runs the reference's CTypes FP64 path with walls (``GetWalls`` +
``MainLoopWalls``, idpy/LBM/MultiPhase.py:157-162,1226-1309: density and psi
on fluid cells only, the fused step on fluid cells only, halfway bounce-back
into the opposite population where the push target is a wall,
idpy/LBM/Collisions.py:705-860) on small channels with a droplet resting on a
wall of given psi, and writes ``walls_<case>.npz`` into this directory:

  * ``walls``        the flag field (1 fluid, 0 wall), shape flip(dims)
  * ``psi_w``        the psi field given to GetWalls (walls keep it)
  * ``n_init``       initial density; ``pop_init`` populations after InitPopulations (SoA)
  * ``pop_<k>``      populations after k steps (SoA, (Q, *flip(dims)))
  * ``n_<k>``        the reference's n array after k steps (density at the start of
                     the last step on fluid cells)

Nothing at test time imports the reference.

Usage:
    python tests/golden/make_golden_walls.py --reference /path/to/idea.deploy [case ...]
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
    # channel in y (one-cell walls at y = 0 and y = Ly - 1), droplet sitting on the lower wall
    'd2e4_bgk_t1': dict(xi='D2Q9', fs='D2E4', tau=1.0, G=-4.5, psi='exp', dims=(48, 32), wall=1,
                        R=8.0, centre=(24.0, 7.0), rl=4.5625, rg=0.2086, n_wall=2.0, steps=[1, 100, 1000]),
    # two-cell walls, the E8 stencil reaches through them
    'd2e8_bgk_t08': dict(xi='D2Q9', fs='D2E8', tau=0.8, G=-4.5, psi='exp', dims=(40, 36), wall=2,
                         R=7.0, centre=(20.0, 8.0), rl=4.646, rg=0.204, n_wall=1.0, steps=[1, 100, 1000]),
    # 3D slab between walls at z = 0 and z = Lz - 1
    'd3e4_bgk_t1': dict(xi='D3Q19', fs='D3E4', tau=1.0, G=-4.5, psi='exp', dims=(16, 14, 12), wall=1,
                        R=4.0, centre=(8.0, 7.0, 4.0), rl=4.5, rg=0.21, n_wall=2.5, steps=[1, 50]),
}


def fields(c):
    dims = c['dims']
    D = len(dims)
    grids = np.meshgrid(*[np.arange(L) for L in reversed(dims)], indexing='ij')
    r2 = np.zeros(grids[0].shape)
    for d in range(D):
        r2 += (grids[D - 1 - d] - c['centre'][d]) ** 2
    r = np.sqrt(r2)
    rho = 0.5 * (c['rl'] + c['rg']) - 0.5 * (c['rl'] - c['rg']) * np.tanh((r - c['R']) / 2.0)
    rng = np.random.default_rng(mg.SEED)
    rho = rho * (1.0 + 1e-4 * rng.uniform(-1.0, 1.0, rho.shape))
    walls = np.ones(rho.shape, np.int32)
    w = c['wall']
    # the last axis of dims (y in 2D, z in 3D) is the first array axis
    walls[:w] = 0
    walls[-w:] = 0
    psi_w = np.full(rho.shape, np.exp(-1.0 / c['n_wall']))
    return rho, walls, psi_w


def gen_case(name, c):
    t0 = time.time()
    sc = mg.make_sim(c)
    Q = 9 if c['xi'] == 'D2Q9' else 19
    rho, walls, psi_w = fields(c)
    mg.set_fields(sc, rho)
    out = dict(walls=walls, psi_w=psi_w, n_init=rho,
               pop_init=mg.aos_to_soa(sc.sims_idpy_memory['pop'].D2H(), Q, c['dims']))
    with contextlib.redirect_stdout(io.StringIO()):
        sc.GetWalls(walls, psi_w)
    done = 0
    for k in c['steps']:
        with contextlib.redirect_stdout(io.StringIO()):
            sc.MainLoopWalls([0, k - done])
        done = k
        out['pop_%d' % k] = mg.aos_to_soa(sc.sims_idpy_memory['pop'].D2H(), Q, c['dims'])
        out['n_%d' % k] = sc.sims_idpy_memory['n'].D2H().reshape(tuple(reversed(c['dims'])))
    out['steps'] = np.array(c['steps'])
    out['config_json'] = json.dumps(c)
    np.savez_compressed(os.path.join(HERE, 'walls_%s.npz' % name), **out)
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
