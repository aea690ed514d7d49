"""Generate the thermodynamic golden values from the reference's own SCThermo.

Runs ``idpy.LBM.SCThermo.ShanChanEquilibriumCache`` (Guo forcing) of the
reference checkout given by ``--reference`` for the 2D force stencils E4, E6
and E8 and a few couplings G, and writes ``thermo.json`` into this directory:
per case the critical point (G_c, n_c), the flat-interface coexistence
densities from the mechanical-equilibrium (Maxwell-type) construction (n_l,
n_g, p_0) and the surface tension sigma_f.  The stencil weights are given
directly (grouped by squared length) instead of being solved for, so no
nonlinear solve of the isotropy equations is needed.

``sclbm.thermo`` restates this construction; the CPU tests compare it with
these values.  Nothing at test time imports the reference.

The reference needs a few modules that are absent here and unused on this path
(h5py, matplotlib, IPython, dill, multiprocess); empty stand-ins are written to
a temporary directory and put on ``sys.path`` first.  Each case takes one to a
few minutes (sympy), so cases run in a spawned process pool.

Usage:
    python tests/golden/make_thermo.py --reference /path/to/idea.deploy
"""
import argparse
import json
import multiprocessing as mp
import os
import sys
import tempfile
import time

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

# stencil -> (x_max of the basis, squared lengths, weights as fractions)
STENCILS = {
    'D2E4': (1, [1, 2], [(1, 3), (1, 12)]),
    'D2E6': (2, [1, 2, 4], [(4, 15), (1, 10), (1, 120)]),
    'D2E8': (2, [1, 2, 4, 5, 8], [(4, 21), (4, 45), (1, 60), (2, 315), (1, 5040)]),
}
PSI = {'exp': 'exp(-1/n)', '1mexp': '1 - exp(-n)'}
CASES = [(st, 'exp', G) for st in STENCILS for G in (-4.5, -5.0, -5.5, -6.0)] + \
        [('D2E4', '1mexp', G) for G in (-1.6, -2.0)]


def run_case(args):
    reference, st_name, psi_name, G = args
    tmp = tempfile.mkdtemp(prefix='thermo_')
    for k, v in STUBS.items():
        p = os.path.join(tmp, k)
        os.makedirs(os.path.dirname(p), exist_ok=True)
        with open(p, 'w') as fh:
            fh.write(v)
    sys.path.insert(0, tmp)
    sys.path.insert(0, reference)
    os.chdir(tmp)
    import sympy as sp
    from idpy.LBM.SCFStencils import SCFStencils, BasisVectors
    from idpy.LBM.SCThermo import ShanChanEquilibriumCache
    n = sp.symbols('n')
    x_max, l2, w = STENCILS[st_name]
    st = SCFStencils(E=BasisVectors(x_max=x_max), len_2s=l2)
    st.GetWolfEqs()
    st.GetTypEqs()
    st.w_sol.append([sp.Rational(a, b) for a, b in w])
    psi = sp.exp(-1 / n) if psi_name == 'exp' else 1 - sp.exp(-n)
    t0 = time.time()
    try:
        c = ShanChanEquilibriumCache(stencil=st, G=G, c2=sp.Rational(1, 3), psi_f=psi,
                                     dump_file=os.path.join(tmp, 'cache.json'))
        out = {k: float(v) for k, v in c.GetFromCache().items()}
    except Exception as e:  # recorded, not hidden
        out = {'error': '%s: %s' % (type(e).__name__, e)}
    out.update(stencil=st_name, psi=PSI[psi_name], G=G, c2=1.0 / 3, seconds=round(time.time() - t0, 1))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--reference', required=True)
    ap.add_argument('--jobs', type=int, default=len(CASES))
    a = ap.parse_args()
    ctx = mp.get_context('spawn')
    with ctx.Pool(min(a.jobs, len(CASES))) as pool:
        res = pool.map(run_case, [(os.path.abspath(a.reference),) + c for c in CASES])
    with open(os.path.join(HERE, 'thermo.json'), 'w') as fh:
        json.dump({'source': 'idpy/LBM/SCThermo.py ShanChanEquilibriumCache (forcing guo)', 'cases': res}, fh,
                  indent=1)
    for r in res:
        print(r)


if __name__ == '__main__':
    main()
