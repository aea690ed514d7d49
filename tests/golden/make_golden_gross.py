"""Generate the fluctuating Shan-Chen fixtures from the reference itself.

Runs the reference's CTypes FP64 path of the Gross et al. (2011) fluctuating
step (``ShanChenMultiPhase(fluctuations='Gross2011', ...)`` +
``MainLoopGross2011SRT``, idpy/LBM/MultiPhase.py:1404-1541; the kernel
``K_ForceGross2011CollideStreamSCMPMeta``, idpy/LBM/MultiPhaseKernelsMeta.py:1369-1557;
noise moments ``GrossShanChenMultiPhase``, idpy/LBM/Fluctuations.py:40-165;
generators and Box-Muller, idpy/PRNGS/CRNGS.py:603-1276) on small droplets and
writes ``gross_<case>.npz`` into this directory:

  * ``n_init``        initial density; ``pop_init`` populations after InitPopulations (SoA)
  * ``seeds_init``    the generator states the reference drew (numpy legacy seeding,
                      CRNGS.InitSeeds, CRNGS.py:289-337), in its CPU ordering
                      (stream + cell * N_PRNG_STREAMS)
  * ``pop_<k>``       populations after k steps (SoA, (Q, *flip(dims))), read from the
                      step loop's own memory dict: ``MainLoopGross2011SRT`` hands its loop a
                      merged copy of the dicts (MultiPhase.py:1483), so after an odd number of
                      steps ``sims_idpy_memory['pop']`` still names the pre-step buffer
  * ``seeds_<k>``     generator states after k steps (CPU ordering)
  * ``n_<k>``         the reference's n array after k steps (density at the start of
                      the last step)
  * ``noise_json``    the generated kernel's noise literals: the variance literal of
                      each random moment and, per population, the (moment, literal)
                      terms in the order the kernel adds them
  * ``config_json``   the case

The ``flat`` distribution is not recorded: the reference's code generator
raises for it (its variances are strings, so ``sqrt(12 * var)`` repeats the
string, CRNGS.py:903 with Fluctuations.py:87-97).

Nothing at test time imports the reference.

Usage:
    python tests/golden/make_golden_gross.py --reference /path/to/idea.deploy [case ...]
"""
import argparse
import contextlib
import glob
import io
import json
import os
import re
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as mg  # noqa: E402

CASES = {
    # one stream per random moment, two successive draws per Gaussian (Box-Muller, cos)
    'd2e4_mmix_t1': dict(xi='D2Q9', fs='D2E4', tau=1.0, G=-4.5, psi='exp', dims=(32, 24), R=6.0,
                         rl=4.5625, rg=0.2086, width=2.0, kind='MMIX', indep=False, kBT=1e-4, n0=1.0,
                         init_seed=3, steps=[1, 10, 200]),
    # two streams per random moment
    'd2e8_minstd_indep_t08': dict(xi='D2Q9', fs='D2E8', tau=0.8, G=-4.5, psi='exp', dims=(24, 28), R=6.0,
                                  rl=4.646, rg=0.204, width=2.0, kind='MINSTD', indep=True, kBT=3e-5,
                                  n0=2.0, init_seed=11, steps=[1, 10, 200]),
    'd2e6_numrec_t12_psi1mexp': dict(xi='D2Q9', fs='D2E6', tau=1.2, G=-1.6, psi='1mexp', dims=(24, 24),
                                     R=6.0, rl=1.736, rg=0.1595, width=2.0, kind='NUMREC', indep=False,
                                     kBT=1e-5, n0=1.0, init_seed=5, steps=[1, 10, 200]),
    'd3e4_mmix_t1': dict(xi='D3Q19', fs='D3E4', tau=1.0, G=-4.5, psi='exp', dims=(12, 10, 8), R=3.0,
                         rl=4.5, rg=0.21, width=2.0, kind='MMIX', indep=False, kBT=1e-4, n0=1.0,
                         init_seed=7, steps=[1, 20]),
    'd3e6_minstd_indep_t09': dict(xi='D3Q19', fs='D3E6', tau=0.9, G=-4.5, psi='exp', dims=(10, 8, 12),
                                  R=3.0, rl=4.636, rg=0.147, width=2.0, kind='MINSTD', indep=True,
                                  kBT=2e-5, n0=1.5, init_seed=13, steps=[1, 20]),
}


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
        sc = ShanChenMultiPhase(lang=CTYPES_T, dim_sizes=tuple(c['dims']), xi_stencil=XIStencils[c['xi']],
                                f_stencil=FStencils[c['fs']], psi_code=psi_code, psi_sym=psi_sym, SC_G=c['G'],
                                tau=c['tau'], fluctuations='Gross2011', prng_kind=c['kind'],
                                init_seed=c['init_seed'], prng_init_from='numpy', prng_distribution='gaussian',
                                indep_gaussian=c['indep'], cl_kind='cpu', device=0)
    return sc


def parse_noise(c):
    """Variance literals and per-population noise terms of the generated
    fluctuating kernel for this case (its macros identify it)."""
    V = int(np.prod(c['dims']))
    want = ['#define V %d\n' % V, '#define L_0 %d\n' % c['dims'][0],
            '#define OMEGA %r\n' % (1. / c['tau']), '#define SC_G %r\n' % c['G']]
    files = sorted(glob.glob('/tmp/idpy_ctypes_kernels/*.c'), key=os.path.getmtime)
    src = None
    for f in reversed(files):
        s = open(f).read()
        if 'int K_ForceGross2011CollideStreamSCMPMeta(' in s and all(w in s for w in want):
            src = s
            break
    if src is None:
        raise RuntimeError('generated fluctuating kernel not found')
    var = {}
    for m in re.finditer(r'Rm_(\d+) = sqrt\(\(PopType\)\(-2\. \* ([0-9.eE+-]+) \* log', src):
        var[int(m.group(1))] = m.group(2)
    terms = {}
    for m in re.finditer(r'\(\*\(pop_swap \+ (\d+) \+ x_dst \* Q\)\) = (.*?);', src):
        q, expr = int(m.group(1)), m.group(2)
        tl = []
        for tm in re.finditer(r'([+-]?)\s*(-?\d[0-9.eE+-]*)\*Rm_(\d+)', expr):
            sign, lit, k = tm.groups()
            if sign == '-':
                lit = lit[1:] if lit.startswith('-') else '-' + lit
            tl.append([int(k), lit])
        terms[q] = tl
    return dict(var=[var[k] for k in range(len(var))], terms=[terms[q] for q in range(len(terms))])


def gen_case(name, c):
    t0 = time.time()
    sc = make_sim(c)
    Q = 9 if c['xi'] == 'D2Q9' else 19
    rho = mg.droplet(c['dims'], c['R'], c['rl'], c['rg'], c['width'])
    mg.set_fields(sc, rho)
    out = dict(n_init=rho, pop_init=mg.aos_to_soa(sc.sims_idpy_memory['pop'].D2H(), Q, c['dims']),
               seeds_init=sc.crng.sims_idpy_memory['seeds'].D2H().copy())
    done = 0
    for k in c['steps']:
        with contextlib.redirect_stdout(io.StringIO()):
            sc.MainLoopGross2011SRT([0, k - done], kBT=c['kBT'], n0=c['n0'])
        done = k
        # the loop runs on a merged copy of the memory dicts, so the buffer swap
        # reaches only that copy: read the populations from the loop's own dict
        # (sims_idpy_memory['pop'] is the pre-step buffer after odd step counts)
        out['pop_%d' % k] = mg.aos_to_soa(sc._MainLoop.args_dicts[0]['pop'].D2H(), Q, c['dims'])
        out['n_%d' % k] = sc.sims_idpy_memory['n'].D2H().reshape(tuple(reversed(c['dims'])))
        out['seeds_%d' % k] = sc.crng.sims_idpy_memory['seeds'].D2H().copy()
    out['steps'] = np.array(c['steps'])
    out['noise_json'] = json.dumps(parse_noise(c))
    out['config_json'] = json.dumps(dict(c, seed=mg.SEED))
    np.savez_compressed(os.path.join(HERE, 'gross_%s.npz' % name), **out)
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
