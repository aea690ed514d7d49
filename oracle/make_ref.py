"""Recipe: the reference's own CPU kernels for the CPU-baseline leg of bench.py.

The reference (lullimat/idea.deploy, ``idpy``) has no C sources in its tree:
its CTypes backend generates C for each kernel at run time (sympy codegen,
idpy/IdpyCode/IdpyCode.py:940-1094) and builds it with
``gcc -fPIC -shared -std=c99 -O3`` (idpy/CTypes/__init__.py:48,
idpy/IdpyCode/IdpyCode.py:585-586).  This recipe runs that generator on the
benchmark configuration (a 64^3 sample box of the D3Q19 E6 MRT workload) and
copies the generated sources, unmodified, into ``oracle/_ref/``; ``build``
below compiles them there with the reference's own flags.  ``oracle/_ref`` is
git-ignored; the generated C travels with the working tree and is compiled on
the machine that runs it.

Usage (needs the reference checkout; ~8 min of sympy for the MRT kernel):
    python oracle/make_ref.py --reference /path/to/idea.deploy
"""
import argparse
import contextlib
import glob
import io
import json
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, '_ref')
MANIFEST = os.path.join(REF_DIR, 'manifest.json')

# (tag, lattice, stencil, collision, rates, G, tau, box)
TARGETS = [
    ('d3q19_e6_mrt1_64', 'D3Q19', 'D3E6', 'mrt', [1.0] * 19, -5.0, 1.0, (64, 64, 64)),
    ('d2q9_e4_bgk_256', 'D2Q9', 'D2E4', 'bgk', None, -5.0, 1.0, (256, 256)),
]
KERNELS = {'density': 'K_ComputeDensityPsiMeta', 'init': 'K_InitPopulationsMeta',
           'bgk': 'K_ForceCollideStreamSCMPMeta', 'mrt': 'K_ForceCollideStreamSCMP_MRTMeta'}


def _stubs():
    tmp = tempfile.mkdtemp(prefix='idpy_stubs_')
    files = {'h5py.py': '', 'dill.py': '', 'multiprocess.py': '', 'matplotlib/__init__.py': '',
             'matplotlib/pyplot.py': 'def figure(*a, **k):\n    pass\n', 'IPython/__init__.py': '',
             'IPython/display.py': 'def display(*a, **k):\n    pass\nMath = Latex = display\n'}
    for rel, body in files.items():
        p = os.path.join(tmp, rel)
        os.makedirs(os.path.dirname(p), exist_ok=True)
        with open(p, 'w') as f:
            f.write(body)
    return tmp


def generate(reference, only=None):
    sys.path.insert(0, reference)
    sys.path.insert(0, _stubs())
    sys.dont_write_bytecode = True
    import warnings
    warnings.filterwarnings('ignore')
    import numpy as np
    import sympy as sp
    from idpy.IdpyCode import CTYPES_T
    from idpy.LBM.MultiPhase import ShanChenMultiPhase
    from idpy.LBM.LBM import XIStencils, FStencils
    from idpy.LBM.Collisions import RelaxationMatrix
    from idpy.LBM.Equilibria import HermiteEquilibria
    os.makedirs(REF_DIR, exist_ok=True)
    manifest = json.load(open(MANIFEST)) if os.path.exists(MANIFEST) else {}
    n = sp.Symbol('n')
    for tag, xi, fs, coll, rates, G, tau, box in TARGETS:
        if only and tag not in only:
            continue
        with contextlib.redirect_stdout(io.StringIO()):
            sc = ShanChenMultiPhase(lang=CTYPES_T, dim_sizes=box, xi_stencil=XIStencils[xi],
                                    f_stencil=FStencils[fs], psi_code='exp(-1./ln_0)',
                                    psi_sym=sp.exp(-1 / n), SC_G=G, tau=tau)
            V = int(np.prod(box))
            sc.sims_idpy_memory['n'].H2D(np.ones(V))
            sc.sims_idpy_memory['u'].SetConst(0.)
            sc.init_status['n'] = sc.init_status['u'] = True
            sc.InitPopulations()
            if coll == 'mrt':
                eq = HermiteEquilibria(XIStencils[xi])
                rm = RelaxationMatrix(eq)
                syms = [sp.Symbol('\\omega_%d' % i) for i in range(len(rates))]
                sc.MainLoopMRT(range(0, 2, 1), relaxation_matrix=rm.GetDiagonalMatrix(syms),
                               omega_syms_vals=list(zip(syms, rates)))
            else:
                sc.MainLoop(range(0, 2, 1))
        want = '#define V %d\n' % V
        files = {}
        for role, kname in [('density', KERNELS['density']), ('init', KERNELS['init']),
                            ('step', KERNELS[coll])]:
            cands = [f for f in glob.glob('/tmp/idpy_ctypes_kernels/*.c')
                     if ('int ' + kname + '(') in open(f).read() and want in open(f).read()
                     and ('#define SC_G %r\n' % G) in open(f).read()]
            cands.sort(key=os.path.getmtime)
            if not cands:
                raise SystemExit('generated source for %s not found' % kname)
            dst = '%s_%s.c' % (tag, role)
            shutil.copyfile(cands[-1], os.path.join(REF_DIR, dst))
            files[role] = {'file': dst, 'kernel': kname}
        manifest[tag] = dict(lattice=xi, stencil=fs, collision=coll, rates=rates, G=G, tau=tau,
                             box=list(box), Q=len(XIStencils[xi]['XIs']), files=files)
        json.dump(manifest, open(MANIFEST, 'w'), indent=1)
        print('generated', tag, flush=True)


def box_variants():
    """Smaller sample boxes of the 3D benchmark kernels (32^3, 16^3) for the
    bounded CPU baseline: the generated sources take the box size only through
    their #define constants (V, L_i, STR_i, N_THREADS), the values the
    reference passes per box (idpy/IdpyCode/IdpyCode.py:567-611)."""
    man = json.load(open(MANIFEST))
    base = man.get('d3q19_e6_mrt1_64')
    if base is None:
        return
    for L in (32, 16):
        tag = 'd3q19_e6_mrt1_%d' % L
        files = {}
        for role, f in base['files'].items():
            src = open(os.path.join(REF_DIR, f['file'])).read()
            defs = {'V': L ** 3, 'L_0': L, 'L_1': L, 'L_2': L, 'STR_0': L, 'STR_1': L * L, 'N_THREADS': L ** 3}
            lines = []
            for line in src.split('\n'):
                parts = line.split()
                if len(parts) == 3 and parts[0] == '#define' and parts[1] in defs:
                    line = '#define %s %d' % (parts[1], defs[parts[1]])
                lines.append(line)
            dst = '%s_%s.c' % (tag, role)
            text = '\n'.join(lines)
            path = os.path.join(REF_DIR, dst)
            if not os.path.exists(path) or open(path).read() != text:
                with open(path, 'w') as fh:
                    fh.write(text)
            files[role] = {'file': dst, 'kernel': f['kernel']}
        man[tag] = dict(base, box=[L, L, L], files=files)
    json.dump(man, open(MANIFEST, 'w'), indent=1)


def build():
    """Compile the generated sources in oracle/_ref with the reference's flags."""
    if not os.path.exists(MANIFEST):
        return []
    box_variants()
    out = []
    for src in sorted(glob.glob(os.path.join(REF_DIR, '*.c'))):
        so = src[:-2] + '.so'
        if os.path.exists(so) and os.path.getmtime(so) >= os.path.getmtime(src):
            out.append(so)
            continue
        subprocess.check_call(['gcc', '-fPIC', '-shared', '-std=c99', '-O3', '-o', so, src, '-lm'],
                              stderr=subprocess.DEVNULL)
        out.append(so)
    return out


if __name__ == '__main__':
    ap = argparse.ArgumentParser()
    ap.add_argument('--reference', required=True)
    ap.add_argument('targets', nargs='*')
    a = ap.parse_args()
    generate(os.path.abspath(a.reference), a.targets)
    print(build())
