"""CPU oracle for the Shan-Chen time step -- TEST INFRASTRUCTURE ONLY.

Restates the reference's CTypes FP64 path (lullimat/idea.deploy, ``idpy``) so
the CUDA path can be checked against it.  Only ``tests/``, the smoke check and
the CPU-baseline leg of ``bench.py`` may import this module; the product never
does.  The numerical kernels live in ``sc_oracle.c`` (plain C, gcc, no FMA
contraction: the reference builds its generated C with ``gcc -std=c99 -O3``,
``idpy/CTypes/__init__.py:48``, which does not contract).

Parity pin: ``tests/test_oracle_golden.py`` checks this oracle against the
fixtures in ``tests/golden/`` that ``tests/golden/make_golden.py`` produced by
running the reference itself; on BGK cases the oracle is bit-identical to it.

What is restated where:
  * coefficients of the expanded BGK+Guo collision: ``bgk_terms``
      idpy/LBM/Collisions.py:163-185,251-273, idpy/LBM/Forcings.py:104-127,
      idpy/LBM/Equilibria.py:107-210
  * MRT+Guo collision: ``mrt_terms``
      idpy/LBM/Collisions.py:96-160,275-316, idpy/LBM/Forcings.py:129-181
  * Hermite moment bases (invertible set, Gram-Schmidt W-orthogonal set):
    ``hermite_bases``  idpy/IdpyStencils/IdpyStencils.py:838-1043
  * literal emission: sympy ``evalf()`` prints 15 significant digits
    (``round15``); force-stencil weights are Python floats printed in full
    (idpy/IdpyStencils/IdpyStencils.py:1538-1544)
  * initial profiles: idpy/LBM/MultiPhaseKernels.py:44-112,605-777
  * CheckUConvergenceSCMP: idpy/LBM/MultiPhaseLoopChecks.py:96-163
  * DeltaPLaplace / PBulk / ComputeCenterOfMass: idpy/LBM/MultiPhase.py:108-137,1690-1768
  * the "simple" step family (MainLoopSimple*, idpy/LBM/MultiPhase.py:164-1014):
    ``OracleSimple``  idpy/LBM/MultiPhaseKernels.py:132-604,
    idpy/LBM/LBMKernels.py:117-258,299-456
  * Gross et al. (2011) fluctuations: ``noise_terms``, ``noise_variance``,
    ``OracleSim.set_fluctuations``  idpy/LBM/Fluctuations.py:40-165,
    idpy/PRNGS/CRNGS.py:603-1276, idpy/LBM/MultiPhaseKernelsMeta.py:1369-1557
"""
import ctypes
import math
import os
import subprocess
import threading
from fractions import Fraction
from itertools import combinations_with_replacement

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(BUILD, 'liboracle.so')

PSI_KINDS = {'exp': 0, '1mexp': 1, 'identity': 2}

_lock = threading.Lock()
_lib = None


def build():
    """Compile sc_oracle.c into oracle/_build/liboracle.so (gcc, ISO C99, no FMA)."""
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, 'sc_oracle.c')
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    tmp = LIB + '.%d.tmp' % os.getpid()
    subprocess.check_call(['gcc', '-std=c99', '-O2', '-ffp-contract=off', '-fno-fast-math',
                           '-fPIC', '-shared', '-o', tmp, src, '-lm'])
    os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    with _lock:
        if _lib is None:
            _lib = ctypes.CDLL(build())
    return _lib


# ----------------------------------------------------------------------------
# coefficient literals
# ----------------------------------------------------------------------------

def round15(x):
    """Value of the 15-significant-digit literal sympy prints for x."""
    if x == 0:
        return 0.0
    return float('%.15g' % float(x))


def _mono_name(kind, a=None, b=None, q=None):
    if kind == 'n':
        return 'ln_0'
    if kind == 'nu':
        return 'ln_0*lu_0_%d' % a
    if kind == 'nuu':
        return 'ln_0*lu_0_%d*lu_0_%d' % (a, b)
    if kind == 'F':
        return 'd_psi_%d' % a
    if kind == 'Fu':
        return 'd_psi_%d*lu_0_%d' % (a, b)
    if kind == 'f':
        return 'lpop_%d' % q
    raise ValueError(kind)


def _factor_ids(name, D):
    """Map 'ln_0*lu_0_1' style names to indices of v = [n, u.., F.., f..]."""
    ids = []
    for tok in name.split('*'):
        if tok == 'ln_0':
            ids.append(0)
        elif tok.startswith('lu_0_'):
            ids.append(1 + int(tok[5:]))
        elif tok.startswith('d_psi_'):
            ids.append(1 + D + int(tok[6:]))
        elif tok.startswith('lpop_'):
            ids.append(1 + 2 * D + int(tok[5:]))
        else:
            raise ValueError(tok)
    return ids


def _exact(x):
    return Fraction(x)


def _monomial_coeffs_bgk(xi, w, c2, omega, q, D):
    """Exact (on the given double inputs) coefficient per monomial name."""
    F = Fraction
    om = _exact(omega)
    wq = _exact(w[q])
    c2 = _exact(c2)
    e = xi[q]
    out = {}
    out[_mono_name('n')] = om * wq
    for a in range(D):
        out[_mono_name('nu', a)] = om * wq * e[a] / c2
    for a in range(D):
        for b in range(a, D):
            if a == b:
                out[_mono_name('nuu', a, a)] = om * wq * (e[a] * e[a] - c2) / (2 * c2 * c2)
            else:
                out[_mono_name('nuu', a, b)] = om * wq * e[a] * e[b] / (c2 * c2)
    g = (1 - om / 2) * wq
    for a in range(D):
        out[_mono_name('F', a)] = g * e[a] / c2
    for a in range(D):
        for b in range(D):
            out[_mono_name('Fu', a, b)] = g * (e[a] * e[b] - (c2 if a == b else 0)) / (c2 * c2)
    out[_mono_name('f', q=q)] = 1 - om
    return out


def _finish(coeffs, mode):
    """Drop zero terms, sort in the reference's print order, apply literal mode."""
    terms = []
    for name in sorted(coeffs):
        c = coeffs[name]
        if c == 0:
            continue
        v = round15(c) if mode == 'round15' else float(c)
        if v == 0.0:
            continue
        terms.append((v, name))
    return terms


def bgk_terms(xi, w, c2, omega, mode='round15'):
    D = len(xi[0])
    return [_finish(_monomial_coeffs_bgk(xi, w, c2, omega, q, D), mode) for q in range(len(xi))]


def eq_terms(xi, w, c2, mode='round15'):
    """Second-order equilibrium (InitPopulations): omega = 1 and no forcing."""
    D = len(xi[0])
    out = []
    for q in range(len(xi)):
        c = _monomial_coeffs_bgk(xi, w, c2, 1.0, q, D)
        c = {k: v for k, v in c.items() if k.startswith('ln_0')}
        # the init kernel names products ln_0_lu_0_a..., same order of factors
        out.append(_finish(c, mode))
    return out


def _hermite_1d_tensor(order, idx, xi, c2):
    """c_s^n H^{(n)}_{idx}(xi / c_s) for a lattice vector xi (exact, Fraction).

    Multivariate probabilists' Hermite tensors; with c2 = c_s^2 the scaled
    polynomial only contains even powers of c_s, so it is rational in c2:
      n=1: x_a
      n=2: x_a x_b - c2 d_ab
      n=3: x_a x_b x_c - c2 (x_a d_bc + x_b d_ac + x_c d_ab)
      n>=4: via the recursion H_{n+1, i+a} = x_a H_{n,i} - c2 sum_k d_{a,i_k} H_{n-1, i\\k}
    """
    def H(idxs):
        if len(idxs) == 0:
            return Fraction(1)
        a, rest = idxs[-1], idxs[:-1]
        val = xi[a] * H(rest)
        for k in range(len(rest)):
            if rest[k] == a:
                val -= c2 * H(rest[:k] + rest[k + 1:])
        return val
    return H(tuple(idx))


def hermite_bases(xi, w, c2, search_depth=6):
    """(M, M_worth) as exact Fractions, following GetInvertibleHermiteSet and
    GetWOrthInvertibleHermiteSet (idpy/IdpyStencils/IdpyStencils.py:905-1043)."""
    Q, D = len(xi), len(xi[0])
    c2 = Fraction(c2).limit_denominator(1000)
    W = [Fraction(x).limit_denominator(10000) for x in w]
    rows = [[Fraction(1)] * Q]
    count, order = 1, 1
    while count < Q + search_depth:
        for tup in combinations_with_replacement(range(D), order):
            r = [_hermite_1d_tensor(order, tup, xi[i], c2) for i in range(Q)]
            if any(v != 0 for v in r):
                rows.append(r)
                count += 1
        order += 1
    # rref of rows^T: pivot columns = first linearly independent rows, in order
    sel = []
    basis = []
    for i, r in enumerate(rows):
        if _independent(basis, r):
            basis.append(r)
            sel.append(i)
        if len(sel) == Q:
            break
    M = [rows[i] for i in sel]
    # classical Gram-Schmidt with <a,b> = sum_i a_i b_i W_i
    def prod(a, b):
        return sum(x * y * z for x, y, z in zip(a, b, W))
    Mw = [M[0]]
    for i in range(1, Q):
        v = list(M[i])
        for u in Mw:
            p = prod(M[i], u) / prod(u, u)
            v = [vi - p * ui for vi, ui in zip(v, u)]
        Mw.append(v)
    return M, Mw


def _independent(basis, r):
    """True if r is not in the span of basis (exact elimination)."""
    rows = [list(b) for b in basis] + [list(r)]
    n = len(rows[0])
    rank = 0
    col = 0
    m = [row[:] for row in rows]
    for col in range(n):
        piv = None
        for i in range(rank, len(m)):
            if m[i][col] != 0:
                piv = i
                break
        if piv is None:
            continue
        m[rank], m[piv] = m[piv], m[rank]
        for i in range(len(m)):
            if i != rank and m[i][col] != 0:
                f = m[i][col] / m[rank][col]
                m[i] = [a - f * b for a, b in zip(m[i], m[rank])]
        rank += 1
    return rank == len(rows)


def _inverse(M):
    n = len(M)
    a = [list(row) + [Fraction(int(i == j)) for j in range(n)] for i, row in enumerate(M)]
    for c in range(n):
        p = next(i for i in range(c, n) if a[i][c] != 0)
        a[c], a[p] = a[p], a[c]
        pv = a[c][c]
        a[c] = [x / pv for x in a[c]]
        for i in range(n):
            if i != c and a[i][c] != 0:
                f = a[i][c]
                a[i] = [x - f * y for x, y in zip(a[i], a[c])]
    return [row[n:] for row in a]


def _matmul(A, B):
    return [[sum(A[i][k] * B[k][j] for k in range(len(B))) for j in range(len(B[0]))]
            for i in range(len(A))]


def mrt_terms(xi, w, c2, rates, mode='round15'):
    """f* = M^-1 [S M feq + (I-S) M f] + Mn^-1 (I - S/2) Mn Fg, expanded on the
    monomials (S diagonal with the given rates; M W-orthogonal, Mn the plain
    invertible Hermite set, exactly as the reference combines them)."""
    Q, D = len(xi), len(xi[0])
    Mn, Mw = hermite_bases(xi, w, c2)
    Mwi, Mni = _inverse(Mw), _inverse(Mn)
    S = [Fraction(r) for r in rates]
    # population-space operators
    A = _matmul(Mwi, [[(1 - S[i]) * Mw[i][j] for j in range(Q)] for i in range(Q)])
    B = _matmul(Mwi, [[S[i] * Mw[i][j] for j in range(Q)] for i in range(Q)])
    C = _matmul(Mni, [[(1 - S[i] / 2) * Mn[i][j] for j in range(Q)] for i in range(Q)])
    # monomial expansion of feq_j and Fg_j (omega = 1, forcing without (1-w/2))
    feq = [_monomial_coeffs_bgk(xi, w, c2, 1.0, j, D) for j in range(Q)]
    fg = []
    for j in range(Q):
        cj = _monomial_coeffs_bgk(xi, w, c2, 0.0, j, D)   # (1 - 0/2) = 1
        fg.append({k: v for k, v in cj.items() if k.startswith('d_psi')})
    out = []
    for i in range(Q):
        coeffs = {}
        for j in range(Q):
            if A[i][j] != 0:
                coeffs[_mono_name('f', q=j)] = coeffs.get(_mono_name('f', q=j), 0) + A[i][j]
            for k, v in feq[j].items():
                if not k.startswith('ln_0'):
                    continue
                coeffs[k] = coeffs.get(k, 0) + B[i][j] * v
            for k, v in fg[j].items():
                coeffs[k] = coeffs.get(k, 0) + C[i][j] * v
        out.append(_finish(coeffs, mode))
    return out


CRNG_KINDS = {'MINSTD': 1, 'NUMREC': 2, 'MMIX': 3}


def noise_variance(norm, kBT, tau, n0, c2=1.0 / 3.0):
    """Variance literal of one random moment, as GetVariances evaluates and
    prints it (idpy/LBM/Fluctuations.py:72-97): norm * kBT * (2 - 1/tau) / tau
    / c_s2 * n0, each product and quotient rounded to double (sympy Float at
    53 bits), printed with 15 significant digits.  tau is 1/OMEGA as the
    kernel passes it (MultiPhaseKernelsMeta.py:1521)."""
    a = float(Fraction(norm)) * kBT
    a = a * (2 - 1 / tau)
    a = a / tau
    a = a / c2
    a = a * n0
    return round15(a)


def noise_terms(xi, w, c2, mode='round15'):
    """Noise populations rpop = Mw^-1 [0 .. 0, Rm_0 .. Rm_{Q-D-2}]
    (Fluctuations.py:158-163) as exact coefficients of the random moments, per
    population a list of (literal, moment) in sympy's print order (the moment
    names sorted as strings: Rm_0, Rm_1, Rm_10, ..., Rm_2, ...), and the
    Hermite norms sum_q w_q Mw[k][q]^2 of the random moments
    (IdpyStencils.py:977-980)."""
    Q, D = len(xi), len(xi[0])
    _, Mw = hermite_bases(xi, w, c2)
    Mwi = _inverse(Mw)
    W = [Fraction(x).limit_denominator(10000) for x in w]
    norms = [sum(W[q] * Mw[k][q] * Mw[k][q] for q in range(Q)) for k in range(D + 1, Q)]
    nr = Q - (D + 1)
    order = sorted(range(nr), key=lambda j: 'Rm_%d' % j)
    out = []
    for q in range(Q):
        tl = []
        for j in order:
            c = Mwi[q][D + 1 + j]
            if c == 0:
                continue
            tl.append((round15(c) if mode == 'round15' else float(c), j))
        out.append(tl)
    return out, norms


def noise_from_literals(noise):
    """(terms, m2var) straight from the reference's generated literals
    (fixture dict with 'var' and 'terms')."""
    terms = [[(float(c), int(k)) for k, c in tl] for tl in noise['terms']]
    return terms, [-2.0 * float(v) for v in noise['var']]


def terms_from_literals(lit):
    """Terms straight from the reference's generated literals (fixture dict)."""
    out = []
    for q in range(len(lit)):
        d = lit[str(q)] if str(q) in lit else lit[q]
        out.append([(float(v), k) for k, v in d.items()])
    return out


# ----------------------------------------------------------------------------
# ctypes configuration
# ----------------------------------------------------------------------------

class _Cfg(ctypes.Structure):
    _fields_ = [('dim', ctypes.c_int), ('L', ctypes.c_int * 3), ('Q', ctypes.c_int),
                ('QE', ctypes.c_int), ('xi', ctypes.c_void_p), ('e', ctypes.c_void_p),
                ('we', ctypes.c_void_p), ('G', ctypes.c_double), ('psi_kind', ctypes.c_int),
                ('t_off', ctypes.c_void_p), ('t_coef', ctypes.c_void_p),
                ('t_nf', ctypes.c_void_p), ('t_fid', ctypes.c_void_p),
                ('v_off', ctypes.c_void_p), ('v_pop', ctypes.c_void_p),
                ('v_sign', ctypes.c_void_p), ('n_order', ctypes.c_void_p)]


class _Noise(ctypes.Structure):
    _fields_ = [('kind', ctypes.c_int), ('indep', ctypes.c_int), ('nr', ctypes.c_int),
                ('m2var', ctypes.c_void_p), ('t_off', ctypes.c_void_p), ('t_mom', ctypes.c_void_p),
                ('t_coef', ctypes.c_void_p)]


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class _Tables:
    def __init__(self, terms, D):
        off, coef, nf, fid = [0], [], [], []
        for tl in terms:
            for c, name in tl:
                ids = _factor_ids(name, D)
                coef.append(c)
                nf.append(len(ids))
                fid.extend(ids + [0] * (3 - len(ids)))
            off.append(len(coef))
        self.off = np.array(off, np.int32)
        self.coef = np.array(coef, np.float64)
        self.nf = np.array(nf, np.int32)
        self.fid = np.array(fid, np.int32)


class OracleSim:
    """FP64 AoS Shan-Chen simulation on the CPU, mirroring the reference's
    ``ShanChenMultiPhase`` step loop (MainLoop / MainLoopMRT)."""

    def __init__(self, dims, xi, w, c2, e, we, G, tau=1.0, psi='exp', rates=None,
                 mode='round15', literals=None, eq_literals=None):
        self.dims = tuple(int(x) for x in dims)
        self.D = len(self.dims)
        self.Q = len(xi)
        self.V = int(np.prod(self.dims))
        self.xi = [tuple(int(v) for v in x) for x in xi]
        self.w, self.c2 = list(w), float(c2)
        self.G = float(G)
        self.psi = psi
        D, Q = self.D, self.Q
        if literals is not None:
            terms = terms_from_literals(literals)
        elif rates is None:
            terms = bgk_terms(self.xi, self.w, self.c2, 1.0 / tau, mode)
        else:
            terms = mrt_terms(self.xi, self.w, self.c2, rates, mode)
        self.terms = terms
        self.eq = eq_terms(self.xi, self.w, self.c2, mode) if eq_literals is None else \
            terms_from_literals(eq_literals)
        self._t = _Tables(terms, D)
        self._te = _Tables(self.eq, D)
        names = sorted('pop_%d' % q for q in range(Q))
        self._n_order = np.array([int(s[4:]) for s in names], np.int32)
        voff, vpop, vsign = [0], [], []
        for d in range(D):
            lst = sorted((('lpop_%d' % q), q) for q in range(Q) if self.xi[q][d] != 0)
            for _, q in lst:
                vpop.append(q)
                vsign.append(1 if self.xi[q][d] > 0 else -1)
            voff.append(len(vpop))
        self._voff = np.array(voff, np.int32)
        self._vpop = np.array(vpop, np.int32)
        self._vsign = np.array(vsign, np.int32)
        self._xi = np.array(self.xi, np.int32).ravel()
        self._e = np.array(e, np.int32).ravel()
        self._we = np.array(we, np.float64)
        self.pop = np.zeros(self.V * Q)
        self.pop_swap = np.zeros(self.V * Q)
        self.n = np.zeros(self.V)
        self.psi_arr = np.zeros(self.V)
        self.u = np.zeros(self.V * D)
        self.cfg = self._make_cfg(self._t)
        self.cfg_eq = self._make_cfg(self._te)
        self.old_u = None

    def _make_cfg(self, t):
        c = _Cfg()
        c.dim = self.D
        for d in range(3):
            c.L[d] = self.dims[d] if d < self.D else 1
        c.Q, c.QE = self.Q, len(self._we)
        c.xi, c.e, c.we = _ptr(self._xi), _ptr(self._e), _ptr(self._we)
        c.G, c.psi_kind = self.G, PSI_KINDS[self.psi]
        c.t_off, c.t_coef, c.t_nf, c.t_fid = _ptr(t.off), _ptr(t.coef), _ptr(t.nf), _ptr(t.fid)
        c.v_off, c.v_pop, c.v_sign = _ptr(self._voff), _ptr(self._vpop), _ptr(self._vsign)
        c.n_order = _ptr(self._n_order)
        return c

    # --- fields -----------------------------------------------------------
    def set_fields(self, n, u=None):
        self.n[:] = np.ascontiguousarray(n, np.float64).ravel()
        if u is None:
            self.u[:] = 0.0
        else:   # u given as (D, *flip(dims))
            self.u[:] = np.asarray(u, np.float64).reshape(self.D, -1).T.ravel()

    def init_populations(self):
        lib().orc_init_populations(ctypes.byref(self.cfg_eq), _ptr(self.n), _ptr(self.u),
                                   _ptr(self.pop))

    def set_walls(self, walls, psi_w):
        """GetWalls (idpy/LBM/MultiPhase.py:157-162): flags (1 fluid, 0 wall,
        shape flip(dims)) and the psi field the walls keep."""
        self.walls = np.ascontiguousarray(np.asarray(walls, np.int32).ravel())
        self.psi_arr[:] = np.asarray(psi_w, np.float64).ravel()
        opp = [self.xi.index(tuple(-v for v in x)) for x in self.xi]
        self.opposite = np.array(opp, np.int32)

    def set_fluctuations(self, kind, indep, kBT, n0, seeds, tau, noise_literals=None, mode='round15'):
        """Gross et al. (2011) fluctuations (MainLoopGross2011SRT,
        idpy/LBM/MultiPhase.py:1404-1541): generator kind ('MINSTD', 'NUMREC',
        'MMIX'), one (indep False) or two (True) streams per random moment,
        seeds in the reference's CPU ordering (stream + cell * streams).  The
        noise operator comes from noise_terms (exact, 15-digit literals) or
        from the reference's own literals."""
        D, Q = self.D, self.Q
        nr = Q - (D + 1)
        if noise_literals is not None:
            terms, m2var = noise_from_literals(noise_literals)
        else:
            terms, norms = noise_terms(self.xi, self.w, self.c2, mode)
            omega = 1.0 / tau
            m2var = [-2.0 * noise_variance(nm, kBT, 1.0 / omega, n0) for nm in norms]
        self.noise_terms, self.noise_m2var = terms, m2var
        off, mom, coef = [0], [], []
        for tl in terms:
            for c, j in tl:
                coef.append(c)
                mom.append(j)
            off.append(len(coef))
        self._z_off = np.array(off, np.int32)
        self._z_mom = np.array(mom, np.int32)
        self._z_coef = np.array(coef, np.float64)
        self._z_m2var = np.array(m2var, np.float64)
        ns = 2 * nr if indep else nr
        seeds = np.asarray(seeds)
        if seeds.size != ns * self.V:
            raise ValueError('expected %d generator states' % (ns * self.V))
        self.seeds = np.ascontiguousarray(seeds.astype(np.uint64).ravel())
        self.seeds_dtype = seeds.dtype
        z = _Noise()
        z.kind, z.indep, z.nr = CRNG_KINDS[kind], int(bool(indep)), nr
        z.m2var, z.t_off, z.t_mom, z.t_coef = _ptr(self._z_m2var), _ptr(self._z_off), _ptr(self._z_mom), \
            _ptr(self._z_coef)
        self.noise = z

    def get_seeds(self):
        """Generator states in the reference's CPU ordering and dtype."""
        return self.seeds.astype(self.seeds_dtype)

    def run(self, nsteps):
        sw = ctypes.c_int(0)
        if getattr(self, 'noise', None) is not None:
            lib().orc_run_noise(ctypes.byref(self.cfg), ctypes.byref(self.noise), _ptr(self.pop), _ptr(self.pop_swap),
                                _ptr(self.n), _ptr(self.psi_arr), _ptr(self.seeds), int(nsteps), ctypes.byref(sw))
        elif getattr(self, 'walls', None) is not None:
            # MainLoopWalls (idpy/LBM/MultiPhase.py:1226-1309)
            lib().orc_run_walls(ctypes.byref(self.cfg), _ptr(self.pop), _ptr(self.pop_swap), _ptr(self.n),
                                _ptr(self.psi_arr), _ptr(self.walls), _ptr(self.opposite), int(nsteps),
                                ctypes.byref(sw))
        else:
            lib().orc_run(ctypes.byref(self.cfg), _ptr(self.pop), _ptr(self.pop_swap),
                          _ptr(self.n), _ptr(self.psi_arr), int(nsteps), ctypes.byref(sw))
        if sw.value:
            self.pop, self.pop_swap = self.pop_swap, self.pop

    def compute_moments(self):
        L = lib()
        L.orc_density_psi(ctypes.byref(self.cfg), _ptr(self.pop), _ptr(self.n),
                          _ptr(self.psi_arr))
        L.orc_velocity_after_force(ctypes.byref(self.cfg), _ptr(self.pop), _ptr(self.n),
                                   _ptr(self.psi_arr), _ptr(self.u))

    def density(self):
        return self.n.reshape(tuple(reversed(self.dims))).copy()

    def velocity(self):
        """(D, *flip(dims)), the reference's 'gpu' ordering shape."""
        return self.u.reshape(-1, self.D).T.reshape((self.D,) + tuple(reversed(self.dims))).copy()

    def populations(self):
        """(Q, *flip(dims))."""
        return self.pop.reshape(-1, self.Q).T.reshape((self.Q,) + tuple(reversed(self.dims))).copy()

    def set_populations(self, pop_soa):
        self.pop[:] = np.asarray(pop_soa, np.float64).reshape(self.Q, -1).T.ravel()

    def mass(self):
        return float(self.pop.sum())

    # --- observables (numpy) --------------------------------------------------
    def check_u(self):
        """CheckUConvergenceSCMP: (u_conv, max_u) after compute_moments()."""
        u = self.u.reshape(-1, self.D)
        if self.old_u is None:
            self.old_u = np.zeros_like(u)
        delta = np.zeros(self.V)
        norm = np.zeros(self.V)
        for d in range(self.D):
            norm += u[:, d] * u[:, d]
            delta += np.abs(u[:, d] - self.old_u[:, d])
        self.old_u = u.copy()
        return float(np.sum(delta) / self.V), float(np.sqrt(np.amax(norm) / self.c2))

    def delta_p(self, e2=1.0):
        """DeltaPLaplace: pressure at the box centre minus at index V-1."""
        strides = [1]
        for d in range(1, self.D):
            strides.append(strides[-1] * self.dims[d - 1])
        inside = sum((self.dims[d] // 2) * strides[d] for d in range(self.D))
        n_in, n_out = self.n[inside], self.n[self.V - 1]
        p = lambda n: n * self.c2 + 0.5 * self.G * e2 * psi_value(self.psi, n) ** 2
        return p(n_in), p(n_out), p(n_in) - p(n_out)


def psi_value(kind, n):
    if kind == 'exp':
        return math.exp(-1.0 / n)
    if kind == '1mexp':
        return 1.0 - math.exp(-n)
    return n


# ----------------------------------------------------------------------------
# initial profiles (reference kernels, FP64)
# ----------------------------------------------------------------------------

def _positions(dims):
    grids = np.meshgrid(*[np.arange(L) for L in reversed(dims)], indexing='ij')
    return [grids[len(dims) - 1 - d] for d in range(len(dims))]   # x, y, (z)


def init_radial(dims, n_g, n_l, R, full_flag=True):
    """K_InitRadialInterface: tanh(r - R) about L//2 (width 1)."""
    pos = _positions(dims)
    r2 = np.zeros(pos[0].shape, np.int64)
    for d, L in enumerate(dims):
        r2 += (L // 2 - pos[d]) * (L // 2 - pos[d])
    r = np.sqrt(r2.astype(np.float64))
    dn = (n_l - n_g) if full_flag else (n_g - n_l)
    return 0.5 * (n_g + n_l) - 0.5 * dn * np.tanh(r - R)


def init_flat(dims, n_g, n_l, width, direction=0, full_flag=True):
    """K_InitFlatInterface with F_NFlatProfilePeriodic."""
    pos = _positions(dims)
    x = pos[direction]
    L = dims[direction]
    x0 = L // 2
    xm = L // 2
    delta = x0 - xm
    if delta >= 0:
        xp = np.where(x < x0 - xm, x - (x0 - xm) + L, x - (x0 - xm))
    else:
        xp = np.where(x < x0 + xm, x - (x0 + xm) + L, x - (x0 + xm))
    prof = np.tanh(xp - (xm - 0.5 * width)) - np.tanh(xp - (xm + 0.5 * width))
    dn = (n_l - n_g) if full_flag else (n_g - n_l)
    return 0.5 * (n_g + n_l) + 0.5 * dn * (prof - 1.0)


def init_single_flat(dims, n_g, n_l, direction=0, full_flag=True):
    pos = _positions(dims)
    x = pos[direction]
    x0 = dims[direction] // 2
    dn = (n_l - n_g) if full_flag else (n_g - n_l)
    return n_g + dn * ((np.tanh((x - x0).astype(np.float64)) + 1.0) * 0.5)


def init_cylinder(dims, n_g, n_l, R, direction=0, full_flag=True):
    pos = _positions(dims)
    r2 = np.zeros(pos[0].shape, np.int64)
    for d, L in enumerate(dims):
        if d == direction:
            continue
        r2 += (L // 2 - pos[d]) * (L // 2 - pos[d])
    r = np.sqrt(r2.astype(np.float64))
    dn = (n_l - n_g) if full_flag else (n_g - n_l)
    return 0.5 * (n_g + n_l) - 0.5 * dn * np.tanh(r - R)


class _Simple(ctypes.Structure):
    _fields_ = [('dim', ctypes.c_int), ('L', ctypes.c_int * 3), ('Q', ctypes.c_int), ('QE', ctypes.c_int),
                ('xi', ctypes.c_void_p), ('w', ctypes.c_void_p), ('e', ctypes.c_void_p), ('we', ctypes.c_void_p),
                ('opposite', ctypes.c_void_p), ('G', ctypes.c_double), ('omega', ctypes.c_double),
                ('psi_kind', ctypes.c_int), ('forcing', ctypes.c_int), ('gravity', ctypes.c_int),
                ('g', ctypes.c_double), ('inout', ctypes.c_int), ('u_in', ctypes.c_double), ('order', ctypes.c_int)]


class OracleSimple:
    """The reference's "simple" step family on the CPU (q-major arrays, as its
    kernels index them): MainLoopSimple[SC] (no walls), MainLoopSimpleWalls[SC],
    MainLoopSimpleWallsGravity, MainLoopSimpleWallsInletOutlet[SC]
    (idpy/LBM/MultiPhase.py:164-1014).  forcing 'guo' or 'sc'; walls flags
    1 fluid, 0 wall, 2 inlet, 3 outlet (shape flip(dims)) or None."""

    def __init__(self, dims, xi, w, e, we, G, tau=1.0, psi='exp', walls=None, psi_w=None, forcing='guo',
                 gravity=None, u_in=None):
        self.dims = tuple(int(x) for x in dims)
        self.D, self.Q = len(self.dims), len(xi)
        self.V = int(np.prod(self.dims))
        xi = [tuple(int(v) for v in x) for x in xi]
        self._xi = np.array(xi, np.int32).ravel()
        self._w = np.array(w, np.float64)
        self._e = np.array(e, np.int32).ravel()
        self._we = np.array(we, np.float64)
        self._opp = np.array([xi.index(tuple(-v for v in x)) for x in xi], np.int32)
        self.walls = np.ones(self.V, np.int32) if walls is None else \
            np.ascontiguousarray(np.asarray(walls, np.int32).ravel())
        self.pop = np.zeros(self.Q * self.V)
        self.pop_b = np.zeros(self.Q * self.V)
        self.n = np.zeros(self.V)
        self.u = np.zeros(self.D * self.V)
        self.psi = np.zeros(self.V) if psi_w is None else np.array(psi_w, np.float64).ravel().copy()
        c = _Simple()
        c.dim = self.D
        for d in range(3):
            c.L[d] = self.dims[d] if d < self.D else 1
        c.Q, c.QE = self.Q, len(self._we)
        c.xi, c.w, c.e, c.we, c.opposite = _ptr(self._xi), _ptr(self._w), _ptr(self._e), _ptr(self._we), \
            _ptr(self._opp)
        c.G, c.omega, c.psi_kind = float(G), 1.0 / tau, PSI_KINDS[psi]
        c.forcing = {'guo': 0, 'sc': 1}[forcing]
        c.gravity, c.g = (0, 0.0) if gravity is None else (1, float(gravity))
        c.inout, c.u_in = (0, 0.0) if u_in is None else (1, float(u_in))
        # MainLoopSimpleWallsInletOutletSC: outlet, inlet, stream, bounce, moments, psi, collide
        c.order = 1 if (u_in is not None and forcing == 'sc') else 0
        self.cfg = c

    def set_state(self, pop, n, u=None):
        self.pop[:] = np.asarray(pop, np.float64).ravel()
        self.n[:] = np.asarray(n, np.float64).ravel()
        self.u[:] = 0.0 if u is None else np.asarray(u, np.float64).ravel()

    def run(self, nsteps):
        sw = ctypes.c_int(0)
        lib().orc_simple_run(ctypes.byref(self.cfg), _ptr(self.pop), _ptr(self.pop_b), _ptr(self.n), _ptr(self.u),
                             _ptr(self.psi), _ptr(self.walls), int(nsteps), ctypes.byref(sw))
        if sw.value:
            self.pop, self.pop_b = self.pop_b, self.pop
