"""Drop-in ``ShanChenMultiPhase``: the reference's class interface over the
sm_103a kernels of libsclbm.so.

Mirrors ``idpy.LBM.MultiPhase.ShanChenMultiPhase`` (idpy/LBM/MultiPhase.py:140-2175)
for the multiphase Shan-Chen path: same constructor keywords, the same
initialisers, ``MainLoop`` / ``MainLoopMRT`` with checkpoint lists and
convergence functions, ``ComputeMomentsMeta``, ``GetDensityField`` /
``GetVelocityField`` / ``GetPopulations``, ``DeltaPLaplace`` / ``PBulk`` and
``End``, with the same exceptions for missing parameters and uninitialised
state.  ``sims_idpy_memory['n'|'u'|'pop'|'psi']`` expose ``H2D`` / ``D2H`` /
``SetConst`` so scripts that set fields by hand keep working.

Differences: every array lives in HBM behind one ``sclbm_sim`` handle (SoA,
the reference's 'gpu' ordering); ``lang`` is accepted but there is one
backend, with no CPU fallback.  Extra keywords: ``precision`` ('fp64' or
'fp32_shifted'; ``fp32_flag=True`` selects the latter), ``rho0`` (shift of
the FP32 storage), ``literals`` ('round15' as the reference prints them, or
'exact'), ``collision_tables`` ((A, B) explicit operator, see include/sclbm.h).
"""
import time

import numpy as np

from . import _lib
from .LBM import identify_lattice, identify_stencil, STENCIL_ORDER

CUDA_T = 'cuda'

_PSI_CODES = {
    'exp(-1./ln_0)': _lib.PSI_EXP_INV,
    'exp(-1/ln_0)': _lib.PSI_EXP_INV,
    'exp(-1.0/ln_0)': _lib.PSI_EXP_INV,
    '1.-exp(-ln_0)': _lib.PSI_ONE_MINUS_EXP,
    '1-exp(-ln_0)': _lib.PSI_ONE_MINUS_EXP,
    '1.0-exp(-ln_0)': _lib.PSI_ONE_MINUS_EXP,
    'ln_0': _lib.PSI_IDENTITY,
}


def psi_kind_of(psi_code):
    """Map the reference's free-text ``psi_code`` to a built-in pseudopotential."""
    s = psi_code.replace(' ', '').replace('(PsiType)', '')
    while s.startswith('(') and s.endswith(')') and s.count('(') == s.count(')'):
        inner = s[1:-1]
        if inner.count('(') != inner.count(')'):
            break
        s = inner
    if s not in _PSI_CODES:
        raise Exception("psi_code %r is not one of the built-in pseudopotentials "
                        "exp(-1./ln_0), (1. - exp(-ln_0)), ln_0" % psi_code)
    return _PSI_CODES[s]


def _psi_numpy(kind):
    if kind == _lib.PSI_EXP_INV:
        return lambda n: np.exp(-1.0 / n)
    if kind == _lib.PSI_ONE_MINUS_EXP:
        return lambda n: 1.0 - np.exp(-n)
    return lambda n: n


def IndexFromPos(pos, dim_strides):
    index = pos[0]
    for i in range(1, len(pos)):
        index += pos[i] * dim_strides[i - 1]
    return index


def ComputeCenterOfMass(lbm, c_i=''):
    """(mass, centre of mass) of the density field (idpy/LBM/MultiPhase.py:108-137)."""
    mass, cm = lbm._sim.center_of_mass()
    return mass, cm


class _Field:
    """``IdpyArray``-like view of one device field of the handle."""

    def __init__(self, owner, name):
        self.owner, self.name = owner, name

    def H2D(self, array):
        s = self.owner._sim
        a = np.asarray(array, np.float64).ravel()
        if self.name == 'n':
            s.set_density(a)
        elif self.name == 'u':
            s.set_velocity(self.owner._u_to_planes(a))
        elif self.name == 'pop':
            s.set_populations(self.owner._pop_to_planes(a))
            self.owner.init_status['pop'] = True
        else:
            raise Exception("H2D of '%s' is not supported" % self.name)

    def SetConst(self, const):
        s = self.owner._sim
        if self.name == 'n':
            s.set_density(np.full(s.V, float(const)))
        elif self.name == 'u':
            s.set_velocity(np.full(s.V * s.dim, float(const)))
        else:
            raise Exception("SetConst of '%s' is not supported" % self.name)

    def D2H(self):
        s = self.owner._sim
        if self.name == 'n':
            return s.get_density()
        if self.name == 'u':
            return self.owner._u_from_planes(s.get_velocity())
        if self.name == 'pop':
            return self.owner._pop_from_planes(s.get_populations())
        raise Exception("D2H of '%s' is not supported" % self.name)


class ShanChenMultiPhase:
    verbose = True

    def __init__(self, *args, **kwargs):
        self.params_dict = dict(kwargs)
        p = self.params_dict
        for key, msg in [('dim_sizes', "Missing parameter 'dim_sizes'"),
                         ('xi_stencil', "Missing parameter 'xi_stencil'"),
                         ('f_stencil', "Missing 'f_stencil'"),
                         ('tau', "Missing 'tau'"),
                         ('SC_G', "Missing 'SC_G'"),
                         ('psi_code', "Missing 'psi_code', e.g. psi_code = '(PsiType) exp(-1/ln_0)'"),
                         ('lang', "Param lang = CUDA_T | OCL_T | CTYPES_T is needed"),
                         ('psi_sym', "Missing sympy expression for the pseudo-potential, parameter 'psi_sym'")]:
            if key not in p:
                raise Exception(msg)
        if p.get('set_ordering') not in ('gpu', 'cpu', None):
            raise Exception("Parameter 'set_ordering' must either be 'gpu' or 'cpu'")
        if p.get('set_ordering') is None:
            p['set_ordering'] = 'gpu'
        xi, fs = p['xi_stencil'], p['f_stencil']
        if identify_lattice(xi) is None:
            raise Exception('xi_stencil is not D2Q9 or D3Q19')
        sname = identify_stencil(fs)
        if sname is None:
            raise Exception('f_stencil is not one of the E4/E6/E8 force stencils')
        dims = tuple(int(x) for x in p['dim_sizes'])
        D = len(dims)
        es = fs.get('Es', fs.get('XIs'))
        self.psi_kind = psi_kind_of(p['psi_code'])
        precision = p.get('precision', 'fp32_shifted' if p.get('fp32_flag') else 'fp64')
        if precision not in ('fp64', 'fp32_shifted'):
            raise Exception("precision must be 'fp64' or 'fp32_shifted'")
        self.precision = precision
        lit = p.get('literals', 'round15')
        self.sims_vars = {
            'DIM': D, 'dim_sizes': np.array(dims, np.int32),
            'dim_strides': np.array([int(np.prod(dims[:i + 1])) for i in range(D - 1)], np.int32),
            'dim_center': np.array([L // 2 for L in dims], np.int32),
            'V': int(np.prod(dims)), 'Q': len(xi['XIs']),
            'XI_list': np.array(xi['XIs'], np.int32).ravel(), 'W_list': np.array(xi['Ws']),
            'c2': float(xi['c2']), 'tau': p['tau'], 'QE': len(es),
            'E_list': np.array(es, np.int32).ravel(), 'EW_list': np.array(fs['Ws']),
            'SC_G': p['SC_G'], 'e2_val': p.get('e2_val', 1), 'psi_sym': p['psi_sym'],
            'stencil': sname, 'stencil_order': STENCIL_ORDER[sname],
        }
        tables = p.get('collision_tables')
        self._sim = _lib.Sim(
            D, dims, xi['XIs'], xi['Ws'], xi['c2'], es, fs['Ws'], p['SC_G'],
            psi_kind=self.psi_kind, collision=_lib.COLL_BGK, tau=p['tau'],
            precision=_lib.FP32_SHIFTED if precision == 'fp32_shifted' else _lib.FP64,
            rho0=float(p.get('rho0', 1.0)),
            literals=_lib.LIT_EXACT if lit == 'exact' else _lib.LIT_ROUND15,
            device=int(p.get('device', 0) or 0),
            coll_a=None if tables is None else tables[0], coll_b=None if tables is None else tables[1])
        self._collision = ('tables',) if tables is not None else ('bgk', p['tau'])
        self.sims_idpy_memory = {k: _Field(self, k) for k in ('n', 'u', 'pop', 'psi')}
        self.init_status = {'n': False, 'u': False, 'pop': False}
        self.aux_vars = []

    # ---- layout helpers ------------------------------------------------------
    def _flip(self):
        return tuple(int(x) for x in np.flip(self.sims_vars['dim_sizes']))

    def _u_to_planes(self, a):
        if self.params_dict['set_ordering'] == 'cpu':
            return a.reshape(-1, self.sims_vars['DIM']).T.ravel()
        return a

    def _u_from_planes(self, a):
        if self.params_dict['set_ordering'] == 'cpu':
            return a.reshape(self.sims_vars['DIM'], -1).T.ravel()
        return a

    def _pop_to_planes(self, a):
        if self.params_dict['set_ordering'] == 'cpu':
            return a.reshape(-1, self.sims_vars['Q']).T.ravel()
        return a

    def _pop_from_planes(self, a):
        if self.params_dict['set_ordering'] == 'cpu':
            return a.reshape(self.sims_vars['Q'], -1).T.ravel()
        return a

    # ---- initialisation ------------------------------------------------------
    def InitPopulations(self):
        if not (self.init_status['n'] and self.init_status['u']):
            raise Exception("Fields u and n are not initialized")
        self._sim.init_populations()
        self.init_status['pop'] = True

    def _after_profile(self):
        self.init_status['n'] = self.init_status['u'] = self.init_status['pop'] = True

    def InitRadialInterface(self, n_g, n_l, R, full_flag=True):
        self.sims_vars.update(init_type='radial', n_g=n_g, n_l=n_l, full_flag=full_flag, R=R)
        self._sim.init_radial(n_g, n_l, R, full_flag)
        self._after_profile()

    def InitFlatInterface(self, n_g, n_l, width, direction=0, full_flag=True):
        self.sims_vars.update(init_type='flat', n_g=n_g, n_l=n_l, full_flag=full_flag, width=width,
                              direction=direction)
        self._sim.init_flat(n_g, n_l, width, direction, full_flag)
        self._after_profile()

    def InitSingleFlatInterface(self, n_g, n_l, direction=0, full_flag=True):
        self.sims_vars.update(init_type='flat', n_g=n_g, n_l=n_l, full_flag=full_flag, direction=direction)
        self._sim.init_single_flat(n_g, n_l, direction, full_flag)
        self._after_profile()

    def InitCylinderInterface(self, n_g, n_l, R, direction=0, full_flag=True):
        self.sims_vars.update(init_type='cylinder', n_g=n_g, n_l=n_l, full_flag=full_flag, R=R,
                              direction=direction)
        self._sim.init_cylinder(n_g, n_l, R, direction, full_flag)
        self._after_profile()

    # ---- main loops ------------------------------------------------------------
    def _check_init(self):
        if not all(self.init_status.values()):
            print(self.init_status)
            raise Exception("Hydrodynamic variables/populations not initialized")

    def _loop(self, time_steps, convergence_functions, profiling):
        old_step, prof = 0, {}
        steps = list(time_steps)
        for step in steps[1:]:
            if self.verbose:
                print("Step:", step)
            t0 = time.perf_counter()
            self._sim.step(step - old_step, sync=True)
            prof[step] = time.perf_counter() - t0
            old_step = step
            if len(convergence_functions):
                checks = [c_f(self) for c_f in convergence_functions]
                if any(checks):
                    break
        return prof if profiling else None

    def MainLoop(self, time_steps, convergence_functions=[], profiling=False):
        self._check_init()
        if self._collision != ('bgk', self.params_dict['tau']) and self._collision != ('tables',):
            self._sim.set_collision(_lib.COLL_BGK, tau=self.params_dict['tau'])
            self._collision = ('bgk', self.params_dict['tau'])
        return self._loop(time_steps, convergence_functions, profiling)

    def MainLoopMRT(self, time_steps, relaxation_matrix=None, omega_syms_vals=None,
                    convergence_functions=[], profiling=False):
        if relaxation_matrix is None:
            raise Exception("Missing argument 'relaxation_matrix'")
        if omega_syms_vals is None:
            raise Exception("Missing argument 'omega_syms_vals'")
        self._check_init()
        S = numeric_relaxation_matrix(relaxation_matrix, omega_syms_vals, self.sims_vars['Q'])
        key = ('mrt', S.tobytes())
        if self._collision != key:
            self._sim.set_collision(_lib.COLL_MRT, mrt_s=S)
            self._collision = key
        return self._loop(time_steps, convergence_functions, profiling)

    def GetWalls(self, walls, psi_w):
        """Wall flags (1 fluid, 0 wall; shape flip(dim_sizes)) and the psi
        field the walls keep (idpy/LBM/MultiPhase.py:157-162,
        idpy/LBM/LBM.py:609-631)."""
        walls = np.asarray(walls)
        if list(walls.shape) != list(self._flip()):
            raise Exception("walls must have shape %s" % (self._flip(),))
        self._sim.set_walls(walls, np.asarray(psi_w, np.float64))
        self._walls = True

    def MainLoopWalls(self, time_steps, convergence_functions=[], profiling=False):
        """MainLoop with the walls of GetWalls (idpy/LBM/MultiPhase.py:1226-1309):
        density and psi on fluid cells, halfway bounce-back at the walls."""
        if not getattr(self, '_walls', False):
            raise Exception("Walls not set (GetWalls)")
        return self.MainLoop(time_steps, convergence_functions, profiling)

    # ---- read-back / observables --------------------------------------------
    def ComputeMomentsMeta(self):
        if not self.init_status['pop']:
            raise Exception("Populations are not initialized")
        self._sim.compute_moments()
        self.init_status['n'] = True
        self.init_status['u'] = True

    def GetDensityField(self):
        return self._sim.get_density().reshape(self._flip())

    def GetVelocityField(self):
        u = self._sim.get_velocity()
        D = self.sims_vars['DIM']
        if self.params_dict['set_ordering'] == 'cpu':
            return u.reshape(D, -1).T.reshape(self._flip() + (D,))
        return u.reshape((D,) + self._flip())

    def GetPopulations(self):
        pop = self._sim.get_populations()
        Q = self.sims_vars['Q']
        if self.params_dict['set_ordering'] == 'cpu':
            return pop.reshape(Q, -1).T.reshape(self._flip() + (Q,))
        return pop.reshape((Q,) + self._flip())

    def PBulk(self, n):
        if 'psi_f' not in self.sims_vars:
            try:
                import sympy as sp
                self.sims_vars['psi_f'] = sp.lambdify(sp.Symbol('n'), self.sims_vars['psi_sym'])
            except Exception:
                self.sims_vars['psi_f'] = _psi_numpy(self.psi_kind)
        return (n * self.sims_vars['c2'] +
                0.5 * self.sims_vars['SC_G'] * self.sims_vars['e2_val'] * (self.sims_vars['psi_f'](n)) ** 2)

    def DeltaPLaplace(self, inside=None, outside=None):
        if inside is None:
            mass, cm = ComputeCenterOfMass(self)
            self.sims_vars['cm_coords'] = np.array(cm)
            self.sims_vars['mass'] = mass
            chk = any(abs(self.sims_vars['dim_center'][d] - cm[d]) > 1e-3 for d in range(self.sims_vars['DIM']))
            self.sims_vars['is_centered'] = not chk
            if chk and self.verbose:
                print("Center of mass: ", list(cm), "; Center of the system: ", self.sims_vars['dim_center'])
            inside = IndexFromPos(self.sims_vars['dim_center'].tolist(), self.sims_vars['dim_strides'])
        if outside is None:
            outside = self.sims_vars['V'] - 1
        n_in, n_out = self._sim.density_at([inside, outside])
        self.sims_vars['n_in_n_out'] = np.array([n_in, n_out])
        p_in, p_out = self.PBulk(n_in), self.PBulk(n_out)
        return p_in, p_out, p_in - p_out

    def MassMomentum(self):
        """Total mass (sum of all populations) and momentum, FP64 reductions on the device."""
        return self._sim.reductions()

    def End(self):
        self._sim.close()


def numeric_relaxation_matrix(relaxation_matrix, omega_syms_vals, Q):
    """The relaxation matrix with the omega values substituted, as a float array."""
    try:
        import sympy as sp
        M = sp.Matrix(relaxation_matrix)
        for sym, val in omega_syms_vals:
            M = M.subs(sym, val)
        S = np.array(M.evalf(), dtype=np.float64)
    except ImportError:
        S = np.array(relaxation_matrix, dtype=np.float64)
    if S.shape != (Q, Q):
        raise Exception('relaxation matrix must be %dx%d' % (Q, Q))
    return S
