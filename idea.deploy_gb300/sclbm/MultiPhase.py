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
the FP32 storage), ``literals`` ('round15' as the reference prints them,
'exact', or 'factored': exact, with the FP64 BGK operator factored by
opposite directions), ``collision_tables`` ((A, B) explicit operator, see include/sclbm.h),
``noise_tables`` ((m2var, coef) explicit noise operator of the fluctuating step).

Fluctuations (``fluctuations='Gross2011'`` with ``prng_kind``, ``init_seed``,
``prng_init_from``, ``prng_distribution``, ``indep_gaussian``, then
``MainLoopGross2011SRT``, idpy/LBM/MultiPhase.py:1404-1541,2029-2069): the
generator states are drawn as the reference's CRNGS draws them
(idpy/PRNGS/CRNGS.py:289-337, numpy's legacy seeding) and mapped to cells by
the same ordering, so a run started from the same seed follows the reference's
random stream.  ``crng.sims_idpy_memory['seeds'].D2H()`` reads them back.  The
``flat`` distribution is refused: the reference's code generator fails on it
(its variances are strings, CRNGS.py:903 with Fluctuations.py:87-97).
"""
import os
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
    # the simple step family's kernels name the density ln
    'exp(-1./ln)': _lib.PSI_EXP_INV,
    'exp(-1/ln)': _lib.PSI_EXP_INV,
    'exp(-1.0/ln)': _lib.PSI_EXP_INV,
    '1.-exp(-ln)': _lib.PSI_ONE_MINUS_EXP,
    '1-exp(-ln)': _lib.PSI_ONE_MINUS_EXP,
    '1.0-exp(-ln)': _lib.PSI_ONE_MINUS_EXP,
    'ln': _lib.PSI_IDENTITY,
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
            literals={'exact': _lib.LIT_EXACT, 'factored': _lib.LIT_FACTORED}.get(lit, _lib.LIT_ROUND15),
            device=int(p.get('device', 0) or 0),
            coll_a=None if tables is None else tables[0], coll_b=None if tables is None else tables[1])
        self._collision = ('tables',) if tables is not None else ('bgk', p['tau'])
        self.sims_idpy_memory = {k: _Field(self, k) for k in ('n', 'u', 'pop', 'psi')}
        self.init_status = {'n': False, 'u': False, 'pop': False}
        self.aux_vars = []
        self.crng = None
        if p.get('fluctuations') is not None:
            self._init_fluctuations()

    # ---- fluctuations ------------------------------------------------------------
    def _init_fluctuations(self):
        """InitMemory's fluctuation branch (idpy/LBM/MultiPhase.py:2029-2069)."""
        p = self.params_dict
        if p['fluctuations'] != 'Gross2011':
            raise Exception("Parameter 'fluctuations' must be 'Gross2011'")
        for key in ('prng_kind', 'prng_distribution'):
            if key not in p:
                raise Exception("Missing parameter '%s'" % key)
        if p['prng_kind'] not in _lib.CRNG_KINDS:
            raise Exception("'prng_kind' must be one of %s" % sorted(_lib.CRNG_KINDS))
        if p['prng_distribution'] not in ('flat', 'gaussian'):
            raise Exception("Parameter 'distribution' must be in ['flat', 'gaussian']")
        if p['prng_distribution'] == 'flat':
            raise Exception("the 'flat' distribution of the fluctuating step is not available: the "
                            "reference's code generator fails on it (string variances)")
        init_from = p.get('prng_init_from', 'numpy')
        if init_from not in ('numpy', 'urandom'):
            raise Exception("'init_from' must be either 'numpy' or 'urandom'")
        indep = bool(p.get('indep_gaussian', False))
        nr, ns = _lib.noise_counts(self.sims_vars['DIM'], self.sims_vars['Q'], indep)
        V = self.sims_vars['V']
        self.crng = CRNGS(p['prng_kind'], ns * V, init_from, p.get('init_seed', 1), self)
        self.sims_vars['N_PRNG_STREAMS'] = ns
        self._noise = dict(indep=indep, streams=ns, moments=nr, key=None)

    def _seeds_layout(self):
        return _lib.SEEDS_CELL_MAJOR if self.params_dict['set_ordering'] == 'cpu' else _lib.SEEDS_STREAM_MAJOR

    def _noise_on(self, kBT, n0):
        nz = self._noise
        key = (float(kBT), float(n0), self._collision)
        if nz['key'] == key:
            return
        seeds = self.crng._host_seeds()
        tables = self.params_dict.get('noise_tables')
        self._sim.set_fluctuations(self.params_dict['prng_kind'], nz['indep'], kBT, n0, seeds, self._seeds_layout(),
                                   None if tables is None else tables[0], None if tables is None else tables[1])
        self.crng._on_device = True
        nz['key'] = key

    def _noise_off(self):
        if self.crng is None or self._noise['key'] is None:
            return
        self.crng._cache = self._sim.get_seeds(self._seeds_layout())
        self.crng._on_device = False
        self._sim.set_fluctuations(None, False, 0.0, 0.0, None)
        self._noise['key'] = None

    def MainLoopGross2011SRT(self, time_steps, convergence_functions=[], convergence_functions_args=[],
                             profiling=False, kBT=None, n0=None, print_flag=True):
        """The fluctuating step of Gross et al. (2011) with the BGK collision
        (idpy/LBM/MultiPhase.py:1404-1541): every step adds the noise
        populations of the Gaussian random moments drawn from the cells'
        generators."""
        if kBT is None:
            raise Exception("Missing parameter 'kBT'")
        elif kBT < 0:
            raise Exception("Paramter 'kBT' must be positive")
        if n0 is None:
            raise Exception("Missing parameter 'n0'")
        if self.crng is None:
            raise Exception("Fluctuations not set up: construct with fluctuations='Gross2011'")
        self._check_init()
        self._simple_off()
        if self._collision != ('bgk', self.params_dict['tau']):
            self._sim.set_collision(_lib.COLL_BGK, tau=self.params_dict['tau'])
            self._collision = ('bgk', self.params_dict['tau'])
        self._noise_on(kBT, n0)
        old_step, prof = 0, {}
        self.sims_vars['time_steps'] = []
        for step in list(time_steps)[1:]:
            if print_flag and self.verbose:
                print("Step:", step)
            t0 = time.perf_counter()
            self._sim.step(step - old_step, sync=True)
            prof[step] = time.perf_counter() - t0
            self.sims_vars['time_steps'].append(step)
            old_step = step
            if len(convergence_functions):
                if len(convergence_functions_args):
                    checks = [c_f(self, **convergence_functions_args[i]) for i, c_f in enumerate(convergence_functions)]
                else:
                    checks = [c_f(self) for c_f in convergence_functions]
                if any(checks):
                    break
        self.sims_vars['time_steps'] = np.array(self.sims_vars['time_steps'])
        return prof if profiling else None

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
        self._noise_off()
        self._simple_off()
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
        self._noise_off()
        self._simple_off()
        S = numeric_relaxation_matrix(relaxation_matrix, omega_syms_vals, self.sims_vars['Q'])
        key = ('mrt', S.tobytes())
        # explicit operator tables given at construction (collision_tables) are
        # the operator to run, as in MainLoop
        if self._collision != key and self._collision != ('tables',):
            self._sim.set_collision(_lib.COLL_MRT, mrt_s=S)
            self._collision = key
        return self._loop(time_steps, convergence_functions, profiling)

    def GetWalls(self, walls, psi_w):
        """Wall flags (1 fluid, 0 wall; shape flip(dim_sizes)) and the psi
        field the walls keep (idpy/LBM/MultiPhase.py:157-162,
        idpy/LBM/LBM.py:609-631)."""
        walls = np.asarray(walls)
        self._noise_off()
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

    # ---- the simple step family (MainLoopSimple*, idpy/LBM/MultiPhase.py:164-1014) ----
    def _simple_off(self):
        if getattr(self, '_simple', None) is not None:
            self._sim.set_simple(_lib.SIMPLE_OFF)
            self._simple = None

    def _simple_loop(self, key, time_steps, convergence_functions, profiling, convergence_functions_args=()):
        forcing, use_walls, gravity, inout, u_in = key
        if use_walls and not getattr(self, '_walls', False):
            raise Exception("Walls not set (GetWalls)")
        self._check_init()
        self._noise_off()
        if self._collision != ('bgk', self.params_dict['tau']):
            self._sim.set_collision(_lib.COLL_BGK, tau=self.params_dict['tau'])
            self._collision = ('bgk', self.params_dict['tau'])
        if getattr(self, '_simple', None) != key:
            self._sim.set_simple(forcing, use_walls=use_walls, gravity=gravity, inlet_outlet=inout, u_in=u_in)
            self._simple = key
        if convergence_functions_args:
            fns = [lambda lbm, f=f, kw=kw: f(lbm, **kw) for f, kw in zip(convergence_functions,
                                                                          convergence_functions_args)]
        else:
            fns = convergence_functions
        return self._loop(time_steps, fns, profiling)

    def MainLoopSimple(self, time_steps, convergence_functions=[], profiling=False):
        """Moments, psi, in-place BGK collision with Guo forcing, periodic
        stream (idpy/LBM/MultiPhase.py:164-255)."""
        return self._simple_loop((_lib.SIMPLE_GUO, False, None, False, 0.0), time_steps, convergence_functions,
                                 profiling)

    def MainLoopSimpleSC(self, time_steps, convergence_functions=[], profiling=False):
        """As MainLoopSimple with the Shan-Chen velocity shift
        (u_eq = u + F/(n omega); idpy/LBM/MultiPhase.py:257-349)."""
        return self._simple_loop((_lib.SIMPLE_SC, False, None, False, 0.0), time_steps, convergence_functions,
                                 profiling)

    def MainLoopSimpleWalls(self, time_steps, convergence_functions=[], profiling=False):
        """MainLoopSimple on the fluid cells of GetWalls with halfway
        bounce-back (idpy/LBM/MultiPhase.py:351-465)."""
        return self._simple_loop((_lib.SIMPLE_GUO, True, None, False, 0.0), time_steps, convergence_functions,
                                 profiling)

    def MainLoopSimpleWallsSC(self, time_steps, convergence_functions=[], profiling=False):
        """(idpy/LBM/MultiPhase.py:467-581)"""
        return self._simple_loop((_lib.SIMPLE_SC, True, None, False, 0.0), time_steps, convergence_functions,
                                 profiling)

    def MainLoopSimpleWallsGravity(self, time_steps, convergence_functions=[], g=0, profiling=False):
        """MainLoopSimpleWalls with gravity g added to F_y of every non-wall
        cell (idpy/LBM/MultiPhase.py:888-1013)."""
        return self._simple_loop((_lib.SIMPLE_GUO, True, float(g), False, 0.0), time_steps,
                                 convergence_functions, profiling)

    def MainLoopSimpleWallsInletOutlet(self, time_steps, convergence_functions=[], profiling=False, n_in=1, u_in=0,
                                       tau_in=100, max_mult=2):
        """Walls with an inlet (flag 2: n = 2, u = (u_in, 0, ..), equilibrium)
        and an outlet (flag 3: the cell at x - 1) (idpy/LBM/MultiPhase.py:583-733).
        n_in, tau_in and max_mult are accepted and unused, as in the
        reference's inlet kernel (LBMKernels.py:299-357)."""
        return self._simple_loop((_lib.SIMPLE_GUO, True, None, True, float(u_in)), time_steps,
                                 convergence_functions, profiling)

    def MainLoopSimpleWallsInletOutletSC(self, time_steps, convergence_functions=[], convergence_functions_args=[],
                                         profiling=False, n_in=1, u_in=0, tau_in=100, max_mult=2):
        """The Shan-Chen-forcing inlet/outlet loop; it streams before it
        collides (idpy/LBM/MultiPhase.py:735-887)."""
        return self._simple_loop((_lib.SIMPLE_SC, True, None, True, float(u_in)), time_steps,
                                 convergence_functions, profiling, convergence_functions_args)

    # ---- read-back / observables --------------------------------------------
    def ComputeMomentsMeta(self):
        if not self.init_status['pop']:
            raise Exception("Populations are not initialized")
        self._sim.compute_moments()
        self.init_status['n'] = True
        self.init_status['u'] = True

    def GetDensityField(self, out=None):
        """The density field (shape flip(dim_sizes)).  out: an optional
        float64 array of V values to read into (e.g. pinned memory reused
        across calls); the result is then a view of it."""
        flat = None if out is None else np.asarray(out).reshape(-1)
        return self._sim.get_density(flat).reshape(self._flip())

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


class CRNGS:
    """The generator states of the fluctuating step, drawn as the reference's
    ``CRNGS.InitSeeds`` draws them (idpy/PRNGS/CRNGS.py:289-337): numpy's
    legacy generator seeded with ``init_seed`` (one stream), integers in
    [1, RANDMAX) of the generator's state type, or 4 bytes of ``os.urandom``
    each; MINSTD states masked to 31 bits.  Entry i of the array belongs to
    (cell, stream) by the simulation's ordering: 'gpu' i = cell + stream * V,
    'cpu' i = stream + cell * streams (MultiPhase.py:1962-1965)."""
    RANDMAX = {'MINSTD': 0x7fffffff, 'NUMREC': 0xffffffff, 'MMIX': 0xffffffffffffffff}

    def __init__(self, kind, n_prngs, init_from, init_seed, owner):
        self.owner = owner
        dt = np.uint64 if kind == 'MMIX' else np.uint32
        if init_from == 'numpy':
            np.random.seed(int(init_seed))
            seeds = np.random.randint(low=1, high=self.RANDMAX[kind], size=int(n_prngs), dtype=dt)
        else:
            seeds = np.array([int.from_bytes(os.urandom(4), byteorder='big', signed=False)
                              for _ in range(int(n_prngs))], dt)
        if kind == 'MINSTD':
            seeds &= dt(self.RANDMAX[kind])
        self.sims_vars = {'kind': kind, 'n_prngs': int(n_prngs), 'init_from': init_from,
                          'init_seed': init_seed, 'ID_RANDMAX': self.RANDMAX[kind], 'n_streams': 1}
        self.constants = {'ID_RANDMAX': self.RANDMAX[kind], 'N_PRNGS': int(n_prngs)}
        self._cache = seeds
        self._on_device = False
        self.sims_idpy_memory = {'seeds': _SeedsField(self)}

    def _host_seeds(self):
        if self._on_device:
            return self.owner._sim.get_seeds(self.owner._seeds_layout())
        return self._cache


class _SeedsField:
    def __init__(self, crng):
        self.crng = crng

    def D2H(self):
        return self.crng._host_seeds().copy()

    def H2D(self, array):
        c = self.crng
        a = np.asarray(array).astype(c._cache.dtype).ravel()
        if a.size != c._cache.size:
            raise Exception('expected %d generator states' % c._cache.size)
        c._cache = a.copy()
        if c._on_device:   # fluctuations running: upload the new states now
            kBT, n0, _ = c.owner._noise['key']
            c.owner._noise['key'] = None
            c._on_device = False
            c.owner._noise_on(kBT, n0)


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
