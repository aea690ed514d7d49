"""ctypes binding of libsclbm.so (include/sclbm.h).

There is no CPU fallback: if the library cannot be loaded, or no sm_100-family
GPU is present, every call raises.
"""
import ctypes
import os
import threading

import numpy as np

from . import build as _build

OK, ERR_ARG, ERR_UNSUPPORTED, ERR_CUDA, ERR_STATE, ERR_NOMEM, ERR_NODEVICE = range(7)
PSI_EXP_INV, PSI_ONE_MINUS_EXP, PSI_IDENTITY = 0, 1, 2
PATH_AUTO, PATH_TWO_PASS, PATH_FUSED, PATH_FUSED_PAIRS = 0, 1, 2, 3
COLL_BGK, COLL_MRT = 0, 1
FP64, FP32_SHIFTED = 0, 1
LIT_ROUND15, LIT_EXACT, LIT_FACTORED = 0, 1, 2
CRNG_NONE, CRNG_MINSTD, CRNG_NUMREC, CRNG_MMIX = 0, 1, 2, 3
CRNG_KINDS = {'MINSTD': CRNG_MINSTD, 'NUMREC': CRNG_NUMREC, 'MMIX': CRNG_MMIX}
SEEDS_STREAM_MAJOR, SEEDS_CELL_MAJOR = 0, 1
SIMPLE_OFF, SIMPLE_GUO, SIMPLE_SC = 0, 1, 2
TRANSFER_AUTO, TRANSFER_STAGED, TRANSFER_DIRECT = 0, 1, 2
STAGE_AUTO, STAGE_NONE, STAGE_HALO_ASYNC, STAGE_OWN_TMA = -1, 0, 1, 2


class SclbmError(RuntimeError):
    def __init__(self, fn, status, message):
        self.status = status
        super().__init__('%s failed (%d: %s): %s' % (fn, status, _STATUS.get(status, '?'), message))


_STATUS = {OK: 'ok', ERR_ARG: 'invalid argument', ERR_UNSUPPORTED: 'unsupported configuration',
           ERR_CUDA: 'CUDA error', ERR_STATE: 'call out of order', ERR_NOMEM: 'out of device memory',
           ERR_NODEVICE: 'no usable device'}


class Tuning(ctypes.Structure):
    _fields_ = [('path', ctypes.c_int), ('chunk', ctypes.c_int), ('staging', ctypes.c_int), ('tile', ctypes.c_int),
                ('order', ctypes.c_int), ('grid', ctypes.c_int)]


class Params(ctypes.Structure):
    _fields_ = [('dim', ctypes.c_int), ('sizes', ctypes.c_int * 3), ('q', ctypes.c_int),
                ('xi', ctypes.c_void_p), ('w', ctypes.c_void_p), ('c2', ctypes.c_double),
                ('qe', ctypes.c_int), ('e', ctypes.c_void_p), ('we', ctypes.c_void_p),
                ('sc_g', ctypes.c_double), ('psi_kind', ctypes.c_int), ('collision', ctypes.c_int),
                ('tau', ctypes.c_double), ('mrt_s', ctypes.c_void_p), ('precision', ctypes.c_int),
                ('rho0', ctypes.c_double), ('literals', ctypes.c_int), ('device', ctypes.c_int),
                ('coll_a', ctypes.c_void_p), ('coll_b', ctypes.c_void_p)]


_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_D = ctypes.c_double
_DP = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)
_I64P = ctypes.POINTER(ctypes.c_int64)

# name -> argtypes (all return int unless listed in _STR)
SIGNATURES = {
    'sclbm_monomial_count': [ctypes.c_int],
    'sclbm_version': [],
    'sclbm_status_string': [ctypes.c_int],
    'sclbm_last_error': [],
    'sclbm_create': [ctypes.POINTER(Params), ctypes.POINTER(_P)],
    'sclbm_destroy': [_P],
    'sclbm_info': [_P, _I64P, _I64P],
    'sclbm_set_density': [_P, _P],
    'sclbm_set_velocity': [_P, _P],
    'sclbm_get_density': [_P, _P],
    'sclbm_get_velocity': [_P, _P],
    'sclbm_get_populations': [_P, _P],
    'sclbm_set_populations': [_P, _P],
    'sclbm_set_collision': [_P, ctypes.c_int, _D, _P, _P, _P],
    'sclbm_init_populations': [_P],
    'sclbm_init_radial': [_P, _D, _D, _D, ctypes.c_int],
    'sclbm_init_flat': [_P, _D, _D, _D, ctypes.c_int, ctypes.c_int],
    'sclbm_init_single_flat': [_P, _D, _D, ctypes.c_int, ctypes.c_int],
    'sclbm_init_cylinder': [_P, _D, _D, _D, ctypes.c_int, ctypes.c_int],
    'sclbm_step': [_P, _I64],
    'sclbm_sync': [_P],
    'sclbm_step_timed': [_P, _I64, _DP],
    'sclbm_profile_step': [_P, _I64, _DP, ctypes.c_int],
    'sclbm_kernels_per_step': [_P, _IP],
    'sclbm_set_tuning': [_P, ctypes.c_int, ctypes.c_int],
    'sclbm_get_tuning': [_P, _IP, _IP, _IP],
    'sclbm_compute_moments': [_P],
    'sclbm_reductions': [_P, _DP, _DP],
    'sclbm_check_u': [_P, _DP, _DP],
    'sclbm_center_of_mass': [_P, _DP, _DP],
    'sclbm_density_at': [_P, _I64P, ctypes.c_int, _DP],
    'sclbm_density_finite': [_P, _IP, _DP],
    'sclbm_batch_create': [ctypes.POINTER(Params), ctypes.c_int, _P, _P, _P, ctypes.POINTER(_P)],
    'sclbm_batch_destroy': [_P],
    'sclbm_batch_info': [_P, _I64P, _I64P],
    'sclbm_batch_set_density': [_P, ctypes.c_int, _P],
    'sclbm_batch_get_density': [_P, ctypes.c_int, _P],
    'sclbm_batch_init_populations': [_P],
    'sclbm_batch_step': [_P, _I64],
    'sclbm_batch_step_timed': [_P, _I64, _DP],
    'sclbm_batch_check': [_P, _P, _P, _P],
    'sclbm_batch_set_active': [_P, _P],
    'sclbm_batch_steps': [_P, _P],
    'sclbm_batch_restore_mass': [_P, _P, _P],
    'sclbm_batch_init_lattice': [_P, ctypes.c_int],
    'sclbm_batch_probe': [_P, _P, _P],
    'sclbm_batch_set_probe_radius': [_P, ctypes.c_int],
    'sclbm_batch_set_tile_width': [_P, ctypes.c_int],
    'sclbm_batch_set_mass_compensation': [_P, ctypes.c_int],
    'sclbm_selftest_bounded_wait': [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                    ctypes.POINTER(ctypes.c_double)],
    'sclbm_restore_mass': [_P, _D, _DP],
    'sclbm_set_walls': [_P, _P, _P],
    'sclbm_noise_counts': [ctypes.c_int, ctypes.c_int, ctypes.c_int, _IP, _IP],
    'sclbm_noise_operator': [ctypes.POINTER(Params), _D, _D, _P, _P],
    'sclbm_set_fluctuations': [_P, ctypes.c_int, ctypes.c_int, _D, _D, _P, ctypes.c_int, _P, _P],
    'sclbm_get_seeds': [_P, _P, ctypes.c_int],
    'sclbm_set_simple': [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _D, ctypes.c_int, _D],
    'sclbm_set_transfer': [_P, ctypes.c_int, _IP],
    'sclbm_mlp_param_count': [_IP],
    'sclbm_mlp_create': [ctypes.c_int, ctypes.c_uint64, ctypes.POINTER(_P)],
    'sclbm_mlp_destroy': [_P],
    'sclbm_mlp_set_params': [_P, _P],
    'sclbm_mlp_get_params': [_P, _P],
    'sclbm_mlp_set_data': [_P, _I64, _P, _P],
    'sclbm_mlp_train': [_P, _I64, _I64, ctypes.c_float, _P],
    'sclbm_mlp_gradient': [_P, _I64, _P, _P, _P, _P],
    'sclbm_mlp_predict': [_P, _I64, _P, _P],
    'sclbm_step_noalloc': [ctypes.POINTER(Params), _P, _P, _P],
    'sclbm_set_tuning_ex': [_P, ctypes.POINTER(Tuning)],
    'sclbm_get_tuning_ex': [_P, ctypes.POINTER(Tuning)],
    'sclbm_autotune': [_P, ctypes.c_int, ctypes.POINTER(Tuning), _DP],
    'sclbm_clear_tuning_cache': [],
}
_STR = {'sclbm_version', 'sclbm_status_string', 'sclbm_last_error'}

_lock = threading.Lock()
_lib = None


def library_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load libsclbm.so (building it with nvcc if it is missing)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if not os.path.exists(path) and build_if_missing:
            _build.build()
        if not os.path.exists(path):
            raise ImportError('libsclbm.so not built (%s); run __graft_entry__.build()' % path)
        lib = ctypes.CDLL(path)
        for name, args in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = ctypes.c_char_p if name in _STR else ctypes.c_int
        _lib = lib
        return lib


def call(name, *args):
    lib = load()
    rc = getattr(lib, name)(*args)
    if rc != OK:
        raise SclbmError(name, rc, lib.sclbm_last_error().decode())
    return rc


def ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def selftest_bounded_wait(device=0, polls=1 << 16):
    """One block waits on an mbarrier that cannot complete and gives up after
    ``polls`` polls (the limit of the single-pass variants' waits is 2^18);
    returns (gave_up flag, milliseconds)."""
    flag, ms = ctypes.c_int(), ctypes.c_double()
    call('sclbm_selftest_bounded_wait', int(device), int(polls), ctypes.byref(flag), ctypes.byref(ms))
    return flag.value, ms.value


def dptr(a):
    return a.ctypes.data_as(_DP)


class Sim:
    """Owning wrapper of one sclbm_sim handle."""

    def __init__(self, dim, sizes, xi, w, c2, e, we, G, psi_kind=PSI_EXP_INV, collision=COLL_BGK,
                 tau=1.0, mrt_s=None, precision=FP64, rho0=0.0, literals=LIT_ROUND15, device=0,
                 coll_a=None, coll_b=None):
        self.dim = int(dim)
        self.sizes = tuple(int(s) for s in sizes)
        self.q = len(xi)
        self.V = int(np.prod(self.sizes))
        self._xi = np.ascontiguousarray(np.array(xi, np.int32).ravel())
        self._w = np.ascontiguousarray(np.array(w, np.float64))
        self._e = np.ascontiguousarray(np.array(e, np.int32).ravel())
        self._we = np.ascontiguousarray(np.array(we, np.float64))
        p = Params()
        p.dim = self.dim
        for d in range(3):
            p.sizes[d] = self.sizes[d] if d < self.dim else 1
        p.q = self.q
        p.xi, p.w, p.c2 = ptr(self._xi), ptr(self._w), float(c2)
        p.qe, p.e, p.we = len(we), ptr(self._e), ptr(self._we)
        p.sc_g, p.psi_kind, p.collision, p.tau = float(G), int(psi_kind), int(collision), float(tau)
        self._keep = []
        p.mrt_s = self._arr(mrt_s)
        p.precision, p.rho0, p.literals, p.device = int(precision), float(rho0), int(literals), int(device)
        p.coll_a, p.coll_b = self._arr(coll_a), self._arr(coll_b)
        self.precision = int(precision)
        h = ctypes.c_void_p()
        call('sclbm_create', ctypes.byref(p), ctypes.byref(h))
        self.h = h
        pa = ctypes.c_int()
        call('sclbm_set_transfer', self.h, TRANSFER_AUTO, ctypes.byref(pa))
        self._direct = bool(pa.value)   # read-backs go straight into (pageable) host arrays

    def _arr(self, a):
        if a is None:
            return None
        a = np.ascontiguousarray(np.asarray(a, np.float64))
        self._keep.append(a)
        return ptr(a)

    def close(self):
        if getattr(self, 'h', None):
            load().sclbm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # fields ---------------------------------------------------------------
    def set_density(self, n):
        n = np.ascontiguousarray(np.asarray(n, np.float64).ravel())
        assert n.size == self.V
        call('sclbm_set_density', self.h, ptr(n))

    def set_velocity(self, u):
        u = np.ascontiguousarray(np.asarray(u, np.float64).ravel())
        assert u.size == self.V * self.dim
        call('sclbm_set_velocity', self.h, ptr(u))

    def _out(self, out, n):
        if out is None:
            out = np.empty(n)
            if self._direct:
                # fault the pages in on the CPU (much faster than the device
                # faulting them in over the link on its first write)
                out.fill(0.0)
            return out
        assert out.dtype == np.float64 and out.size == n and out.flags['C_CONTIGUOUS']
        return out

    def get_density(self, out=None):
        out = self._out(out, self.V)
        call('sclbm_get_density', self.h, ptr(out))
        return out

    def get_velocity(self, out=None):
        out = self._out(out, self.V * self.dim)
        call('sclbm_get_velocity', self.h, ptr(out))
        return out

    def get_populations(self, out=None):
        out = self._out(out, self.V * self.q)
        call('sclbm_get_populations', self.h, ptr(out))
        return out

    def set_populations(self, pop):
        pop = np.ascontiguousarray(np.asarray(pop, np.float64).ravel())
        assert pop.size == self.V * self.q
        call('sclbm_set_populations', self.h, ptr(pop))

    def set_collision(self, collision, tau=1.0, mrt_s=None, coll_a=None, coll_b=None):
        call('sclbm_set_collision', self.h, int(collision), float(tau), self._arr(mrt_s),
             self._arr(coll_a), self._arr(coll_b))

    # init / step --------------------------------------------------------------
    def init_populations(self):
        call('sclbm_init_populations', self.h)

    def init_radial(self, n_g, n_l, R, full_flag=True):
        call('sclbm_init_radial', self.h, n_g, n_l, R, int(bool(full_flag)))

    def init_flat(self, n_g, n_l, width, direction=0, full_flag=True):
        call('sclbm_init_flat', self.h, n_g, n_l, width, int(direction), int(bool(full_flag)))

    def init_single_flat(self, n_g, n_l, direction=0, full_flag=True):
        call('sclbm_init_single_flat', self.h, n_g, n_l, int(direction), int(bool(full_flag)))

    def init_cylinder(self, n_g, n_l, R, direction=0, full_flag=True):
        call('sclbm_init_cylinder', self.h, n_g, n_l, R, int(direction), int(bool(full_flag)))

    def step(self, nsteps, sync=True):
        call('sclbm_step', self.h, int(nsteps))
        if sync:
            call('sclbm_sync', self.h)

    def sync(self):
        call('sclbm_sync', self.h)

    def step_timed(self, nsteps):
        ms = ctypes.c_double()
        call('sclbm_step_timed', self.h, int(nsteps), ctypes.byref(ms))
        return ms.value

    def profile_step(self, nsteps):
        ms = (ctypes.c_double * 2)()
        call('sclbm_profile_step', self.h, int(nsteps), ms, 2)
        return ms[0], ms[1]

    def kernels_per_step(self):
        c = ctypes.c_int()
        call('sclbm_kernels_per_step', self.h, ctypes.byref(c))
        return c.value

    def set_tuning(self, path=0, chunk=0):
        call('sclbm_set_tuning', self.h, int(path), int(chunk))

    def get_tuning(self):
        p, c, g = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        call('sclbm_get_tuning', self.h, ctypes.byref(p), ctypes.byref(c), ctypes.byref(g))
        return p.value, c.value, g.value

    def set_tuning_ex(self, path=PATH_AUTO, chunk=0, staging=STAGE_AUTO, tile=-1, order=-1):
        t = Tuning(int(path), int(chunk), int(staging), int(tile), int(order), 0)
        call('sclbm_set_tuning_ex', self.h, ctypes.byref(t))

    def get_tuning_ex(self):
        """dict(path, chunk, staging, tile, order, grid) of what runs"""
        t = Tuning()
        call('sclbm_get_tuning_ex', self.h, ctypes.byref(t))
        return dict(path=t.path, chunk=t.chunk, staging=t.staging, tile=t.tile, order=t.order, grid=t.grid)

    def autotune(self, trial_steps=20):
        """Time the bit-identical variants of this handle's step, apply and
        cache the fastest; returns (dict of the configuration, ms per step)."""
        t, ms = Tuning(), ctypes.c_double()
        call('sclbm_autotune', self.h, int(trial_steps), ctypes.byref(t), ctypes.byref(ms))
        return dict(path=t.path, chunk=t.chunk, staging=t.staging, tile=t.tile, order=t.order, grid=t.grid), ms.value

    def info(self):
        v, b = ctypes.c_int64(), ctypes.c_int64()
        call('sclbm_info', self.h, ctypes.byref(v), ctypes.byref(b))
        return v.value, b.value

    # observables -------------------------------------------------------------
    def compute_moments(self):
        call('sclbm_compute_moments', self.h)

    def reductions(self):
        m = ctypes.c_double()
        mom = (ctypes.c_double * 3)()
        call('sclbm_reductions', self.h, ctypes.byref(m), mom)
        return m.value, np.array(mom[:self.dim])

    def check_u(self):
        a, b = ctypes.c_double(), ctypes.c_double()
        call('sclbm_check_u', self.h, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def center_of_mass(self):
        m = ctypes.c_double()
        cm = (ctypes.c_double * 3)()
        call('sclbm_center_of_mass', self.h, ctypes.byref(m), cm)
        return m.value, tuple(cm[:self.dim])

    def density_at(self, idx):
        idx = np.ascontiguousarray(np.asarray(idx, np.int64).ravel())
        out = np.empty(idx.size)
        call('sclbm_density_at', self.h, idx.ctypes.data_as(_I64P), int(idx.size), dptr(out))
        return out

    def set_walls(self, walls, psi):
        """Wall flags (1 fluid, 0 wall) and the psi field the walls keep."""
        w = np.ascontiguousarray(np.asarray(walls, np.int32).ravel())
        p = np.ascontiguousarray(np.asarray(psi, np.float64).ravel())
        assert w.size == self.V and p.size == self.V
        call('sclbm_set_walls', self.h, ptr(w), ptr(p))

    def set_fluctuations(self, kind, indep, kBT, n0, seeds, layout=SEEDS_STREAM_MAJOR, m2var=None, coef=None):
        """Gross (2011) fluctuations: generator kind ('MINSTD', 'NUMREC', 'MMIX'
        or None to switch them off), seeds (uint32 / uint64 for MMIX, V x streams
        in the given layout), optional explicit operator (m2var[nr], coef[q, nr])."""
        if kind is None:
            call('sclbm_set_fluctuations', self.h, CRNG_NONE, 0, 0.0, 0.0, None, 0, None, None)
            self.noise = None
            return
        k = CRNG_KINDS[kind] if isinstance(kind, str) else int(kind)
        nr, ns = noise_counts(self.dim, self.q, indep)
        dt = np.uint64 if k == CRNG_MMIX else np.uint32
        seeds = np.ascontiguousarray(np.asarray(seeds).astype(dt).ravel())
        assert seeds.size == ns * self.V, (seeds.size, ns * self.V)
        mv = None if m2var is None else np.ascontiguousarray(np.asarray(m2var, np.float64).ravel())
        cf = None if coef is None else np.ascontiguousarray(np.asarray(coef, np.float64).ravel())
        if mv is not None:
            assert mv.size == nr and cf.size == self.q * nr
        call('sclbm_set_fluctuations', self.h, k, int(bool(indep)), float(kBT), float(n0), ptr(seeds), int(layout),
             None if mv is None else ptr(mv), None if cf is None else ptr(cf))
        self.noise = (k, ns, dt)

    def get_seeds(self, layout=SEEDS_STREAM_MAJOR):
        k, ns, dt = self.noise
        out = np.empty(ns * self.V, dt)
        call('sclbm_get_seeds', self.h, ptr(out), int(layout))
        return out

    def set_simple(self, forcing, use_walls=False, gravity=None, inlet_outlet=False, u_in=0.0):
        """The reference's simple step family: forcing SIMPLE_GUO / SIMPLE_SC
        (SIMPLE_OFF: back to the generated-kernel step), gravity along y (Guo),
        inlet / outlet wall flags 2 / 3 with inlet velocity u_in."""
        call('sclbm_set_simple', self.h, int(forcing), int(bool(use_walls)), int(gravity is not None),
             float(gravity or 0.0), int(bool(inlet_outlet)), float(u_in))

    def set_transfer(self, mode):
        """TRANSFER_AUTO / _STAGED / _DIRECT; returns whether the device can
        access pageable host memory."""
        pa = ctypes.c_int()
        call('sclbm_set_transfer', self.h, int(mode), ctypes.byref(pa))
        self._direct = bool(pa.value) and int(mode) != TRANSFER_STAGED
        return bool(pa.value)

    def restore_mass(self, target=float('nan')):
        """FP64 mass before; if target is finite, restore it (rest populations)."""
        m = ctypes.c_double()
        call('sclbm_restore_mass', self.h, float(target), ctypes.byref(m))
        return m.value

    def density_finite(self):
        f, m = ctypes.c_int(), ctypes.c_double()
        call('sclbm_density_finite', self.h, ctypes.byref(f), ctypes.byref(m))
        return bool(f.value), m.value


def clear_tuning_cache():
    call('sclbm_clear_tuning_cache')


def monomial_count(dim):
    return load().sclbm_monomial_count(int(dim))


def noise_counts(dim, q, indep):
    """(random moments, generator states per cell)."""
    m, n = ctypes.c_int(), ctypes.c_int()
    call('sclbm_noise_counts', int(dim), int(q), int(bool(indep)), ctypes.byref(m), ctypes.byref(n))
    return m.value, n.value


def noise_operator(dim, xi, w, c2, tau, kBT, n0, literals=LIT_ROUND15):
    """Host-side noise operator (m2var[nr], coef[q, nr]) for a BGK lattice."""
    xi_a = np.ascontiguousarray(np.array(xi, np.int32).ravel())
    w_a = np.ascontiguousarray(np.array(w, np.float64))
    q = len(w_a)
    p = Params()
    p.dim, p.q, p.xi, p.w, p.c2 = int(dim), q, ptr(xi_a), ptr(w_a), float(c2)
    p.tau, p.literals = float(tau), int(literals)
    nr = q - int(dim) - 1
    mv, cf = np.empty(nr), np.empty(q * nr)
    call('sclbm_noise_operator', ctypes.byref(p), float(kBT), float(n0), ptr(mv), ptr(cf))
    return mv, cf.reshape(q, nr)
