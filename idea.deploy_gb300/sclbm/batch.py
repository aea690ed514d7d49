"""Batches of independent periodic lattices (ragged droplet sweeps).

Wraps ``sclbm_batch_*`` (include/sclbm.h): lattices of different sizes,
couplings G and FP32 shifts live in one SoA array and are stepped by one
launch per step; converged lattices are retired individually.  The reference
has no counterpart: it runs one ``ShanChenMultiPhase`` per droplet
(idpy/LBM/MultiPhase.py:140), each stepping the same update as this batch.
"""
import ctypes

import numpy as np

from . import _lib
from .LBM import XIStencils, FStencils
from .MultiPhase import psi_kind_of


class Batch:
    """``n`` lattices of one lattice type / force stencil / BGK tau.

    ``sizes``: list of per-lattice sizes (x first); ``G``, ``rho0``: per lattice.
    """

    def __init__(self, xi_stencil, f_stencil, sizes, G, rho0, tau=1.0, psi_code='exp(-1./ln_0)', device=0):
        self.sizes = [tuple(int(v) for v in s) for s in sizes]
        self.n = len(self.sizes)
        self.dim = len(self.sizes[0])
        es = f_stencil.get('Es', f_stencil.get('XIs'))
        self._xi = np.ascontiguousarray(np.array(xi_stencil['XIs'], np.int32).ravel())
        self._w = np.ascontiguousarray(np.array(xi_stencil['Ws'], np.float64))
        self._e = np.ascontiguousarray(np.array(es, np.int32).ravel())
        self._we = np.ascontiguousarray(np.array(f_stencil['Ws'], np.float64))
        self.c2 = float(xi_stencil['c2'])
        p = _lib.Params()
        p.dim = self.dim
        p.q = len(xi_stencil['XIs'])
        p.xi, p.w, p.c2 = _lib.ptr(self._xi), _lib.ptr(self._w), self.c2
        p.qe, p.e, p.we = len(es), _lib.ptr(self._e), _lib.ptr(self._we)
        p.psi_kind = psi_kind_of(psi_code)
        p.collision, p.tau = _lib.COLL_BGK, float(tau)
        p.precision, p.device = _lib.FP32_SHIFTED, int(device)
        self._sizes = np.ascontiguousarray(np.array(self.sizes, np.int32).ravel())
        self.G = np.ascontiguousarray(np.asarray(G, np.float64))
        self.rho0 = np.ascontiguousarray(np.asarray(rho0, np.float64))
        h = ctypes.c_void_p()
        _lib.call('sclbm_batch_create', ctypes.byref(p), self.n, _lib.ptr(self._sizes), _lib.ptr(self.G),
                  _lib.ptr(self.rho0), ctypes.byref(h))
        self.h = h
        self.active = np.ones(self.n, np.int32)

    def close(self):
        if getattr(self, 'h', None):
            _lib.load().sclbm_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def cells(self, i):
        return int(np.prod(self.sizes[i]))

    def info(self):
        c, b = ctypes.c_int64(), ctypes.c_int64()
        _lib.call('sclbm_batch_info', self.h, ctypes.byref(c), ctypes.byref(b))
        return c.value, b.value

    def set_density(self, i, n):
        n = np.ascontiguousarray(np.asarray(n, np.float64).ravel())
        assert n.size == self.cells(i)
        _lib.call('sclbm_batch_set_density', self.h, int(i), _lib.ptr(n))

    def get_density(self, i):
        out = np.empty(self.cells(i))
        _lib.call('sclbm_batch_get_density', self.h, int(i), _lib.ptr(out))
        return out.reshape(tuple(reversed(self.sizes[i])))

    def init_populations(self):
        _lib.call('sclbm_batch_init_populations', self.h)

    def init_lattice(self, i):
        """Equilibrium populations of lattice i alone from its last set density."""
        _lib.call('sclbm_batch_init_lattice', self.h, int(i))

    def step(self, nsteps, sync=True):
        _lib.call('sclbm_batch_step', self.h, int(nsteps))
        if sync:
            self.check_only_sync()

    def check_only_sync(self):
        # a zero-step timed call waits for the stream
        ms = ctypes.c_double()
        _lib.call('sclbm_batch_step_timed', self.h, 0, ctypes.byref(ms))

    def step_timed(self, nsteps):
        ms = ctypes.c_double()
        _lib.call('sclbm_batch_step_timed', self.h, int(nsteps), ctypes.byref(ms))
        return ms.value

    def check(self):
        """Per-lattice (u_conv, max_u, mass); retired lattices keep NaN."""
        uc, mu, m = (np.full(self.n, np.nan) for _ in range(3))
        _lib.call('sclbm_batch_check', self.h, _lib.ptr(uc), _lib.ptr(mu), _lib.ptr(m))
        return uc, mu, m

    def restore_mass(self, target=None):
        """Per-lattice FP64 mass before; where target is finite, restore it."""
        t = np.full(self.n, np.nan) if target is None else np.ascontiguousarray(np.asarray(target, np.float64))
        before = np.full(self.n, np.nan)
        _lib.call('sclbm_batch_restore_mass', self.h, _lib.ptr(t), _lib.ptr(before))
        return before

    def set_tile_width(self, tx):
        """2D batches: 0 (256-cell tiles, the default) or 64; bit-identical results."""
        _lib.call('sclbm_batch_set_tile_width', self.h, int(tx))

    def set_mass_compensation(self, on):
        """Compensated rest population (default on); off only for 3D batches
        with paired halo loads."""
        _lib.call('sclbm_batch_set_mass_compensation', self.h, int(bool(on)))

    def set_probe_radius(self, rad):
        """probe() returns means over the cube of side 2 rad + 1 about each cell."""
        _lib.call('sclbm_batch_set_probe_radius', self.h, int(rad))

    def probe(self):
        """Per-lattice density at the centre cell and at the last cell."""
        a, b = np.full(self.n, np.nan), np.full(self.n, np.nan)
        _lib.call('sclbm_batch_probe', self.h, _lib.ptr(a), _lib.ptr(b))
        return a, b

    def set_active(self, active):
        self.active = np.ascontiguousarray(np.asarray(active, np.int32))
        _lib.call('sclbm_batch_set_active', self.h, _lib.ptr(self.active))

    def steps(self):
        out = np.zeros(self.n, np.int64)
        _lib.call('sclbm_batch_steps', self.h, _lib.ptr(out))
        return out
