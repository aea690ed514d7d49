"""sclbm_step_noalloc: one step into caller-owned device buffers, with the
scratch between the two passes in the library's fixed device array.

This entry point is for callers that cannot let the library allocate device
memory (a host that reserves its whole device-memory budget once in its own
pool, or a service that must not synchronize the device with an allocation or
free while stepping).  The test owns the population buffers itself (torch
tensors stand in for the caller's pool), calls the entry point twice in a row
through the C ABI, and checks both results against a handle stepped with
sclbm_step on the same kernels.  The file is collected last so that a run
stopping at the first failure has run every other test before it.
"""
import ctypes

import numpy as np
import pytest

from helpers import rel_err
from sclbm import _lib, XIStencils, FStencils
from sclbm.profiles import droplet

pytestmark = pytest.mark.gpu

MAX_CELLS = 1 << 20   # SCLBM_NOALLOC_MAX_CELLS


class _Params:
    """sclbm_params for a lattice; keeps the tables it points to alive."""

    def __init__(self, lat, st, dims, G, precision, rho0=0.0, tau=1.0, mrt_rates=None,
                 literals=_lib.LIT_ROUND15):
        x, f = XIStencils[lat], FStencils[st]
        self.keep = [np.ascontiguousarray(np.array(x['XIs'], np.int32).ravel()),
                     np.ascontiguousarray(np.array(x['Ws'], np.float64)),
                     np.ascontiguousarray(np.array(f['Es'], np.int32).ravel()),
                     np.ascontiguousarray(np.array(f['Ws'], np.float64))]
        p = _lib.Params()
        p.dim = len(dims)
        for d in range(3):
            p.sizes[d] = dims[d] if d < len(dims) else 1
        p.q = len(x['XIs'])
        p.xi, p.w, p.c2 = _lib.ptr(self.keep[0]), _lib.ptr(self.keep[1]), float(x['c2'])
        p.qe, p.e, p.we = len(f['Ws']), _lib.ptr(self.keep[2]), _lib.ptr(self.keep[3])
        p.sc_g, p.psi_kind, p.tau = float(G), _lib.PSI_EXP_INV, float(tau)
        if mrt_rates is not None:
            s = np.ascontiguousarray(np.diag(mrt_rates))
            self.keep.append(s)
            p.collision, p.mrt_s = _lib.COLL_MRT, _lib.ptr(s)
        else:
            p.collision = _lib.COLL_BGK
        p.precision, p.rho0, p.literals, p.device = precision, float(rho0), literals, 0
        self.p = p


def _step_noalloc(prm, src, dst):
    _lib.call('sclbm_step_noalloc', ctypes.byref(prm.p), ctypes.c_void_p(src.data_ptr()),
              ctypes.c_void_p(dst.data_ptr()), None)


CASES = {
    # FP64, the reference's literals and arithmetic
    'd2q9_e8_bgk_fp64': dict(lat='D2Q9', st='D2E8', dims=(96, 64), G=-5.0, precision=_lib.FP64, tol=1e-12),
    # FP32-shifted storage, general MRT rates, ragged 3D box
    'd3q19_e6_mrt_fp32': dict(lat='D3Q19', st='D3E6', dims=(40, 24, 20), G=-4.5, precision=_lib.FP32_SHIFTED,
                              rho0=1.0, mrt=True, tol=1e-6),
}


@pytest.mark.parametrize('case', sorted(CASES))
def test_step_noalloc_matches_handle_step(case):
    torch = pytest.importorskip('torch')
    c = CASES[case]
    x = XIStencils[c['lat']]
    dims, D, Q = c['dims'], len(c['dims']), len(x['XIs'])
    fp32 = c['precision'] == _lib.FP32_SHIFTED
    rho0 = c.get('rho0', 0.0)
    rates = np.array([1.0, 1.0, 1.0] + [1.1 + 0.02 * i for i in range(Q - 3)]) if c.get('mrt') else None
    prm = _Params(c['lat'], c['st'], dims, c['G'], c['precision'], rho0=rho0, mrt_rates=rates)
    kw = dict(collision=_lib.COLL_MRT, mrt_s=np.diag(rates)) if rates is not None else {}
    f = FStencils[c['st']]
    h = _lib.Sim(D, dims, x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], c['G'], precision=c['precision'],
                 rho0=rho0, **kw)
    h.set_tuning(_lib.PATH_TWO_PASS, 0)
    h.set_density(droplet(dims, min(dims) / 4, 4.6, 0.2, 2.0, 7))
    h.set_velocity(np.zeros(D * h.V))
    h.init_populations()
    f0 = h.get_populations()

    # the caller's own device buffers, in the storage of the chosen precision
    shift = np.repeat(np.asarray(x['Ws'], np.float64) * rho0, h.V) if fp32 else 0.0
    dtype = torch.float32 if fp32 else torch.float64
    store = (f0 - shift).astype(np.float32 if fp32 else np.float64)
    buf = [torch.from_numpy(store).to('cuda'), torch.empty(Q * h.V, dtype=dtype, device='cuda')]
    buf[1].fill_(float('nan'))
    for call in range(2):
        _step_noalloc(prm, buf[call % 2], buf[(call + 1) % 2])
        torch.cuda.synchronize()
        h.step(1)
        got = buf[(call + 1) % 2].cpu().numpy().astype(np.float64) + shift
        want = h.get_populations()
        assert np.isfinite(got).all(), call
        assert rel_err(got, want) <= c['tol'], (call, rel_err(got, want))
    h.close()


def test_step_noalloc_on_a_caller_stream():
    """Two calls enqueued back to back on a stream the caller created, with no
    host synchronisation between them: the second call's passes must run after
    the first's (same stream), and both results equal the handle's steps."""
    torch = pytest.importorskip('torch')
    x, f = XIStencils['D3Q19'], FStencils['D3E6']
    dims, Q = (24, 20, 16), 19
    prm = _Params('D3Q19', 'D3E6', dims, -4.5, _lib.FP64)
    h = _lib.Sim(3, dims, x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], -4.5)
    h.set_tuning(_lib.PATH_TWO_PASS, 0)
    h.set_density(droplet(dims, 5.0, 4.6, 0.2, 2.0, 9))
    h.set_velocity(np.zeros(3 * h.V))
    h.init_populations()
    f0 = h.get_populations()
    buf = [torch.from_numpy(f0).to('cuda'), torch.full((Q * h.V,), float('nan'), dtype=torch.float64, device='cuda')]
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    handle = ctypes.c_void_p(s.cuda_stream)
    for call in range(2):
        _lib.call('sclbm_step_noalloc', ctypes.byref(prm.p), ctypes.c_void_p(buf[call % 2].data_ptr()),
                  ctypes.c_void_p(buf[(call + 1) % 2].data_ptr()), handle)
    s.synchronize()
    h.step(2)
    got = buf[0].cpu().numpy()
    assert np.isfinite(got).all()
    assert rel_err(got, h.get_populations()) <= 1e-12
    h.close()


def test_step_noalloc_rejects_lattices_beyond_its_scratch():
    torch = pytest.importorskip('torch')
    a = torch.empty(9 * 8, dtype=torch.float64, device='cuda')
    b = torch.empty(9 * 8, dtype=torch.float64, device='cuda')
    prm = _Params('D2Q9', 'D2E4', (1025, 1024), -4.5, _lib.FP64)   # one column more than fits
    with pytest.raises(_lib.SclbmError) as e:
        _step_noalloc(prm, a, b)
    assert e.value.status == _lib.ERR_ARG and 'exceeds' in str(e.value)
    assert 1025 * 1024 > MAX_CELLS >= 1024 * 1024
