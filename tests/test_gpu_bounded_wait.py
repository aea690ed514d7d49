"""The device waits of the single-pass variants are bounded: a wait on an
mbarrier whose phase cannot complete gives up, reports it, and leaves the
device usable (no fault, no hang)."""
import numpy as np
import pytest

from sclbm import _lib, XIStencils, FStencils
from sclbm.profiles import droplet

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_device_stays_usable():
    flag, ms = _lib.selftest_bounded_wait(0, 1 << 10)
    assert flag == 1, flag          # gave up; bit 2 would mean the phase completed
    assert 0.0 < ms < 2000.0, ms
    # the variants' full limit (2^18 polls, about a second), run only when the
    # measured time per poll puts it under a few seconds
    full_ms = ms * (1 << 8)
    print('bounded wait: 2^10 polls %.3f ms, 2^18 polls extrapolated %.1f ms' % (ms, full_ms))
    if full_ms < 3000.0:
        flag, ms_full = _lib.selftest_bounded_wait(0, 1 << 18)
        assert flag == 1, flag
        assert ms_full < 3000.0, ms_full
        print('bounded wait: 2^18 polls %.1f ms' % ms_full)
    # the context still steps a lattice
    x, f = XIStencils['D3Q19'], FStencils['D3E6']
    dims = (32, 24, 20)
    s = _lib.Sim(3, dims, x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], -4.5, precision=_lib.FP32_SHIFTED, rho0=0.2)
    s.set_density(droplet(dims, 6, 4.6, 0.2, 2.0, 1))
    s.set_velocity(np.zeros(3 * s.V))
    s.init_populations()
    s.step(10)
    assert np.isfinite(s.get_density()).all()
    s.close()


def test_bounded_wait_rejects_bad_arguments():
    with pytest.raises(_lib.SclbmError):
        _lib.selftest_bounded_wait(0, 0)
    with pytest.raises(_lib.SclbmError):
        _lib.selftest_bounded_wait(0, (1 << 18) + 1)
