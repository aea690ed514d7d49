"""Host <-> device transfers of the field arrays (sclbm_set_transfer): the
direct path (a kernel reads / writes the caller's FP64 array: pinned memory,
or pageable memory where the device reaches it over NVLink-C2C) and the staged
path (pinned staging buffer, conversion on the host) give bit-identical
arrays, in FP64 and FP32-shifted storage."""
import numpy as np
import pytest

from sclbm import _lib, XIStencils, FStencils
from sclbm.profiles import droplet

pytestmark = pytest.mark.gpu


def pinned(a):
    torch = pytest.importorskip('torch')
    t = torch.empty(a.size, dtype=torch.float64, pin_memory=True)
    out = t.numpy()
    out[:] = a.ravel()
    return out, t


@pytest.mark.parametrize('precision', [_lib.FP64, _lib.FP32_SHIFTED])
def test_direct_and_staged_transfers_agree(precision):
    x, f = XIStencils['D3Q19'], FStencils['D3E6']
    dims = (40, 36, 30)
    n0 = droplet(dims, 8.0, 4.636, 0.147, 2.0, 4)
    res = {}
    s = _lib.Sim(3, dims, x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], -4.5, precision=precision, rho0=0.147)
    pageable = s.set_transfer(_lib.TRANSFER_AUTO)
    for mode, src in (('staged', n0), ('pinned', None), ('pageable', n0)):
        if mode == 'pageable' and not pageable:
            continue
        s.set_transfer(_lib.TRANSFER_STAGED if mode == 'staged' else _lib.TRANSFER_DIRECT)
        if src is None:
            src, keep = pinned(n0)
        s.set_density(src)
        s.set_velocity(np.zeros(3 * s.V))
        s.init_populations()
        s.step(10)
        # read back into pageable arrays: directly where the device reaches them
        s.set_transfer(_lib.TRANSFER_STAGED if mode == 'staged' else _lib.TRANSFER_AUTO)
        res[mode] = (s.get_populations(), s.get_density())
    s.close()
    base = res.pop('staged')
    for mode, (pop, n) in res.items():
        assert np.array_equal(pop, base[0]), mode
        assert np.array_equal(n, base[1]), mode


def test_direct_refuses_unreachable_arrays():
    x, f = XIStencils['D2Q9'], FStencils['D2E4']
    s = _lib.Sim(2, (32, 32), x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], -4.5)
    if s.set_transfer(_lib.TRANSFER_DIRECT):
        pytest.skip('the device reaches pageable host memory')
    with pytest.raises(_lib.SclbmError):
        s.set_density(np.ones(s.V))
    s.close()
