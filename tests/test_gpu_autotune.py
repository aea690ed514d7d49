"""The autotuner (sclbm_autotune): it picks one of the handle's bit-identical
step variants by timing them, leaves the state alone, and later handles of the
same configuration on the automatic choice take its pick from the cache.
No counterpart in the reference (fixed 128-thread blocks,
idpy/LBM/MultiPhase.py:2072-2085)."""
import numpy as np
import pytest

from sclbm import _lib, XIStencils, FStencils
from sclbm.profiles import droplet

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _fresh_cache():
    _lib.clear_tuning_cache()
    yield
    _lib.clear_tuning_cache()   # other tests expect the planner's defaults


def _sim(dims, st='D3E6', precision=_lib.FP32_SHIFTED, **kw):
    D = len(dims)
    x, f = XIStencils['D3Q19' if D == 3 else 'D2Q9'], FStencils[st]
    s = _lib.Sim(D, dims, x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], -4.5, precision=precision,
                 rho0=0.2 if precision == _lib.FP32_SHIFTED else 0.0, **kw)
    s.set_density(droplet(dims, min(dims) / 4, 4.6, 0.2, 2.0, 31))
    s.set_velocity(np.zeros(D * s.V))
    s.init_populations()
    return s


@pytest.mark.parametrize('dims,st', [((96, 64, 48), 'D3E6'), ((64, 40, 36), 'D3E8'), ((200, 120), 'D2E4')])
def test_autotune_picks_a_bit_identical_variant(dims, st):
    a = _sim(dims, st)
    before = a.get_populations()
    cfg, ms = a.autotune(trial_steps=3)
    assert ms > 0 and cfg['grid'] > 0
    assert cfg['path'] in (_lib.PATH_FUSED, _lib.PATH_FUSED_PAIRS) and a.kernels_per_step() == 1
    assert cfg['staging'] in (0, 1, 2, 3) and cfg['tile'] in (0, 1, 2, 3, 4, 5) and cfg['order'] in (0, 1, 2)
    assert cfg['staging'] == 0 or cfg['tile'] == 0
    if len(dims) == 2:
        assert cfg['path'] == _lib.PATH_FUSED and cfg['staging'] == 0 and cfg['tile'] == 0 and cfg['order'] in (0, 1)
    assert np.array_equal(a.get_populations(), before)      # trials leave the state as it was
    _lib.clear_tuning_cache()
    b = _sim(dims, st)                                      # the planner's default variant
    assert b.get_tuning_ex()['staging'] == 0
    for s in (a, b):
        s.step(12)
    assert np.array_equal(a.get_populations(), b.get_populations())
    a.close()
    b.close()


def test_tuned_configuration_is_cached_for_automatic_handles():
    dims = (96, 64, 48)
    a = _sim(dims)
    a.autotune(trial_steps=2)
    want = a.get_tuning_ex()
    b = _sim(dims)
    assert b.get_tuning_ex() == want                         # AUTO, chunk 0, staging -1: the cached pick
    c = _sim(dims)
    c.set_tuning_ex(_lib.PATH_AUTO, 7, 0)                   # an explicit choice is kept
    assert c.get_tuning_ex()['chunk'] == 7 and c.get_tuning_ex()['staging'] == 0
    d = _sim((96, 64, 50))                                  # another box: its own planner
    assert d.get_tuning_ex()['chunk'] != 0
    for s in (a, b, c, d):
        s.close()


def test_autotune_two_pass_handle_keeps_its_kernels():
    s = _sim((40, 32, 24), precision=_lib.FP64)
    before = s.get_populations()
    cfg, ms = s.autotune(trial_steps=2)
    assert cfg['path'] == _lib.PATH_TWO_PASS and ms > 0
    assert np.array_equal(s.get_populations(), before)
    s.close()


def test_autotune_refuses_fluctuating_handles():
    s = _sim((32, 24, 16), precision=_lib.FP64)
    nr, ns = _lib.noise_counts(3, 19, False)
    seeds = np.random.default_rng(5).integers(1, 2 ** 31 - 1, ns * s.V, dtype=np.uint32)
    s.set_fluctuations('MINSTD', False, 1e-5, 1.0, seeds)
    with pytest.raises(_lib.SclbmError) as e:
        s.autotune(2)
    assert e.value.status == _lib.ERR_UNSUPPORTED
    s.close()
