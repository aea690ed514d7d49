"""CPU-side checks of the boundary: the C-ABI library loads and exports every
symbol include/sclbm.h declares; host-side argument handling of the shim.
No kernels run here."""
import ctypes
import os
import re

import numpy as np
import pytest

from sclbm import _lib, ShanChenMultiPhase, XIStencils, FStencils, CUDA_T
from sclbm.MultiPhase import psi_kind_of, numeric_relaxation_matrix

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = []
    for h in os.listdir(os.path.join(ROOT, 'include')):
        if h.endswith('.h'):
            src = open(os.path.join(ROOT, 'include', h)).read()
            syms += re.findall(r'SCLBM_API\s+[\w\s\*]*?\b(sclbm_\w+)\s*\(', src)
    return sorted(set(syms))


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    syms = declared_symbols()
    assert len(syms) >= 30
    for s in syms:
        assert hasattr(lib, s), s
        assert s in _lib.SIGNATURES, s


def test_library_metadata_calls():
    lib = _lib.load()
    assert b'sm_103a' in lib.sclbm_version()
    assert lib.sclbm_status_string(_lib.ERR_STATE) == b'call out of order'
    assert _lib.monomial_count(2) == 12 and _lib.monomial_count(3) == 22
    assert _lib.monomial_count(4) == 0


def test_create_without_gpu_fails_loudly():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip('a GPU is present')
    except ImportError:
        pass
    x, f = XIStencils['D2Q9'], FStencils['D2E4']
    with pytest.raises(_lib.SclbmError) as e:
        _lib.Sim(2, (16, 16), x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], -4.5)
    assert e.value.status in (_lib.ERR_NODEVICE, _lib.ERR_CUDA)


def test_create_rejects_bad_tables_before_touching_the_device():
    x, f = XIStencils['D2Q9'], FStencils['D2E4']
    with pytest.raises(_lib.SclbmError) as e:
        _lib.Sim(2, (16, 16), [(1, 0)] * 9, x['Ws'], x['c2'], f['Es'], f['Ws'], -4.5)
    assert e.value.status == _lib.ERR_UNSUPPORTED
    with pytest.raises(_lib.SclbmError) as e:
        _lib.Sim(2, (16, 16), x['XIs'], x['Ws'], x['c2'], f['Es'][:7], f['Ws'][:7], -4.5)
    assert e.value.status == _lib.ERR_UNSUPPORTED
    with pytest.raises(_lib.SclbmError) as e:
        _lib.Sim(2, (1, 16), x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], -4.5)
    assert e.value.status == _lib.ERR_ARG


def test_batch_rejects_unequal_weights_on_opposite_vectors():
    """The single-pass kernels pair every force-stencil vector with its
    opposite (one psi difference per pair), so a stencil whose opposite
    vectors carry different weights is refused before the device is touched."""
    from sclbm.batch import Batch
    x, f = XIStencils['D2Q9'], FStencils['D2E4']
    ws = list(f['Ws'])
    ws[0] = ws[0] * 1.5
    bad = dict(f, Ws=ws)
    with pytest.raises(_lib.SclbmError) as e:
        Batch(x, bad, [(32, 32)], [-4.5], [1.0])
    assert e.value.status == _lib.ERR_UNSUPPORTED
    assert 'opposite' in str(e.value)
    try:
        import torch
        if torch.cuda.is_available():
            return
    except ImportError:
        pass
    with pytest.raises(_lib.SclbmError) as e:
        Batch(x, f, [(32, 32)], [-4.5], [1.0])   # symmetric: passes the check, no device
    assert e.value.status in (_lib.ERR_NODEVICE, _lib.ERR_CUDA)


@pytest.mark.parametrize('missing,msg', [
    ('f_stencil', "Missing 'f_stencil'"), ('tau', "Missing 'tau'"), ('SC_G', "Missing 'SC_G'"),
    ('psi_code', "Missing 'psi_code'"), ('lang', 'Param lang'), ('psi_sym', "parameter 'psi_sym'")])
def test_shim_missing_parameters_raise_like_the_reference(missing, msg):
    kw = dict(lang=CUDA_T, dim_sizes=(16, 16), xi_stencil=XIStencils['D2Q9'], f_stencil=FStencils['D2E4'],
              psi_code='exp(-1./ln_0)', psi_sym=None, SC_G=-4.5, tau=1.0)
    del kw[missing]
    with pytest.raises(Exception) as e:
        ShanChenMultiPhase(**kw)
    assert msg in str(e.value)


def test_psi_code_forms():
    assert psi_kind_of('exp(-1./ln_0)') == _lib.PSI_EXP_INV
    assert psi_kind_of('(PsiType) exp(-1/ln_0)') == _lib.PSI_EXP_INV
    assert psi_kind_of('(1. - exp(-ln_0))') == _lib.PSI_ONE_MINUS_EXP
    assert psi_kind_of('ln_0') == _lib.PSI_IDENTITY
    with pytest.raises(Exception):
        psi_kind_of('pow(ln_0, 2)')


def test_relaxation_matrix_substitution():
    sp = pytest.importorskip('sympy')
    syms = [sp.Symbol('w%d' % i) for i in range(9)]
    S = numeric_relaxation_matrix(sp.Matrix.diag(syms), [(s, 1.0 + 0.1 * i) for i, s in enumerate(syms)], 9)
    assert np.allclose(np.diag(S), 1.0 + 0.1 * np.arange(9)) and S.shape == (9, 9)
