"""Shared test helpers: fixture loading, oracle construction, literal tables."""
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


def load(name):
    p = os.path.join(GOLDEN, name + '.npz')
    if not os.path.exists(p):
        pytest.skip('fixture %s not generated' % name)
    z = np.load(p)
    return z, json.loads(str(z['config_json']))


def mono_index(name, D):
    """Monomial name of the reference's generated code -> index in the library layout."""
    NU, NUU = 1, 1 + D
    F = 1 + D + D * (D + 1) // 2
    FU = F + D
    toks = name.split('*')
    if toks == ['ln_0']:
        return 0
    if toks[0] == 'ln_0':
        us = sorted(int(t[5:]) for t in toks[1:])
        if len(us) == 1:
            return NU + us[0]
        a, b = us
        return NUU + a * D - a * (a - 1) // 2 + (b - a)
    if toks[0].startswith('d_psi_'):
        a = int(toks[0][6:])
        if len(toks) == 1:
            return F + a
        return FU + a * D + int(toks[1][5:])
    raise ValueError(name)


def literal_tables(lit, Q, D):
    """(A, B) operator tables from the reference's printed literals."""
    K = 1 + D + D * (D + 1) // 2 + D + D * D
    A = np.zeros((Q, Q))
    B = np.zeros((Q, K))
    for q in range(Q):
        for name, v in lit[str(q)].items():
            if name.startswith('lpop_'):
                A[q, int(name[5:])] = float(v)
            else:
                B[q, mono_index(name, D)] = float(v)
    return A, B


def rel_err(a, b):
    """max |a - b| / max |b|"""
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))
