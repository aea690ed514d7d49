"""Lattice and force-stencil tables, keyed like the reference's ``XIStencils`` and
``FStencils`` (idpy/LBM/LBM.py:74-185) so reference scripts can pass them unchanged.

The vectors, weights and their ORDER are the reference's: the order fixes the
summation order of the Shan-Chen gradient and of the moments, which is what
makes bit-level parity with the reference possible.  Weights are Python floats
(``4/9`` etc.) exactly as the reference holds them.

``XIs``: lattice velocities (x first), ``Ws``: lattice weights, ``c2``: squared
sound speed; ``Es``/``Ws``: isotropic force-stencil vectors and weights with
e2 = 1 (E4, E6, E8 in 2D and 3D).
"""

XIStencils = {}
FStencils = {}


def _shells(*groups):
    es, ws = [], []
    for w, vecs in groups:
        for v in vecs:
            es.append(tuple(v))
            ws.append(w)
    return {'Es': tuple(es), 'Ws': tuple(ws)}


XIStencils['D2Q9'] = {
    'XIs': ((0, 0), (1, 0), (0, 1), (-1, 0), (0, -1), (1, 1), (-1, 1), (-1, -1), (1, -1)),
    'Ws': (4/9,) + (1/9,) * 4 + (1/36,) * 4,
    'c2': 1/3,
}

XIStencils['D3Q19'] = {
    'XIs': ((0, 0, 0),
            (1, 0, 0), (0, 1, 0), (-1, 0, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1),
            (1, 1, 0), (-1, 1, 0), (-1, -1, 0), (1, -1, 0),
            (1, 0, 1), (-1, 0, 1), (-1, 0, -1), (1, 0, -1),
            (0, 1, 1), (0, -1, 1), (0, -1, -1), (0, 1, -1)),
    'Ws': (1/3,) + (1/18,) * 6 + (1/36,) * 12,
    'c2': 1/3,
}

FStencils['D2E4'] = _shells(
    (1/3, [(1,0), (0,1), (-1,0), (0,-1)]),
    (1/12, [(1,1), (-1,1), (-1,-1), (1,-1)]),
)

FStencils['D2E6'] = _shells(
    (4/15, [(1,0), (0,1), (-1,0), (0,-1)]),
    (1/10, [(1,1), (-1,1), (-1,-1), (1,-1)]),
    (1/120, [(2,0), (0,2), (-2,0), (0,-2)]),
)

FStencils['D2E8'] = _shells(
    (4/21, [(1,0), (0,1), (-1,0), (0,-1)]),
    (4/45, [(1,1), (-1,1), (-1,-1), (1,-1)]),
    (1/60, [(2,0), (0,2), (-2,0), (0,-2)]),
    (2/315, [(2,1), (1,2), (-1,2), (-2,1), (-2,-1), (-1,-2), (1,-2), (2,-1)]),
    (1/5040, [(2,2), (-2,2), (-2,-2), (2,-2)]),
)

FStencils['D3E4'] = _shells(
    (1/6, [(1,0,0), (0,1,0), (-1,0,0), (0,-1,0), (0,0,1), (0,0,-1)]),
    (1/12, [(1,1,0), (-1,1,0), (-1,-1,0), (1,-1,0), (0,1,1), (0,-1,1), (0,-1,-1), (0,1,-1), (1,0,1), (1,0,-1), (-1,0,-1), (-1,0,1)]),
)

FStencils['D3E6'] = _shells(
    (2/15, [(1,0,0), (0,1,0), (-1,0,0), (0,-1,0), (0,0,1), (0,0,-1)]),
    (1/15, [(1,1,0), (-1,1,0), (-1,-1,0), (1,-1,0), (0,1,1), (0,-1,1), (0,-1,-1), (0,1,-1), (1,0,1), (1,0,-1), (-1,0,-1), (-1,0,1)]),
    (1/60, [(1,1,1), (-1,1,1), (-1,-1,1), (1,-1,1), (1,1,-1), (-1,1,-1), (-1,-1,-1), (1,-1,-1)]),
    (1/120, [(2,0,0), (0,2,0), (-2,0,0), (0,-2,0), (0,0,2), (0,0,-2)]),
)

FStencils['D3E8'] = _shells(
    (4/45, [(1,0,0), (0,1,0), (-1,0,0), (0,-1,0), (0,0,1), (0,0,-1)]),
    (1/21, [(1,1,0), (-1,1,0), (-1,-1,0), (1,-1,0), (0,1,1), (0,-1,1), (0,-1,-1), (0,1,-1), (1,0,1), (1,0,-1), (-1,0,-1), (-1,0,1)]),
    (2/105, [(1,1,1), (-1,1,1), (-1,-1,1), (1,-1,1), (1,1,-1), (-1,1,-1), (-1,-1,-1), (1,-1,-1)]),
    (5/504, [(2,0,0), (0,2,0), (-2,0,0), (0,-2,0), (0,0,2), (0,0,-2)]),
    (1/315, [(2,1,0), (2,-1,0), (2,0,1), (2,0,-1), (1,2,0), (-1,2,0), (0,2,1), (0,2,-1), (-2,1,0), (-2,-1,0), (-2,0,1), (-2,0,-1), (1,-2,0), (-1,-2,0), (0,-2,1), (0,-2,-1), (1,0,2), (-1,0,2), (0,1,2), (0,-1,2), (1,0,-2), (-1,0,-2), (0,1,-2), (0,-1,-2)]),
    (1/630, [(2,1,1), (2,-1,1), (2,-1,-1), (2,1,-1), (1,2,1), (-1,2,1), (-1,2,-1), (1,2,-1), (-2,1,1), (-2,-1,1), (-2,-1,-1), (-2,1,-1), (1,-2,1), (-1,-2,1), (-1,-2,-1), (1,-2,-1), (1,1,2), (-1,1,2), (-1,-1,2), (1,-1,2), (1,1,-2), (-1,1,-2), (-1,-1,-2), (1,-1,-2)]),
    (1/5040, [(2,2,0), (-2,2,0), (-2,-2,0), (2,-2,0), (2,0,2), (-2,0,2), (-2,0,-2), (2,0,-2), (0,2,2), (0,-2,2), (0,-2,-2), (0,2,-2)]),
)


# (dimension, Q) -> lattice name; (dimension, vectors) -> stencil order E4/E6/E8
LATTICE_OF = {(2, 9): 'D2Q9', (3, 19): 'D3Q19'}
STENCIL_ORDER = {'D2E4': 4, 'D2E6': 6, 'D2E8': 8, 'D3E4': 4, 'D3E6': 6, 'D3E8': 8}


def identify_lattice(xi_stencil):
    """Name of a lattice table, matched on vectors, weights and c2."""
    for name, t in XIStencils.items():
        if tuple(map(tuple, xi_stencil['XIs'])) == t['XIs'] and \
                tuple(xi_stencil['Ws']) == t['Ws'] and float(xi_stencil['c2']) == t['c2']:
            return name
    return None


def identify_stencil(f_stencil):
    """Name of a force stencil, matched on its vectors in order."""
    es = f_stencil.get('Es', f_stencil.get('XIs'))
    for name, t in FStencils.items():
        if tuple(map(tuple, es)) == t['Es']:
            return name
    return None
