"""Host-side checks (no GPU) of two pairings in the single-pass kernel: the
paired halo loads' index arithmetic, and the opposite-direction split of the
BGK operator.

The single-pass kernel (idea.deploy_gb300/csrc/fused.cuh, PAIRS) loads the
populations of two x-adjacent halo cells with one 8-byte load.  Pair c of a
tile at (x0, y0) starts at x = wrap(x0 - R + 2 (c mod HP)) with HP = (TX + 2R)/2
pairs per row.  For the load to be aligned and to read the right cells, the
first cell must be even and the second must be the first's periodic
neighbour in x.  This restates that arithmetic for every tile of many even
lattice widths and checks both, and that the pairs of a row cover exactly the
halo cells x0 - R .. x0 + TX + R - 1.
"""
import pytest

TX, TY = 32, 8


def wrapm(x, L):
    return x % L


@pytest.mark.parametrize('R', [2])
def test_pairs_are_aligned_and_adjacent_for_even_widths(R):
    HX = TX + 2 * R
    HP = HX // 2
    for Lx in range(2, 200, 2):
        for x0 in range(0, Lx, TX):
            covered = []
            for hp in range(HP):
                x = x0 - R + 2 * hp
                g0 = wrapm(x, Lx)
                g1 = wrapm(x + 1, Lx)
                assert g0 % 2 == 0, (Lx, x0, hp)
                assert g0 + 1 < Lx and g1 == g0 + 1, (Lx, x0, hp)
                covered += [g0, g1]
            want = [wrapm(x0 - R + i, Lx) for i in range(HX)]
            assert covered == want


def test_pair_count_fits_the_block():
    for R in (2,):
        HP = (TX + 2 * R) // 2
        assert HP * (TY + 2 * R) <= TX * TY


def test_odd_width_would_straddle_the_wrap():
    """Why odd Lx keeps one cell per load: some pair would start at Lx - 1."""
    R, Lx = 2, 35
    starts = [wrapm(x0 - R + 2 * hp, Lx) for x0 in range(0, Lx, TX) for hp in range((TX + 2 * R) // 2)]
    assert any(s == Lx - 1 or s % 2 for s in starts)


def test_bgk_opposite_pair_split_equals_per_direction_form():
    """A check of the algebra only (FP64 numpy, the kernel is not run): the
    single pass makes a direction q and its opposite together from the
    even part t = a eu^2 + c eu eF and the odd part s = b eu + d eF of the
    factored BGK + Guo operator; in exact arithmetic (FP64 here) that equals
    the per-direction form w_q [C0 + eu (a eu + b + c eF) + d eF]."""
    import numpy as np
    from sclbm import XIStencils
    rng = np.random.default_rng(3)
    x = XIStencils['D3Q19']
    xi = np.array(x['XIs'], float)
    w = np.array(x['Ws'], float)
    opp = [int(np.where((xi == -xi[q]).all(axis=1))[0][0]) for q in range(19)]
    for _ in range(20):
        u, F = rng.normal(0, 0.05, 3), rng.normal(0, 0.01, 3)
        n, om = rng.uniform(0.2, 4.0), rng.uniform(0.5, 1.8)
        dn = n - 1.0
        C0 = om * dn - 1.5 * om * n * (u @ u) - 3 * (1 - om / 2) * (u @ F)
        a, b, c, d = 4.5 * om * n, 3 * om * n, 9 * (1 - om / 2), 3 * (1 - om / 2)
        for q in range(1, 19):
            eu, eF = xi[q] @ u, xi[q] @ F
            per_q = w[q] * (C0 + eu * (a * eu + b + c * eF) + d * eF)
            t, s = eu * (a * eu + c * eF), b * eu + d * eF
            assert abs(per_q - w[q] * (C0 + t + s)) < 1e-15
            qb = opp[q]
            eub, eFb = xi[qb] @ u, xi[qb] @ F
            per_qb = w[qb] * (C0 + eub * (a * eub + b + c * eFb) + d * eFb)
            assert abs(per_qb - w[qb] * (C0 + t - s)) < 1e-15
