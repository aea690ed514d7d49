"""Host-side check of the paired halo loads' index arithmetic (no GPU).

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
