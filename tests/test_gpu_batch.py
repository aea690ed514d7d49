"""Batched ragged lattices: each lattice of a batch steps exactly like the
same lattice on its own handle; retired lattices stop; per-lattice checks."""
import numpy as np
import pytest

from helpers import rel_err
from sclbm import _lib, XIStencils, FStencils
from sclbm.batch import Batch
from sclbm.profiles import droplet

pytestmark = pytest.mark.gpu

CASES = {
    '2d': ('D2Q9', 'D2E8', [(64, 64), (96, 96), (32, 32)], [-4.5, -5.0, -4.8], [0.8, 2.0, 1.0]),
    '3d': ('D3Q19', 'D3E6', [(32, 32, 32), (48, 40, 36)], [-4.5, -4.7], [1.0, 2.4]),
    # an odd Lx: the whole batch keeps one halo cell per load
    '3d_odd': ('D3Q19', 'D3E6', [(33, 20, 16), (32, 32, 24)], [-4.5, -4.7], [1.0, 2.4]),
}


def make_single(lat, st, dims, G, rho0):
    x, f = XIStencils[lat], FStencils[st]
    return _lib.Sim(len(dims), dims, x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], G,
                    precision=_lib.FP32_SHIFTED, rho0=rho0)


def densities(dims_list):
    return [droplet(d, min(d) / 4.0, 4.6, 0.2, 2.0, 30 + i) for i, d in enumerate(dims_list)]


@pytest.mark.parametrize('case', ['2d', '3d', '3d_odd'])
def test_batch_matches_single_lattices(case):
    lat, st, dims, G, rho0 = CASES[case]
    n0 = densities(dims)
    b = Batch(XIStencils[lat], FStencils[st], dims, G, rho0)
    for i, n in enumerate(n0):
        b.set_density(i, n)
    b.init_populations()
    singles = []
    for i, d in enumerate(dims):
        s = make_single(lat, st, d, G[i], rho0[i])
        s.set_density(n0[i])
        s.set_velocity(np.zeros(len(d) * s.V))
        s.init_populations()
        singles.append(s)
    b.step(40)       # graph replay (32) + 8 direct launches
    for i, s in enumerate(singles):
        s.step(40)
        assert rel_err(b.get_density(i).ravel(), s.get_density()) < 1e-6, i
    # per-lattice observables against the single handles' reductions
    uc, mu, m = b.check()
    for i, s in enumerate(singles):
        s.compute_moments()
        uc1, mu1 = s.check_u()
        m1, _ = s.reductions()
        assert abs(m[i] - m1) / m1 < 1e-6
        assert abs(mu[i] - mu1) / mu1 < 1e-3
        assert abs(uc[i] - uc1) / uc1 < 1e-3
        s.close()
    b.close()


def test_batch_retires_lattices_individually():
    lat, st, dims, G, rho0 = CASES['2d']
    n0 = densities(dims)
    b = Batch(XIStencils[lat], FStencils[st], dims, G, rho0)
    for i, n in enumerate(n0):
        b.set_density(i, n)
    b.init_populations()
    b.step(21)
    frozen = b.get_density(1).copy()
    b.set_active([1, 0, 1])
    b.step(33)
    assert np.array_equal(b.get_density(1), frozen)
    assert list(b.steps()) == [54, 21, 54]
    s = make_single(lat, st, dims[2], G[2], rho0[2])
    s.set_density(n0[2])
    s.set_velocity(np.zeros(2 * s.V))
    s.init_populations()
    s.step(54)
    assert rel_err(b.get_density(2).ravel(), s.get_density()) < 1e-6
    # resuming continues from the frozen state
    b.set_active([1, 1, 1])
    b.step(1)
    assert not np.array_equal(b.get_density(1), frozen)
    s.close()
    b.close()


@pytest.mark.parametrize('st', ['D2E4', 'D2E8'])
def test_narrow_2d_tiles_bit_identical(st):
    """64-cell tiles (four times the work items) step every lattice bit for
    bit as the default 256-cell tiles, also across retirement and re-planning;
    lattices narrower than, equal to and wider than either tile."""
    dims = [(32, 32), (50, 40), (64, 70), (100, 100), (224, 96), (300, 36)]
    G, rho0 = [-4.5, -4.8, -4.6, -4.6, -4.7, -4.5], [0.2, 1.0, 2.0, 0.5, 0.22, 0.3]
    n0 = densities(dims)
    out = []
    for tx in (0, 64):
        b = Batch(XIStencils['D2Q9'], FStencils[st], dims, G, rho0)
        b.set_tile_width(tx)
        for i, n in enumerate(n0):
            b.set_density(i, n)
        b.init_populations()
        b.step(45)
        b.set_active([1, 0, 1, 1, 0, 1])
        b.step(38)
        out.append([b.get_density(i) for i in range(len(dims))])
        b.close()
    for i in range(len(dims)):
        assert np.isfinite(out[0][i]).all(), i
        assert np.array_equal(out[0][i], out[1][i]), i


def test_mass_compensation_off():
    """Plain FP32 sums for the rest population (3D paired batches): the same
    step up to FP32 rounding; refused where it is not built."""
    lat, st, dims, G, rho0 = CASES['3d']
    n0 = densities(dims)
    out, mass = [], []
    for on in (True, False):
        b = Batch(XIStencils[lat], FStencils[st], dims, G, rho0)
        b.set_mass_compensation(on)
        for i, n in enumerate(n0):
            b.set_density(i, n)
        b.init_populations()
        m0 = b.restore_mass()
        b.step(60)
        mass.append(b.restore_mass() / m0 - 1)
        out.append([b.get_density(i) for i in range(len(dims))])
        b.close()
    for i in range(len(dims)):
        assert rel_err(out[1][i], out[0][i]) < 1e-5, i
    # compensated: one FP32 rounding of the rest population per cell and step
    # (~1e-9 after 60 steps); plain sums drift two orders of magnitude more
    assert np.abs(mass[0]).max() < 1e-8 and np.abs(mass[1]).max() < 1e-5, mass
    assert np.abs(mass[1]).max() > 10 * np.abs(mass[0]).max(), mass
    lat, st, dims, G, rho0 = CASES['2d']
    b = Batch(XIStencils[lat], FStencils[st], dims, G, rho0)
    with pytest.raises(_lib.SclbmError):
        b.set_mass_compensation(False)
    b.close()


def test_narrow_tiles_refused_in_3d():
    lat, st, dims, G, rho0 = CASES['3d']
    b = Batch(XIStencils[lat], FStencils[st], dims, G, rho0)
    with pytest.raises(_lib.SclbmError):
        b.set_tile_width(64)
    b.set_tile_width(0)
    b.close()


def test_batch_rejects_bad_input():
    lat, st = 'D2Q9', 'D2E8'
    with pytest.raises(_lib.SclbmError):
        Batch(XIStencils[lat], FStencils[st], [(64, 1)], [-4.5], [1.0])
    with pytest.raises(_lib.SclbmError):
        Batch(XIStencils[lat], FStencils['D3E6'], [(64, 64)], [-4.5], [1.0])


def test_batch_probe_reads_centre_and_last_cell():
    lat, st, dims, G, rho0 = CASES['2d']
    n0 = densities(dims)
    b = Batch(XIStencils[lat], FStencils[st], dims, G, rho0)
    for i, n in enumerate(n0):
        b.set_density(i, n)
    b.init_populations()
    b.step(17)
    ni, no = b.probe()
    for i, d in enumerate(dims):
        nf = b.get_density(i)
        assert abs(ni[i] - nf[d[1] // 2, d[0] // 2]) < 1e-12 * abs(ni[i])
        assert abs(no[i] - nf[-1, -1]) < 1e-12 * abs(no[i])
    # retired lattices keep the caller's values
    b.set_active([1, 0, 1])
    a, c = np.full(3, -1.0), np.full(3, -1.0)
    _lib.call('sclbm_batch_probe', b.h, _lib.ptr(a), _lib.ptr(c))
    assert a[1] == -1.0 and c[1] == -1.0 and a[0] != -1.0
    b.close()


def test_batch_probe_block_means():
    """With a probe radius the probes are FP64 means over the (2 rad + 1)^D
    block about the centre cell and about the last cell (periodic)."""
    lat, st, dims, G, rho0 = CASES['2d']
    n0 = densities(dims)
    b = Batch(XIStencils[lat], FStencils[st], dims, G, rho0)
    for i, n in enumerate(n0):
        b.set_density(i, n)
    b.init_populations()
    b.step(11)
    b.set_probe_radius(2)
    ni, no = b.probe()
    for i, d in enumerate(dims):
        nf = b.get_density(i)
        cy, cx = d[1] // 2, d[0] // 2
        blk = nf[cy - 2:cy + 3, cx - 2:cx + 3]
        corner = np.roll(np.roll(nf, -2, axis=0), -2, axis=1)[-5:, -5:]   # rows/cols L-3 .. L+1 (periodic)
        assert abs(ni[i] - blk.mean()) < 1e-12 * abs(ni[i])
        assert abs(no[i] - corner.mean()) < 1e-12 * abs(no[i])
    b.close()


def test_batch_restore_mass_sets_each_lattice_mass():
    lat, st, dims, G, rho0 = CASES['2d']
    n0 = densities(dims)
    b = Batch(XIStencils[lat], FStencils[st], dims, G, [0.2, 0.2, 0.2])
    for i, n in enumerate(n0):
        b.set_density(i, n)
    b.init_populations()
    m0 = b.restore_mass()
    for i, n in enumerate(n0):
        assert abs(m0[i] / n.sum() - 1) < 1e-6   # FP32 storage of the initial field
    b.step(300)
    m1 = b.restore_mass()
    target = m1 * (1 + np.array([1e-5, 0.0, -2e-5]))
    target[1] = np.nan                           # lattice 1: no correction
    b.restore_mass(target)
    m2 = b.restore_mass()
    assert abs(m2[0] / target[0] - 1) < 1e-7 and abs(m2[2] / target[2] - 1) < 1e-7
    assert m2[1] == m1[1]
    b.close()


def test_restore_mass_single_handle():
    x, f = XIStencils['D2Q9'], FStencils['D2E8']
    dims = (96, 80)
    s = _lib.Sim(2, dims, x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], -4.6, precision=_lib.FP32_SHIFTED,
                 rho0=0.2)
    s.set_density(droplet(dims, 20, 4.7, 0.2, 2.0, 5))
    s.set_velocity(np.zeros(2 * s.V))
    s.init_populations()
    m0 = s.restore_mass()
    s.step(500)
    s.restore_mass(m0 * (1 + 3e-5))
    m1 = s.restore_mass()
    assert abs(m1 / (m0 * (1 + 3e-5)) - 1) < 1e-7
    m2, _ = s.reductions()
    assert m2 == m1
    s.close()


def test_3d_droplets_batch_matches_plain_fp64():
    from sclbm import sweep
    radii, G = [6.0, 8.0], [-4.6, -4.7]
    guess = [sweep.thermo_guess(g, 'D2E6') for g in G]
    rl, rg = [a for a, _ in guess], [b for _, b in guess]
    # both paths run the same 6000 steps (no early stop), then the Laplace
    # pressures of the FP32 batch and the FP64 plain path are compared
    b = sweep.ragged_sweep(radii, G, rl, rg, stencil='D3E6', dim=3, boxes=[32, 32], max_steps=6000, tol_dp=0.0)
    assert (b['status'] == 'max_steps').all() and (b['steps'] == 6000).all(), (b['status'], b['steps'])
    for i in range(2):
        p = sweep.plain_run(radii[i], G[i], rl[i], rg[i], stencil='D3E6', dim=3, L=32, max_steps=6000, tol=0.0)
        assert p['steps'] == 6000 and p['status'] == 'max_steps'
        assert abs(b["dp"][i] / p["dp"] - 1) < 2e-4, (b["dp"][i], p["dp"])
