"""Fluctuating Shan-Chen step on the GPU (sclbm_set_fluctuations, the drop-in
MainLoopGross2011SRT) against the reference's own runs
(tests/golden/gross_*.npz):

* generator states bit-identical to the reference after every recorded step
  count (integer recurrences);
* FP64 populations within 1e-12 (relative, max-norm) of the reference: the
  Box-Muller uses CUDA's log and cos, which may differ from glibc's by an ulp;
* the same through the drop-in class with the reference's seeding and CPU
  ordering;
* at sizes beyond the fixtures, equipartition of the ideal gas (G = 0):
  <n u_a^2> = kBT and <dn^2> c_s^2 / n0 = kBT within 5 %, FP64 and FP32, in
  2D and 3D; mass conserved by the noise.
"""
import numpy as np
import pytest

from helpers import rel_err
from sclbm import _lib, XIStencils, FStencils
from sclbm.MultiPhase import ShanChenMultiPhase
from test_gross import CASES, load

pytestmark = pytest.mark.gpu


def ref_tables(nl, Q, D):
    nr = Q - D - 1
    coef = np.zeros((Q, nr))
    for q, tl in enumerate(nl['terms']):
        for k, lit in tl:
            coef[q, int(k)] = float(lit)
    return np.array([-2.0 * float(v) for v in nl['var']]), coef


def start(z, c, nl=None, **kw):
    x, f = XIStencils[c['xi']], FStencils[c['fs']]
    D = len(c['dims'])
    psi = _lib.PSI_EXP_INV if c['psi'] == 'exp' else _lib.PSI_ONE_MINUS_EXP
    s = _lib.Sim(D, c['dims'], x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], c['G'], psi_kind=psi, tau=c['tau'],
                 **kw)
    s.set_density(z['n_init'])
    s.set_velocity(np.zeros(D * s.V))
    s.init_populations()
    mv = cf = None
    if nl is not None:
        mv, cf = ref_tables(nl, len(x['XIs']), D)
    s.set_fluctuations(c['kind'], c['indep'], c['kBT'], c['n0'], z['seeds_init'], _lib.SEEDS_CELL_MAJOR, mv, cf)
    return s


@pytest.mark.parametrize('own', [False, True])
@pytest.mark.parametrize('name', CASES)
def test_fluctuating_step_matches_reference(name, own):
    z, c, nl = load(name)
    s = start(z, c, None if own else nl)
    assert s.kernels_per_step() == 2
    Q = z['pop_init'].shape[0]
    done = 0
    for k in z['steps']:
        s.step(int(k) - done)
        done = int(k)
        assert np.array_equal(s.get_seeds(_lib.SEEDS_CELL_MAJOR), z['seeds_%d' % k]), (name, k)
        got = s.get_populations().reshape(Q, -1)
        want = z['pop_%d' % k].reshape(Q, -1)
        assert rel_err(got, want) < 1e-12, (name, own, k, rel_err(got, want))
    s.close()


@pytest.mark.parametrize('name', ['d2e4_mmix_t1', 'd3e6_minstd_indep_t09'])
def test_dropin_gross_loop_matches_reference(name):
    """ShanChenMultiPhase(fluctuations='Gross2011', ...) seeded like the
    reference, CPU ordering, MainLoopGross2011SRT in the fixture's chunks."""
    sp = pytest.importorskip('sympy')
    z, c, _ = load(name)
    n = sp.Symbol('n')
    sc = ShanChenMultiPhase(lang='cuda', dim_sizes=tuple(c['dims']), xi_stencil=XIStencils[c['xi']],
                            f_stencil=FStencils[c['fs']], psi_code='exp(-1./ln_0)', psi_sym=sp.exp(-1 / n),
                            SC_G=c['G'], tau=c['tau'], fluctuations='Gross2011', prng_kind=c['kind'],
                            init_seed=c['init_seed'], prng_init_from='numpy', prng_distribution='gaussian',
                            indep_gaussian=c['indep'], set_ordering='cpu')
    sc.verbose = False
    assert np.array_equal(sc.crng.sims_idpy_memory['seeds'].D2H(), z['seeds_init'])
    sc.sims_idpy_memory['n'].H2D(z['n_init'].ravel())
    sc.sims_idpy_memory['u'].SetConst(0.0)
    sc.init_status['n'] = sc.init_status['u'] = True
    sc.InitPopulations()
    Q = z['pop_init'].shape[0]
    done = 0
    for k in z['steps']:
        sc.MainLoopGross2011SRT([0, int(k) - done], kBT=c['kBT'], n0=c['n0'], print_flag=False)
        done = int(k)
        pop = sc.GetPopulations()   # cpu ordering: (*flip(dims), Q)
        want = np.moveaxis(z['pop_%d' % k], 0, -1)
        assert rel_err(pop, want) < 1e-12, (name, k)
        assert np.array_equal(sc.crng.sims_idpy_memory['seeds'].D2H(), z['seeds_%d' % k])
    # a deterministic loop afterwards keeps the generator states
    sc.MainLoop([0, 3])
    assert np.array_equal(sc.crng.sims_idpy_memory['seeds'].D2H(), z['seeds_%d' % z['steps'][-1]])
    sc.End()


def equipartition(lat, dims, precision, kind, indep, steps_eq, samples, every, kBT=1e-4, n0=1.0, tau=1.0):
    x = XIStencils[lat]
    f = FStencils['D2E4' if lat == 'D2Q9' else 'D3E4']
    D = len(dims)
    s = _lib.Sim(D, dims, x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], 0.0, psi_kind=_lib.PSI_IDENTITY, tau=tau,
                 precision=precision, rho0=n0)
    s.set_density(np.full(s.V, n0))
    s.set_velocity(np.zeros(D * s.V))
    s.init_populations()
    nr, ns = _lib.noise_counts(D, len(x['Ws']), indep)
    rng = np.random.default_rng(5)
    hi = 2 ** 63 if kind == 'MMIX' else 2 ** 31 - 2
    dt = np.uint64 if kind == 'MMIX' else np.uint32
    seeds = rng.integers(1, hi, ns * s.V, dtype=np.int64).astype(dt)
    s.set_fluctuations(kind, indep, kBT, n0, seeds, _lib.SEEDS_STREAM_MAJOR)
    m0, _ = s.reductions()
    s.step(steps_eq)
    ju, dn = [], []
    for _ in range(samples):
        s.step(every)
        s.compute_moments()
        n = s.get_density()
        u = s.get_velocity().reshape(D, -1)
        ju.append(np.mean(n * u * u) * 1.0)
        dn.append(np.mean((n - n.mean()) ** 2))
    m1, _ = s.reductions()
    s.close()
    return np.mean(ju) / kBT, np.mean(dn) * x['c2'] / (n0 * kBT), abs(m1 - m0) / m0


@pytest.mark.parametrize('lat,dims,precision,kind,indep', [
    ('D2Q9', (128, 128), _lib.FP64, 'MMIX', False),
    ('D2Q9', (128, 128), _lib.FP32_SHIFTED, 'MINSTD', True),
    ('D3Q19', (48, 48, 48), _lib.FP64, 'NUMREC', False),
    ('D3Q19', (48, 48, 48), _lib.FP32_SHIFTED, 'MMIX', False),
])
def test_equipartition_ideal_gas(lat, dims, precision, kind, indep):
    """G = 0: every velocity component carries kBT / n0 and the density
    fluctuations n0 kBT / c_s^2 (fluctuation-dissipation of the noise
    variances norm_k kBT (2 - 1/tau)/tau / c_s^2 n0)."""
    ju, dn, dm = equipartition(lat, dims, precision, kind, indep, 2000, 40, 25)
    assert abs(ju - 1.0) < 0.05, ju
    assert abs(dn - 1.0) < 0.05, dn
    # the 15-digit noise literals sum to zero only to ~1e-16 per column: FP64
    # mass random-walks by ~1e-12 over the 3000 steps
    assert dm < (1e-10 if precision == _lib.FP64 else 1e-4), dm


@pytest.mark.parametrize('lat,kind,indep', [('D2Q9', 'MINSTD', False), ('D3Q19', 'MMIX', False),
                                            ('D3Q19', 'NUMREC', True)])
def test_fp32_single_pass_equals_two_pass(lat, kind, indep):
    """The FP32 fluctuating step in one pass (k_fused_noise) and in two
    (k_fcs_noise): identical generator states, populations within FP32
    rounding of the two collision forms.  Two generators per moment always
    run the two-pass kernels."""
    x = XIStencils[lat]
    f = FStencils['D2E6' if lat == 'D2Q9' else 'D3E6']
    dims = (96, 80) if lat == 'D2Q9' else (40, 36, 32)
    D = len(dims)
    from sclbm.profiles import droplet
    n_init = droplet(dims, 12.0 if D == 2 else 8.0, 4.5625, 0.2086, 2.0, 3)
    nr, ns = _lib.noise_counts(D, len(x['Ws']), indep)
    dt = np.uint64 if kind == 'MMIX' else np.uint32
    seeds = np.random.default_rng(9).integers(1, 2 ** 31 - 2, ns * n_init.size, dtype=np.int64).astype(dt)
    out = []
    for path in (_lib.PATH_FUSED, _lib.PATH_TWO_PASS):
        s = _lib.Sim(D, dims, x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], -4.5, precision=_lib.FP32_SHIFTED,
                     rho0=0.2086)
        s.set_density(n_init)
        s.set_velocity(np.zeros(D * s.V))
        s.init_populations()
        s.set_tuning(path)
        s.set_fluctuations(kind, indep, 1e-5, 1.0, seeds)
        assert s.kernels_per_step() == (1 if path == _lib.PATH_FUSED and not indep else 2)
        s.step(50)
        out.append((s.get_populations(), s.get_seeds()))
        s.close()
    assert np.array_equal(out[0][1], out[1][1])
    assert rel_err(out[0][0], out[1][0]) < 1e-5, rel_err(out[0][0], out[1][0])


def test_fluctuations_refused_with_mrt_and_walls():
    z, c, nl = load('d2e4_mmix_t1')
    s = start(z, c, nl)
    with pytest.raises(_lib.SclbmError):
        s.set_collision(_lib.COLL_MRT, mrt_s=np.diag(np.linspace(1.0, 1.4, 9)))
    with pytest.raises(_lib.SclbmError):
        s.set_walls(np.ones(s.V, np.int32), np.zeros(s.V))
    s.set_fluctuations(None, False, 0, 0, None)
    s.set_collision(_lib.COLL_MRT, mrt_s=np.diag(np.linspace(1.0, 1.4, 9)))
    s.step(2)
    s.close()


def test_zero_generator_state_stays_finite():
    """A NUMREC stream whose next state is 0 makes the reference's Box-Muller
    take log(0): the oracle (which restates the reference) gets infinite
    populations around that cell; the library reads the zero state as state 1
    for the uniform and stays finite, and every cell the planted cell does not
    push into equals the oracle.  The stored states are the reference's."""
    from oracle import oracle as O
    z, c, nl = load('d2e6_numrec_t12_psi1mexp')
    seeds = z['seeds_init'].copy()          # cpu ordering: stream + cell * streams
    ns = seeds.size // int(np.prod(c['dims']))
    cell = 5 + 24 * 7
    # the state whose successor is 0: x * 1664525 + 1013904223 = 0 mod 2^32
    inv = pow(1664525, -1, 2 ** 32)
    seeds[0 + cell * ns] = np.uint32(((-1013904223) * inv) % 2 ** 32)
    x, f = XIStencils[c['xi']], FStencils[c['fs']]
    ora = O.OracleSim(c['dims'], x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], c['G'], tau=c['tau'], psi=c['psi'])
    ora.set_fields(z['n_init'])
    ora.init_populations()
    ora.set_fluctuations(c['kind'], c['indep'], c['kBT'], c['n0'], seeds, c['tau'], nl)
    with np.errstate(all='ignore'):
        ora.run(1)
    want = ora.populations().reshape(9, -1)
    s = _lib.Sim(2, c['dims'], x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], c['G'],
                 psi_kind=_lib.PSI_ONE_MINUS_EXP, tau=c['tau'])
    s.set_density(z['n_init'])
    s.set_velocity(np.zeros(2 * s.V))
    s.init_populations()
    mv, cf = ref_tables(nl, 9, 2)
    s.set_fluctuations(c['kind'], c['indep'], c['kBT'], c['n0'], seeds, _lib.SEEDS_CELL_MAJOR, mv, cf)
    s.step(1)
    got = s.get_populations().reshape(9, -1)
    assert np.isfinite(got).all()
    bad = ~np.isfinite(want)
    assert bad.any()                         # the reference's arithmetic blows up there
    assert rel_err(got[~bad], want[~bad]) < 1e-12
    assert np.array_equal(s.get_seeds(_lib.SEEDS_CELL_MAJOR), ora.get_seeds())
    s.close()


@pytest.mark.parametrize('st,kind,dims', [('D3E6', 'MINSTD', (40, 36, 32)), ('D3E6', 'MMIX', (66, 18, 20)),
                                          ('D3E8', 'NUMREC', (32, 32, 24))])
def test_fp32_single_pass_paired_halo_loads_bit_identical(st, kind, dims):
    """The fluctuating single pass with paired halo loads gives the same
    populations and generator states, bit for bit, as with one halo cell per
    load (the sums run in the same order)."""
    x, f = XIStencils['D3Q19'], FStencils[st]
    from sclbm.profiles import droplet
    n_init = droplet(dims, 8.0, 4.5625, 0.2086, 2.0, 5)
    nr, ns = _lib.noise_counts(3, 19, False)
    dt = np.uint64 if kind == 'MMIX' else np.uint32
    seeds = np.random.default_rng(11).integers(1, 2 ** 31 - 2, ns * n_init.size, dtype=np.int64).astype(dt)
    out = []
    for path in (_lib.PATH_FUSED, _lib.PATH_FUSED_PAIRS):
        s = _lib.Sim(3, dims, x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], -4.5, precision=_lib.FP32_SHIFTED,
                     rho0=0.2086)
        s.set_density(n_init)
        s.set_velocity(np.zeros(3 * s.V))
        s.init_populations()
        s.set_tuning(path, 5)
        s.set_fluctuations(kind, False, 1e-5, 1.0, seeds)
        assert s.get_tuning()[0] == path and s.kernels_per_step() == 1
        s.step(20)
        out.append((s.get_populations(), s.get_seeds()))
        s.close()
    assert np.array_equal(out[0][1], out[1][1])
    assert np.array_equal(out[0][0], out[1][0])
