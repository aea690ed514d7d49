"""Droplet sweeps: coexistence densities, batched FP32 droplets, FP64 plain runs.

* ``coexistence_many(Gs, ...)``: the plain method (FP64 GPU path) on flat
  interfaces (periodic slabs, the reference's ``InitFlatInterface``,
  idpy/LBM/MultiPhase.py:1855-1895), one handle and stream per coupling, all
  stepped together.  With psi = exp(-1/n) well below the critical coupling
  (G_c = -e^2/3 = -2.46) the slabs do not settle: they keep breathing
  (max|u| ~ 1e-2 .. 1e-1 for 10^6 steps, on the CPU oracle as on the GPU), so
  the bulk densities are averaged over the second half of the run and their
  spread is reported; the slabs that blow up are reported as diverged.  The
  thermodynamic coexistence (``sclbm.thermo``, the reference's SCThermo) is
  the starting guess and the comparison.
* ``ragged_sweep(...)``: droplets of radius R in boxes of side 4R rounded up
  to a multiple of 32, couplings G, all in one ``Batch`` (FP32-shifted storage
  shifted by the gas density, FP64 reductions), retired one by one as they
  converge.  At every check the FP64 mass of each lattice is restored (FP32
  rounding repeats in a near-steady state and would drift the mass
  linearly).
* ``plain_run(...)``: the same droplet on the plain FP64 GPU path.

Convergence.  A Shan-Chen droplet keeps steady spurious currents (max|u| of
0.1 .. 0.3 here), so max|u| never falls to 1e-9; the criteria are the
reference's: the FP64 run stops when u_conv = sum|u(t) - u(t-K)| / V < 1e-12
(CheckUConvergenceSCMP, idpy/LBM/MultiPhaseLoopChecks.py:96-163, FP64
threshold); the FP32 batch stops when the Laplace pressure changes by less
than ``tol_dp`` (relative) between ``patience`` consecutive checks
(CheckCenterOfMassDeltaPConvergence, MultiPhaseLoopChecks.py:35-91, whose
threshold is 1e-5), and reports the mean of those last values.
"""
import math
import time

import numpy as np

from . import _lib
from .LBM import XIStencils, FStencils
from .profiles import droplet
from . import thermo


def psi_exp(n):
    return np.exp(-1.0 / n)


def laplace_dp(n_in, n_out, G, c2=1.0 / 3, e2=1.0, psi=psi_exp):
    """p = c2 n + G e2 psi^2 / 2 (PBulk, idpy/LBM/MultiPhase.py:1759-1768)."""
    p = lambda n: c2 * n + 0.5 * G * e2 * psi(n) ** 2
    return p(n_in) - p(n_out), p(n_in), p(n_out)


def slab(L, n_l, n_g, width=4.0, rows=4):
    """Periodic liquid slab in x (two flat interfaces at L/4 and 3L/4)."""
    x = np.arange(L, dtype=np.float64)
    prof = n_g + 0.5 * (n_l - n_g) * (np.tanh((x - L / 4) / width) - np.tanh((x - 3 * L / 4) / width))
    return np.tile(prof, (rows, 1))


def thermo_guess(G, stencil='D2E8'):
    """(rho_l, rho_g) of the thermodynamic flat-interface construction, or None."""
    f = FStencils[stencil]
    try:
        t = thermo.coexistence(G, f['Es'], f['Ws'])
        return t['n_l'], t['n_g']
    except (ValueError, RuntimeError):
        return None


def coexistence_many(Gs, stencil='D2E8', L=128, rows=4, steps=200000, sample_every=2000, tol=1e-11,
                     width=4.0, device=0):
    """Flat-interface (slab) runs for many couplings at once on the FP64 plain
    path.  Returns per G: rho_l, rho_g (final values if the slab settled, else
    means over the second half), their spread, max|u| at the end, status
    'steady' / 'breathing' / 'diverged', and the thermodynamic values."""
    x, f = XIStencils['D2Q9'], FStencils[stencil]
    sims, out = [], []
    for G in Gs:
        th = thermo_guess(G, stencil)
        nl0, ng0 = th if th else (max(0.25, 4.6 + 1.4 * (-4.5 - G)), 0.2)
        s = _lib.Sim(2, (L, rows), x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], G, literals=_lib.LIT_EXACT,
                     device=device)
        s.set_density(slab(L, nl0, ng0, width, rows))
        s.set_velocity(np.zeros(2 * s.V))
        s.init_populations()
        sims.append(s)
        out.append(dict(G=float(G), thermo_rho_l=th[0] if th else None, thermo_rho_g=th[1] if th else None,
                        samples=[]))
    probe = [L // 2, 0]
    for k in range(steps // sample_every):
        for s in sims:
            s.step(sample_every, sync=False)
        if 2 * (k + 1) * sample_every > steps:
            for i, s in enumerate(sims):
                out[i]['samples'].append(s.density_at(probe))
    for i, s in enumerate(sims):
        smp = np.array(out[i].pop('samples'))
        s.compute_moments()
        s.check_u()
        s.step(sample_every)
        s.compute_moments()
        uc, mu = s.check_u()
        fin = np.isfinite(smp).all() and np.isfinite(uc) and s.density_finite()[0]
        o = out[i]
        o.update(steps=steps, u_conv=float(uc), max_u=float(mu))
        if not fin:
            o.update(status='diverged', rho_l=float('nan'), rho_g=float('nan'))
        elif uc < tol:
            n = s.density_at(probe)
            o.update(status='steady', rho_l=float(n[0]), rho_g=float(n[1]), rho_l_spread=0.0, rho_g_spread=0.0)
        else:
            o.update(status='breathing', rho_l=float(smp[:, 0].mean()), rho_g=float(smp[:, 1].mean()),
                     rho_l_spread=float(smp[:, 0].std()), rho_g_spread=float(smp[:, 1].std()))
        s.close()
    return out


def sweep_geometry(radii, multiple=32, factor=4):
    return [int(math.ceil(factor * R / multiple) * multiple) for R in radii]


def ragged_sweep(radii, G, rho_l, rho_g, stencil='D2E8', tau=1.0, width=2.0, check_every=500, tol_dp=2e-5,
                 patience=4, max_steps=200000, noise=0.0, seed=0, device=0, init=None, mass_fix=True,
                 residual_steps=100, residual_max=None, return_fields=False, dim=2, boxes=None, probe_rad=None,
                 compensate=None):
    """Run all droplets in one FP32 batch until each converges; returns a dict
    of per-droplet arrays and the wall time.  ``init`` may give initial
    density fields (e.g. a learned warm start) instead of the tanh profile,
    shifted by a constant to the tanh start's mass; with ``residual_max``
    every such start is first stepped ``residual_steps`` steps, and a lattice
    whose density changed by more than residual_max (relative L2 norm of the
    change against the spread of the start) is restarted from the tanh
    profile (cold-start fallback)."""
    boxes = list(boxes) if boxes is not None else sweep_geometry(radii)
    sizes = [(L,) * dim for L in boxes]
    n = len(radii)
    t0 = time.perf_counter()
    cold = lambda i: droplet(sizes[i], radii[i], rho_l[i], rho_g[i], width, seed + i, noise)
    if init is not None:
        # a given start carries the mass of the tanh start, so both reach the same equilibrium
        init = [np.asarray(f, np.float64) + (cold(i).sum() - np.sum(f)) / np.size(f) for i, f in enumerate(init)]
    # the shift is the gas density: most cells are gas, whose small
    # populations then keep most of their FP32 digits
    b = Batch_(XIStencils['D2Q9' if dim == 2 else 'D3Q19'], FStencils[stencil], sizes, G, list(rho_g), tau=tau,
               device=device)
    if dim == 2:
        # 64-cell tiles: boxes of 32 .. 288 cells leave 256-cell rows part
        # empty, and a few boxes make too few items to fill the GPU (same
        # results, bit for bit; ~30 % shorter steps with 20-30 boxes active)
        b.set_tile_width(64)
    # compensated rest population (compensate None: on in 2D, where the
    # droplets then meet the criterion sooner; off in 3D, where it costs 11 %
    # of the batch time and the sampled dP stay within 1e-5 of FP64 without it)
    if not (compensate if compensate is not None else dim == 2):
        try:
            b.set_mass_compensation(False)
        except _lib.SclbmError as e:
            # built for 3D batches with paired halo loads only: the others keep it
            if e.status != _lib.ERR_UNSUPPORTED:
                raise
    for i in range(n):
        b.set_density(i, init[i] if init is not None else cold(i))
    b.init_populations()
    # the Laplace-pressure probes: single cells, as DeltaPLaplace reads them
    # (probe_rad > 0 averages a bulk block about each)
    b.set_probe_radius(0 if probe_rad is None else probe_rad)
    residual = np.full(n, np.nan)
    fallback = np.zeros(n, bool)
    if init is not None and residual_max is not None:
        b.step(residual_steps)
        for i in range(n):
            d = b.get_density(i) - init[i]
            residual[i] = np.linalg.norm(d) / max(np.linalg.norm(init[i] - init[i].mean()), 1e-300)
            if not (residual[i] <= residual_max):
                fallback[i] = True
                b.set_density(i, cold(i))
                b.init_lattice(i)
    m0 = b.restore_mass()
    active = np.ones(n, np.int32)
    u_conv, max_u = np.full(n, np.nan), np.full(n, np.nan)
    status = np.array(['running'] * n, dtype=object)
    hist = [[] for _ in range(n)]
    calm = np.zeros(n, np.int64)
    n_in, n_out = np.full(n, np.nan), np.full(n, np.nan)
    b.check()  # u_old := u of the initial state
    total = 0
    while active.any() and total < max_steps:
        b.step(check_every, sync=False)
        total += check_every
        uc, mu, _ = b.check()
        if mass_fix:
            b.restore_mass(m0)
        ni, no = b.probe()
        for i in np.nonzero(active)[0]:
            u_conv[i], max_u[i] = uc[i], mu[i]
            n_in[i], n_out[i] = ni[i], no[i]
            dp = laplace_dp(ni[i], no[i], G[i])[0]
            if not (np.isfinite(uc[i]) and np.isfinite(dp)):
                status[i], active[i] = 'diverged', 0
                continue
            if hist[i] and abs(dp - hist[i][-1]) <= tol_dp * abs(dp):
                calm[i] += 1
            else:
                calm[i] = 0
            hist[i].append(dp)
            if calm[i] >= patience:
                status[i], active[i] = 'converged', 0
        if not active.all():
            b.set_active(active)
    steps = b.steps()
    wall = time.perf_counter() - t0
    fields = [b.get_density(i) for i in range(n)] if return_fields else None
    b.close()
    status[status == 'running'] = 'max_steps'
    # converged: the mean of the calm checks; otherwise the last value
    dp = np.array([(np.mean(h[-patience:]) if st == 'converged' else h[-1]) if h else np.nan
                   for h, st in zip(hist, status)])
    return dict(radii=np.array(radii), boxes=np.array(boxes), G=np.array(G), steps=steps, u_conv=u_conv,
                max_u=max_u, status=status, dp=dp, n_in=n_in, n_out=n_out, wall_s=wall, residual=residual,
                fallback=fallback, fields=fields, dp_history=hist)


def plain_run(R, G, rho_l, rho_g, stencil='D2E8', tau=1.0, width=2.0, check_every=500, tol=1e-12,
              max_steps=200000, noise=0.0, seed=0, device=0, tol_dp=2e-5, patience=4, dim=2, L=None,
              stop_at_dp=False, literals=None):
    """One droplet on the plain FP64 GPU path (exact coefficients; ``literals``
    _lib.LIT_FACTORED factors the BGK operator as well), stopped by
    the reference's FP64 criterion u_conv < tol.  The step and wall time at
    which the FP32 batch's criterion (Laplace pressure calm to tol_dp for
    `patience` checks) would first have stopped it are recorded too; with
    stop_at_dp the run stops there (the same criterion as the batch; the
    Laplace pressure is then the mean of the calm checks, as the batch's)."""
    L = L or sweep_geometry([R])[0]
    dims = (L,) * dim
    x, f = XIStencils['D2Q9' if dim == 2 else 'D3Q19'], FStencils[stencil]
    t0 = time.perf_counter()
    s = _lib.Sim(dim, dims, x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], G, tau=tau,
                 literals=_lib.LIT_EXACT if literals is None else literals, device=device)
    s.set_density(droplet(dims, R, rho_l, rho_g, width, seed, noise))
    s.set_velocity(np.zeros(dim * s.V))
    s.init_populations()
    s.compute_moments()
    s.check_u()
    steps, uc, mu, status = 0, float('nan'), float('nan'), 'max_steps'
    c = L // 2
    probe = [c + L * c + (L * L * c if dim == 3 else 0), s.V - 1]
    prev, calm, steps_dp, wall_dp, hist = None, 0, None, None, []
    while steps < max_steps:
        s.step(check_every)
        steps += check_every
        s.compute_moments()
        uc, mu = s.check_u()
        if not np.isfinite(uc) or not s.density_finite()[0]:
            status = 'diverged'
            break
        if steps_dp is None:
            ni, no = s.density_at(probe)
            dp = laplace_dp(ni, no, G)[0]
            calm = calm + 1 if prev is not None and abs(dp - prev) <= tol_dp * abs(dp) else 0
            prev = dp
            hist.append(dp)
            if calm >= patience:
                steps_dp, wall_dp = steps, time.perf_counter() - t0
                if stop_at_dp:
                    status = 'converged'
                    break
        if uc < tol and not stop_at_dp:
            status = 'converged'
            break
    ni, no = s.density_at(probe)
    s.close()
    dp_end = laplace_dp(ni, no, G)[0]
    if stop_at_dp and status == 'converged':
        dp_end = float(np.mean(hist[-patience:]))
    return dict(R=R, L=L, steps=steps, u_conv=uc, max_u=mu, status=status, dp=dp_end, n_in=ni,
                n_out=no, wall_s=time.perf_counter() - t0, steps_dp=steps_dp, wall_dp_s=wall_dp)


def laplace_fit(G=-4.5, radii=(12, 16, 20, 24, 32, 40, 48), stencil='D2E8', device=0, **kw):
    """Laplace test at one coupling: the FP32 batch at several radii, then
    dP = sigma / R + c fitted by least squares (2D Laplace law); returns
    sigma, c, the per-droplet values and the thermodynamic sigma_f."""
    f = FStencils[stencil]
    th = thermo.coexistence(G, f['Es'], f['Ws'])
    radii = list(radii)
    r = ragged_sweep(radii, [G] * len(radii), [th['n_l']] * len(radii), [th['n_g']] * len(radii),
                     stencil=stencil, device=device, return_fields=True, **kw)
    ok = r['status'] == 'converged'
    # equimolar radius of each equilibrated droplet: the area the liquid would
    # fill at the measured inside / outside densities, A = (M - n_out V) / (n_in - n_out)
    req = []
    for j, fld in enumerate(r['fields']):
        A = (fld.sum() - r['n_out'][j] * fld.size) / (r['n_in'][j] - r['n_out'][j])
        req.append(math.sqrt(max(A, 0.0) / math.pi))
    req = np.array(req)

    def fit(R):
        M = np.stack([1.0 / R[ok], np.ones(ok.sum())], 1)
        (sg, c), *_ = np.linalg.lstsq(M, r['dp'][ok], rcond=None)
        return float(sg), float(c)

    sigma, c = fit(r['radii'].astype(float))
    sigma_eq, c_eq = fit(req)
    # the curvature (Tolman) correction of the 2D Laplace law instead of a
    # constant offset: dP R = sigma + b / R, fitted on the equimolar radii; a
    # free intercept in dP = sigma / R + c absorbs the 1/R^2 term and lowers sigma
    M = np.stack([np.ones(ok.sum()), 1.0 / req[ok]], 1)
    (sigma_t, b_t), *_ = np.linalg.lstsq(M, r['dp'][ok] * req[ok], rcond=None)
    return dict(G=G, sigma=sigma, intercept=c, sigma_equimolar=sigma_eq, intercept_equimolar=c_eq,
                sigma_tolman=float(sigma_t), tolman_b=float(b_t),
                sigma_thermo=th['sigma_f'], radii=[int(v) for v in r['radii']],
                radii_equimolar=[float(v) for v in req], dp=[float(v) for v in r['dp']],
                n_in=[float(v) for v in r['n_in']], n_out=[float(v) for v in r['n_out']],
                rho_l_thermo=th['n_l'], rho_g_thermo=th['n_g'],
                status=[str(v) for v in r['status']], steps=[int(v) for v in r['steps']])


def run_sweep(n=64, r_min=8, seed=2024, G_range=(-6.0, -4.5), stencil='D2E8', check_every=500, tol_dp=2e-5,
              tol64=1e-12, max_steps=100000, coex_steps=200000, plain=True, device=0, init=None, mlp=None,
              residual_max=0.1, plain_stop_at_dp=False, plain_literals=None, plain_extra_literals=()):
    """The ragged droplet sweep: radii r_min .. r_min+n-1, box 4R rounded up to
    32, G uniform in G_range (seeded), densities from the flat-interface runs
    (from the thermodynamic construction where the slab diverged); batched
    FP32 run vs the plain FP64 path droplet by droplet."""
    rng = np.random.default_rng(seed)
    radii = list(range(r_min, r_min + n))
    Gs = rng.uniform(G_range[0], G_range[1], n)
    t0 = time.perf_counter()
    coex = coexistence_many(Gs, stencil=stencil, steps=coex_steps, device=device)
    t_coex = time.perf_counter() - t0
    rl, rg, source = [], [], []
    for c in coex:
        ok = c['status'] != 'diverged'
        rl.append(c['rho_l'] if ok else c['thermo_rho_l'])
        rg.append(c['rho_g'] if ok else c['thermo_rho_g'])
        source.append('flat interface (%s)' % c['status'] if ok else 'thermodynamics')
    sw = ragged_sweep(radii, [float(g) for g in Gs], rl, rg, stencil=stencil, check_every=check_every,
                      tol_dp=tol_dp, max_steps=max_steps, device=device, init=init)
    warm = None
    if mlp is not None:
        # the same droplets started from the network's predicted profiles,
        # their radii set so that each carries the mass of its tanh start
        from .warmstart import warm_fields
        t1 = time.perf_counter()
        masses = [droplet((L, L), R, a, b_, 2.0, 0, 0.0).sum()
                  for R, L, a, b_ in zip(radii, sweep_geometry(radii), rl, rg)]
        fields = warm_fields(mlp, radii, [float(g) for g in Gs], order=int(stencil[-1]), masses=masses)
        t_pred = time.perf_counter() - t1
        warm = ragged_sweep(radii, [float(g) for g in Gs], rl, rg, stencil=stencil, check_every=check_every,
                            tol_dp=tol_dp, max_steps=max_steps, device=device, init=fields,
                            residual_max=residual_max)
        warm['predict_wall_s'] = t_pred
        warm['wall_s'] += t_pred
    unstable = []
    for i in range(n):
        why = []
        if coex[i]['status'] == 'diverged':
            why.append('flat interface diverged (droplet densities from thermodynamics)')
        if sw['status'][i] == 'diverged':
            why.append('droplet diverged after %d steps (FP32 batch)' % sw['steps'][i])
        if why:
            unstable.append(dict(R=radii[i], G=float(Gs[i]), reason='; '.join(why)))
    res = dict(config=dict(n=n, radii=[r_min, r_min + n - 1], box='4R rounded up to 32', G_range=list(G_range),
                           seed=seed, stencil=stencil, tau=1.0, check_every=check_every, tol_dp_fp32=tol_dp,
                           patience=4, tol_u_fp64=tol64, coexistence_steps=coex_steps,
                           fp32_shift='rho_g per droplet', fp32_mass='restored to the initial FP64 mass at each check',
                           criterion_fp32='relative change of the Laplace pressure between checks '
                                          '(CheckCenterOfMassDeltaPConvergence)',
                           criterion_fp64='u_conv = sum|u(t)-u(t-K)|/V < tol (CheckUConvergenceSCMP)'),
               coexistence_wall_s=t_coex, unstable=unstable, batch=sw, coexistence=coex, rho_l=rl, rho_g=rg,
               rho_source=source, warm=warm)
    if plain:
        # the plain FP64 arm (plain_literals: None = exact coefficients, or
        # _lib.LIT_FACTORED), and optionally the same arm in other arithmetics
        def arm(lit):
            runs = []
            t1 = time.perf_counter()
            for i in range(n):
                if sw['status'][i] == 'diverged':
                    runs.append(None)
                    continue
                runs.append(plain_run(radii[i], float(Gs[i]), rl[i], rg[i], stencil=stencil, check_every=check_every,
                                      tol=tol64, max_steps=max_steps, device=device, tol_dp=tol_dp,
                                      stop_at_dp=plain_stop_at_dp, literals=lit))
            return runs, time.perf_counter() - t1
        res['plain'], res['plain_wall_s'] = arm(plain_literals)
        res['plain_extra'] = {}
        for lit in plain_extra_literals:
            runs, wall = arm(lit)
            res['plain_extra'][int(lit)] = dict(runs=runs, wall_s=wall)
    return res


def run_sweep3d(n=256, seed=2025, R_range=(10.0, 30.0), G_range=(-6.0, -4.5), L=96, stencil='D3E6', check_every=500,
                tol_dp=2e-5, tol64=1e-12, max_steps=20000, plain_sample=8, device=0, mlp=None, residual_max=None,
                plain_stop_at_dp=False, plain_literals=None):
    """Batched 3D droplets: n D3Q19 droplets, radius and G uniform in their
    ranges (seeded), each in an L^3 periodic box, FP32-shifted batches (split
    so that Q * cells < 2^31 per batch); then the plain FP64 path, cold
    started, on `plain_sample` of the droplets the batch converged, timed one
    after another.  Start densities: the flat-interface thermodynamic
    construction of the 2D stencil of the same order (sclbm.thermo has the 2D
    pressure-tensor constants).  With ``mlp`` (a network trained on 3D
    profiles, warmstart.equilibrium_profiles_3d) the same droplets are run
    again from its predicted radial profiles (mass-matched to the tanh starts)
    with the cold-start fallback above ``residual_max``."""
    rng = np.random.default_rng(seed)
    radii = rng.uniform(*R_range, n)
    Gs = rng.uniform(*G_range, n)
    guess = [thermo_guess(g, 'D2E' + stencil[-1]) or (4.6, 0.2) for g in Gs]
    rl = [a for a, _ in guess]
    rg = [b for _, b in guess]
    per = max(1, ((1 << 31) - 1) // (19 * L ** 3) - 1)
    groups = np.array_split(np.arange(n), int(math.ceil(n / per)))
    t0 = time.perf_counter()
    parts = []
    for gi in groups:
        parts.append(ragged_sweep([float(radii[i]) for i in gi], [float(Gs[i]) for i in gi], [rl[i] for i in gi],
                                  [rg[i] for i in gi], stencil=stencil, check_every=check_every, tol_dp=tol_dp,
                                  max_steps=max_steps, device=device, dim=3, boxes=[L] * len(gi), seed=seed))
    wall = time.perf_counter() - t0
    cat = lambda k: np.concatenate([p[k] for p in parts])
    batch = dict(radii=radii, G=Gs, steps=cat('steps'), status=cat('status'), dp=cat('dp'), max_u=cat('max_u'),
                 wall_s=wall, batches=[len(g) for g in groups])
    warm = None
    if mlp is not None:
        from .warmstart import warm_fields
        t1 = time.perf_counter()
        wparts = []
        for gi in groups:
            masses = [droplet((L,) * 3, float(radii[i]), rl[i], rg[i], 2.0, seed + k, 0.0).sum()
                      for k, i in enumerate(gi)]
            fields = warm_fields(mlp, [float(radii[i]) for i in gi], [float(Gs[i]) for i in gi], tau=1.0,
                                 order=int(stencil[-1]), masses=masses, dim=3, box=L)
            wparts.append(ragged_sweep([float(radii[i]) for i in gi], [float(Gs[i]) for i in gi],
                                       [rl[i] for i in gi], [rg[i] for i in gi], stencil=stencil,
                                       check_every=check_every, tol_dp=tol_dp, max_steps=max_steps, device=device,
                                       dim=3, boxes=[L] * len(gi), seed=seed, init=fields,
                                       residual_max=residual_max))
            del fields
        wcat = lambda k: np.concatenate([p[k] for p in wparts])
        warm = dict(steps=wcat('steps'), status=wcat('status'), dp=wcat('dp'), residual=wcat('residual'),
                    fallback=wcat('fallback'), wall_s=time.perf_counter() - t1)
    ok = np.nonzero(batch['status'] == 'converged')[0]
    pick = rng.choice(ok, size=min(plain_sample, len(ok)), replace=False) if len(ok) else []
    plain = []
    for i in pick:
        r = plain_run(float(radii[i]), float(Gs[i]), rl[i], rg[i], stencil=stencil, check_every=check_every,
                      tol=tol64, max_steps=max_steps, device=device, dim=3, L=L, seed=seed + int(i),
                      tol_dp=tol_dp, stop_at_dp=plain_stop_at_dp, literals=plain_literals)
        r['index'] = int(i)
        plain.append(r)
    return dict(config=dict(n=n, seed=seed, R_range=list(R_range), G_range=list(G_range), box=L, stencil=stencil,
                            tau=1.0, check_every=check_every, tol_dp_fp32=tol_dp, tol_u_fp64=tol64,
                            max_steps=max_steps, plain_sample=len(plain)),
                batch=batch, plain=plain, rho_l=rl, rho_g=rg, warm=warm)


# late import (batch imports MultiPhase, which imports this package's _lib)
from .batch import Batch as Batch_  # noqa: E402
