"""Learned warm start of droplet equilibria.

1. ``equilibrium_profiles``: droplets with seeded (G, R, tau, stencil order)
   are run to equilibrium by the plain method (the LBM itself, FP32 batches,
   one batch per (tau, order)), and each final density field is reduced to its
   radial profile (bins of half a lattice unit about the box centre L//2).
2. ``train``: the MLP (sclbm.mlp) learns rho(G, tau, R, order, r) from those
   profiles with the library's own BF16/FP32 training kernels (its scalar
   output is ln rho, scaled, so that the predicted density is positive and the
   gas keeps its relative accuracy).
3. ``evaluate``: profile RMSE and coexistence-density error (the predicted
   centre and far-field densities against the plain method's) on held-out
   profiles.
4. ``warm_fields``: initial density fields of new droplets from the predicted
   radial profile; ``sweep.ragged_sweep(init=..., residual_max=...)`` runs them
   and falls back to the tanh start where the warm start's residual (relative
   density change over its first steps) is too large.

The reference has no counterpart: it starts every droplet from a tanh profile
(InitRadialInterface, idpy/LBM/MultiPhase.py:1815-1852).
"""
import math
import time

import numpy as np

from . import thermo
from .LBM import FStencils
from .mlp import MLP
from .profiles import radius_field
from . import sweep

ORDERS = {4: 'D2E4', 6: 'D2E6', 8: 'D2E8'}

# input / output scaling of the network
_G0, _GS = -5.25, 0.75
_T0, _TS = 1.0, 0.2
_R0, _RS = 43.0, 37.0
_O0, _OS = 6.0, 2.0
_Y0, _YS = 0.5, 1.2   # the network's output is (ln rho - _Y0) / _YS: rho > 0 everywhere


def features(G, tau, R, order, r):
    G, tau, R, order, r = np.broadcast_arrays(*(np.asarray(v, np.float64) for v in (G, tau, R, order, r)))
    return np.stack([(G - _G0) / _GS, (tau - _T0) / _TS, (R - _R0) / _RS, (order - _O0) / _OS, (r - _R0) / _RS],
                    -1).astype(np.float32)


def to_target(rho):
    return ((np.log(np.asarray(rho, np.float64)) - _Y0) / _YS).astype(np.float32)


def from_target(y):
    return np.exp(_Y0 + _YS * np.asarray(y, np.float64))


def box_of(R):
    return int(math.ceil(4 * R / 32) * 32)


class ThermoTable:
    """Flat-interface coexistence densities (sclbm.thermo) on a G grid per
    stencil, interpolated: the tanh start of the profile runs."""

    def __init__(self, G_range=(-6.0, -4.5), points=31, orders=(4, 6, 8)):
        self.G = np.linspace(G_range[0], G_range[1], points)
        self.tab = {}
        for order in orders:
            f = FStencils[ORDERS[order]]
            v = [thermo.coexistence(g, f['Es'], f['Ws']) for g in self.G]
            self.tab[order] = (np.array([x['n_l'] for x in v]), np.array([x['n_g'] for x in v]))

    def __call__(self, G, order):
        l, g = self.tab[order]
        return float(np.interp(G, self.G, l)), float(np.interp(G, self.G, g))


def radial_profile(field, bin_width=0.5):
    """(r, rho) bin means of a square field about its centre L//2, r <= L/2."""
    dims = tuple(reversed(field.shape))
    r = radius_field(dims).ravel()
    rho = np.asarray(field, np.float64).ravel()
    sel = r <= min(dims) / 2
    k = (r[sel] / bin_width).astype(np.int64)
    cnt = np.bincount(k)
    ok = cnt > 0
    return np.bincount(k, r[sel])[ok] / cnt[ok], np.bincount(k, rho[sel])[ok] / cnt[ok]


def draw(n, seed, G_range=(-6.0, -4.5), R_range=(6.0, 80.0), taus=(0.8, 1.0, 1.2), orders=(4, 6, 8)):
    rng = np.random.default_rng(seed)
    return dict(G=rng.uniform(*G_range, n), R=rng.uniform(*R_range, n), tau=rng.choice(taus, n),
                order=rng.choice(orders, n))


def equilibrium_profiles(n=4096, seed=7, max_steps=60000, check_every=500, tol_dp=2e-5, device=0, table=None,
                         G_range=(-6.0, -4.5), R_range=(6.0, 80.0), taus=(0.8, 1.0, 1.2), orders=(4, 6, 8)):
    """Plain-method equilibrium profiles of n seeded droplets.  Returns
    (profiles, stats): one dict per droplet (G, tau, R, order, status, steps,
    r, rho) and the wall time / status counts."""
    d = draw(n, seed, G_range, R_range, taus, orders)
    table = table or ThermoTable(G_range, orders=orders)
    prof = [None] * n
    t0 = time.perf_counter()
    for tau in taus:
        for order in orders:
            idx = np.nonzero((d['tau'] == tau) & (d['order'] == order))[0]
            if not len(idx):
                continue
            rl, rg = zip(*[table(d['G'][i], order) for i in idx])
            r = sweep.ragged_sweep([float(d['R'][i]) for i in idx], [float(d['G'][i]) for i in idx], list(rl),
                                   list(rg), stencil=ORDERS[order], tau=float(tau), check_every=check_every,
                                   tol_dp=tol_dp, max_steps=max_steps, seed=seed, device=device,
                                   return_fields=True)
            for j, i in enumerate(idx):
                p = dict(G=float(d['G'][i]), tau=float(tau), R=float(d['R'][i]), order=int(order),
                         status=str(r['status'][j]), steps=int(r['steps'][j]), dp=float(r['dp'][j]))
                if p['status'] == 'converged':
                    p['r'], p['rho'] = radial_profile(r['fields'][j])
                prof[i] = p
    wall = time.perf_counter() - t0
    st = {}
    for p in prof:
        st[p['status']] = st.get(p['status'], 0) + 1
    return prof, dict(wall_s=wall, status=st)


def equilibrium_profiles_3d(n=128, seed=11, R_range=(10.0, 30.0), G_range=(-6.0, -4.5), L=96, stencil='D3E6',
                            max_steps=20000, check_every=500, tol_dp=2e-5, device=0):
    """Plain-method equilibrium profiles of n seeded 3D droplets (D3Q19, tau 1,
    cubic boxes of side L), in FP32 batches of at most 2^31 population values;
    start densities from the thermodynamic construction of the 2D stencil of
    the same order, as sweep.run_sweep3d starts them."""
    rng = np.random.default_rng(seed)
    R = rng.uniform(*R_range, n)
    G = rng.uniform(*G_range, n)
    guess = [sweep.thermo_guess(g, 'D2E' + stencil[-1]) or (4.6, 0.2) for g in G]
    per = max(1, ((1 << 31) - 1) // (19 * L ** 3) - 1)
    prof = []
    t0 = time.perf_counter()
    for gi in np.array_split(np.arange(n), int(math.ceil(n / per))):
        r = sweep.ragged_sweep([float(R[i]) for i in gi], [float(G[i]) for i in gi], [guess[i][0] for i in gi],
                               [guess[i][1] for i in gi], stencil=stencil, check_every=check_every, tol_dp=tol_dp,
                               max_steps=max_steps, device=device, dim=3, boxes=[L] * len(gi), seed=seed,
                               return_fields=True)
        for j, i in enumerate(gi):
            p = dict(G=float(G[i]), tau=1.0, R=float(R[i]), order=int(stencil[-1]), status=str(r['status'][j]),
                     steps=int(r['steps'][j]), dp=float(r['dp'][j]))
            if p['status'] == 'converged':
                p['r'], p['rho'] = radial_profile(r['fields'][j])
            prof.append(p)
        del r
    st = {}
    for p in prof:
        st[p['status']] = st.get(p['status'], 0) + 1
    return prof, dict(wall_s=time.perf_counter() - t0, status=st)


def split(profiles, holdout=512, seed=0, min_train_share=0.4):
    """(train, held out): `holdout` converged profiles held out, or fewer when
    that would leave less than min_train_share of them for training."""
    ok = [p for p in profiles if p['status'] == 'converged']
    rng = np.random.default_rng(seed)
    perm = rng.permutation(len(ok))
    k = min(holdout, int(len(ok) * (1 - min_train_share)))
    return [ok[i] for i in perm[k:]], [ok[i] for i in perm[:k]]


def samples(profiles):
    x = np.concatenate([features(p['G'], p['tau'], p['R'], p['order'], p['r']) for p in profiles])
    t = np.concatenate([to_target(p['rho']) for p in profiles])
    return x, t


def train(profiles, steps=20000, batch=8192, lr=1e-3, seed=0, device=0):
    """Train a fresh MLP on the profiles; returns (mlp, loss per step, wall s)."""
    x, t = samples(profiles)
    m = MLP(seed=seed, device=device)
    m.set_data(x, t)
    t0 = time.perf_counter()
    loss = m.train(steps, batch=batch, lr=lr)
    return m, loss, time.perf_counter() - t0


def predict_profile(m, G, tau, R, order, r):
    return from_target(m.predict(features(G, tau, R, order, r)))


def evaluate(m, profiles):
    """Profile RMSE (density units) and coexistence-density errors on profiles."""
    x, t = samples(profiles)
    y = from_target(m.predict(x))
    rho = from_target(t)
    err = y - rho
    per, cin, cout = [], [], []
    k = 0
    for p in profiles:
        nb = len(p['r'])
        e = err[k:k + nb]
        per.append(float(np.sqrt((e * e).mean())))
        cin.append(abs(e[0]) / p['rho'][0])
        cout.append(abs(e[-1]) / p['rho'][-1])
        k += nb
    return dict(n_profiles=len(profiles), n_samples=int(t.size), rmse=float(np.sqrt((err * err).mean())),
                rmse_median_profile=float(np.median(per)), rmse_max_profile=float(np.max(per)),
                coexistence_rel_err_liquid={'median': float(np.median(cin)), 'max': float(np.max(cin))},
                coexistence_rel_err_gas={'median': float(np.median(cout)), 'max': float(np.max(cout))})


def warm_fields(m, radii, G, tau=1.0, order=8, dr=0.02, masses=None, iterations=4, dim=2, box=None):
    """Initial density fields (box 4R rounded up to 32, or ``box``) from the
    predicted radial profiles, linearly interpolated in r.  The profiles are
    learned for r <= L/2; the corners beyond take the value at L/2.  With
    ``masses`` the radius fed to the network is adjusted (Newton steps on M(R))
    until each field carries that mass, so the extra or missing mass goes into
    the size of the droplet, not into its bulk densities.  dim = 3: spherical
    droplets in cubic boxes (a network trained on 3D profiles)."""
    boxes = [box or box_of(R) for R in radii]
    grids = [np.arange(0.0, L * (math.sqrt(dim) / 2) + 2 * dr, dr) for L in boxes]
    rfield = [radius_field((L,) * dim) for L in boxes]

    def fields_for(Rs):
        # the network saw r <= L/2 only: beyond, the value at L/2
        y = from_target(m.predict(np.concatenate([features(g, tau, R, order, np.minimum(rg, L / 2))
                                                  for R, g, rg, L in zip(Rs, G, grids, boxes)])))
        out, k = [], 0
        for rg, rf in zip(grids, rfield):
            out.append(np.interp(rf, rg, y[k:k + len(rg)]))
            k += len(rg)
        return out

    Rs = np.asarray(radii, np.float64)
    out = fields_for(Rs)
    if masses is None:
        return out
    for _ in range(iterations):
        mass = np.array([f.sum() for f in out])
        # dM/dR of a disc (sphere) of liquid in gas: 2 pi R (4 pi R^2) times (rho_in - rho_out)
        drho = np.array([f[tuple(n // 2 for n in f.shape)] - f[(-1,) * dim] for f in out])
        area = 2 * np.pi * Rs if dim == 2 else 4 * np.pi * Rs ** 2
        step = (np.asarray(masses) - mass) / np.maximum(area * drho, 1e-6)
        Rs = np.clip(Rs + step, 0.5 * np.asarray(radii), 1.5 * np.asarray(radii))
        out = fields_for(Rs)
    return out
