"""Shan-Chen thermodynamics: critical point, coexistence and surface tension.

Host-side restatement of the reference's ``idpy/LBM/SCThermo.py``:

* bulk pressure p(n) = theta n + G e2 psi(n)^2 / 2 (``ShanChen.P``, :83-85);
* critical point from p' = p'' = 0 (``ShanChen.__init__``, :104-115);
* spinodal extrema of p(n) and the coexistence range, i.e. the gas density
  at the pressure of the liquid-branch minimum and the liquid density at the
  pressure of the gas-branch maximum (``FindExtrema`` :75-90,
  ``FindCoexistenceRange`` :160-186);
* the flat-interface mechanical equilibrium with Guo forcing: the pair
  (n_g, n_l) at equal pressure p0 with
      int_{n_g}^{n_l} (p0 - p(n)) psi'(n) / psi(n)^(1 + eps) dn = 0
  (``FlatInterface`` :190-335), where eps = -2 alpha / beta comes from the
  force stencil's weights grouped by squared length (``PressureTensor``
  :431-575);
* the surface tension sigma = G sigma_c int (dn/dx) psi'^2 dn with
  dn/dx = sqrt(24 psi^eps I(n) / (beta G psi'^2)), I(n) the same integral from
  n_g to n (``DNDXLambda``/``SurfaceTension`` :337-352).

The reference evaluates these with sympy and scipy's bisect/quad; here the
same quantities are computed with closed forms where they exist and scipy's
brentq/quad otherwise.  The golden values in tests/golden/thermo.json come from
the reference's own ``ShanChanEquilibriumCache``.
"""
import math
import warnings

import numpy as np
from scipy import integrate, optimize

# per squared length of a stencil group: coefficients of the pressure-tensor
# constants alpha, beta and sigma_c (SCThermo.py:431-491)
_ALPHA = {4: 24, 5: 48, 8: 48, 9: 144, 10: 288, 13: 336, 16: 480, 17: 960}
_BETA = {1: 6, 2: 12, 4: 72, 5: 156, 8: 144, 9: 342, 10: 696, 13: 828, 16: 1056, 17: 2124}
_SIGMA_C = {1: -6, 4: -96, 5: -108, 9: -486, 10: -768, 13: -300, 16: -1536, 17: -2700}


class Psi:
    """psi(n) with its first two derivatives: 'exp' = exp(-1/n), '1mexp' = 1 - exp(-n)."""

    def __init__(self, kind='exp'):
        if kind not in ('exp', '1mexp'):
            raise ValueError('psi kind %r (exp, 1mexp)' % kind)
        self.kind = kind

    def __call__(self, n):
        return np.exp(-1.0 / n) if self.kind == 'exp' else 1.0 - np.exp(-n)

    def d1(self, n):
        return np.exp(-1.0 / n) / n ** 2 if self.kind == 'exp' else np.exp(-n)

    def d2(self, n):
        return np.exp(-1.0 / n) * (1.0 / n ** 4 - 2.0 / n ** 3) if self.kind == 'exp' else -np.exp(-n)

    def d1_over_pow(self, n, eps):
        """psi' / psi^(1 + eps), evaluated without underflow for small n."""
        if self.kind == 'exp':
            return np.exp(eps / n) / n ** 2
        return np.exp(-n) / (1.0 - np.exp(-n)) ** (1.0 + eps)


def stencil_groups(es, ws):
    """{squared length: weight} of a force stencil (vectors es, weights ws)."""
    es = np.asarray(es)
    ws = np.asarray(ws, np.float64)
    l2 = (es ** 2).sum(1)
    out = {}
    for k in np.unique(l2):
        w = ws[l2 == k]
        if not np.allclose(w, w[0], rtol=0, atol=1e-15):
            raise ValueError('weights of squared length %d differ' % k)
        out[int(k)] = float(w[0])
    return out


def stencil_constants(es, ws):
    """alpha, beta, eps = -2 alpha / beta, sigma_c and e2 of a 2D force stencil."""
    g = stencil_groups(es, ws)
    alpha = -sum(_ALPHA.get(k, 0) * w for k, w in g.items())
    beta = sum(_BETA.get(k, 0) * w for k, w in g.items())
    sigma_c = sum(_SIGMA_C.get(k, 0) * w for k, w in g.items()) / 12.0
    es = np.asarray(es)
    e2 = float((np.asarray(ws) * es[:, 0] ** 2).sum())
    return dict(alpha=alpha, beta=beta, eps=-2.0 * alpha / beta, sigma_c=sigma_c, e2=e2)


class ShanChen:
    """Bulk thermodynamics of the Shan-Chen equation of state at coupling G."""

    def __init__(self, G, psi='exp', theta=1.0 / 3, e2=1.0, n_eps=0.01):
        self.G, self.theta, self.e2, self.n_eps = float(G), float(theta), float(e2), float(n_eps)
        self.psi = Psi(psi)
        self.n_c, self.G_c = self.critical_point()
        self.P_c = self.p(self.n_c, self.G_c)
        if self.G * self.e2 > self.G_c * self.e2:
            raise ValueError('G = %g is above the critical coupling %g: no phase separation' % (self.G, self.G_c))
        self.extrema = self.find_extrema()
        self.coexistence_range = self.find_coexistence_range()

    def p(self, n, G=None):
        G = self.G if G is None else G
        return self.theta * n + 0.5 * G * self.e2 * self.psi(n) ** 2

    def dp(self, n):
        return self.theta + self.G * self.e2 * self.psi(n) * self.psi.d1(n)

    def critical_point(self):
        """(n_c, G_c): (psi psi')' = 0 fixes n_c, then p'(n_c) = 0 fixes G_c."""
        if self.psi.kind == 'exp':
            n_c = 1.0
        else:
            n_c = math.log(2.0)
        G_c = -self.theta / (self.e2 * self.psi(n_c) * self.psi.d1(n_c))
        return n_c, G_c

    def find_extrema(self):
        """[(n, p)] at the gas-branch maximum and the liquid-branch minimum of p."""
        # the liquid root of p = P_c bounds the extrema from above
        hi = self.n_eps
        while self.p(hi) - self.P_c <= 0 or hi < self.n_c:
            hi += self.n_eps
            if hi > 1e4:
                raise RuntimeError('no upper bound for the extrema')
        self.range_ext = hi
        ns = np.linspace(self.n_eps, hi, 4097)
        d = self.dp(ns)
        idx = np.nonzero(np.sign(d[1:]) != np.sign(d[:-1]))[0]
        if len(idx) < 2:
            raise RuntimeError('p(n) has no spinodal pair on [%g, %g]' % (self.n_eps, hi))
        out = []
        for i in idx[:2]:
            n = optimize.brentq(self.dp, ns[i], ns[i + 1], xtol=1e-15, rtol=1e-15)
            out.append((n, float(self.p(n))))
        return out

    def find_coexistence_range(self):
        (n1, p1), (n2, p2) = self.extrema
        if p2 > 0:
            left = optimize.brentq(lambda n: self.p(n) - p2, 1e-12, n1, xtol=1e-15, rtol=1e-15)
            left = (left, float(self.p(left)))
        else:
            left = (0.0, 0.0)
        right = optimize.brentq(lambda n: self.p(n) - p1, n2, self.range_ext + 1.0, xtol=1e-15, rtol=1e-15)
        return [left, (right, float(self.p(right)))]

    # ---- flat interface -------------------------------------------------
    def _pair(self, p0):
        (n1, _), (n2, _) = self.extrema
        g = optimize.brentq(lambda n: self.p(n) - p0, 1e-12, n1, xtol=1e-15, rtol=1e-15)
        lo, hi = n2, max(self.coexistence_range[1][0], n2) + 1.0
        while self.p(hi) - p0 < 0:
            hi *= 2.0
        l = optimize.brentq(lambda n: self.p(n) - p0, lo, hi, xtol=1e-15, rtol=1e-15)
        return g, l

    def _integral(self, p0, a, b, eps):
        f = lambda n: (p0 - self.p(n)) * self.psi.d1_over_pow(n, eps)
        with warnings.catch_warnings():
            # quad flags round-off when the integral is already near zero
            warnings.simplefilter('ignore', integrate.IntegrationWarning)
            return integrate.quad(f, a, b, limit=400, epsabs=1e-15, epsrel=1e-13)[0]

    def flat_interface(self, es, ws):
        """Mechanical equilibrium of a flat interface with Guo forcing for the
        force stencil (es, ws): dict(n_g, n_l, p_0, eps, sigma_f)."""
        k = stencil_constants(es, ws)
        eps = k['eps']
        (n1, p1), (n2, p2) = self.extrema
        lo = max(p2, float(self.p(self.coexistence_range[0][0] + self.n_eps)))
        hi = p1
        I = lambda p0: self._integral(p0, *self._pair(p0), eps)
        ps = np.linspace(lo, hi, 65)[1:-1]
        vals = np.array([I(p) for p in ps])
        s = np.nonzero(np.sign(vals[1:]) != np.sign(vals[:-1]))[0]
        if not len(s):
            raise RuntimeError('no mechanical equilibrium between p = %g and %g' % (lo, hi))
        p0 = optimize.brentq(I, ps[s[0]], ps[s[0] + 1], xtol=1e-16, rtol=1e-15)
        n_g, n_l = self._pair(p0)
        sigma = self.surface_tension(n_g, n_l, p0, eps, k['beta'], k['sigma_c'])
        return dict(n_g=n_g, n_l=n_l, p_0=float(p0), eps=eps, sigma_f=sigma)

    def surface_tension(self, n_g, n_l, p0, eps, beta, sigma_c):
        def dndx(n):
            v = 24.0 * self.psi(n) ** eps / (beta * self.G * self.psi.d1(n) ** 2) * \
                self._integral(p0, n_g, n, eps)
            return math.sqrt(max(v, 0.0))
        f = lambda n: dndx(n) * self.psi.d1(n) ** 2
        return self.G * sigma_c * integrate.quad(f, n_g, n_l, limit=200, epsabs=1e-13, epsrel=1e-10)[0]


def coexistence(G, es, ws, psi='exp', theta=1.0 / 3):
    """Flat-interface coexistence of the Shan-Chen fluid at coupling G for a
    force stencil: dict(G_c, n_c, n_l, n_g, p_0, eps, sigma_f)."""
    k = stencil_constants(es, ws)
    sc = ShanChen(G, psi=psi, theta=theta, e2=k['e2'])
    out = sc.flat_interface(es, ws)
    out.update(G_c=sc.G_c, n_c=sc.n_c, G=float(G))
    return out
