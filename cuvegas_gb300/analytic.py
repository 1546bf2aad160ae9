"""Closed-form integrals over [0,1]^d of the benchmark integrand families, used to check estimates.

- Gaussian, width s, centre m:  prod_d erf-difference; for m=0.5, s=0.1 the
  normalised form integrates to erf(5)^d.
- Two-Gaussian mixture:  sum_k w_k prod_d s_k sqrt(pi)/2 [erf((1-mu)/s)+erf(mu/s)],
  with analytic derivatives in w, s and mu.
- Product peak:  prod_d c_d [atan(c_d (1-u_d)) + atan(c_d u_d)].
- Corner peak:  (1/(d! prod c)) sum_{S subset [d]} (-1)^|S| / (1 + sum_{i in S} c_i),
  evaluated with mpmath at high precision (heavy cancellation) when available,
  else with a pairwise exact-rational recursion.
"""
import math
from fractions import Fraction

import numpy as np


def gauss_normalised(dim, mu=0.5, s=0.1):
    one = 0.5 * (math.erf((1 - mu) / s) + math.erf(mu / s))
    return one ** dim


def _g1(m, s):
    """int_0^1 exp(-((x-m)/s)^2) dx"""
    return s * math.sqrt(math.pi) / 2 * (math.erf((1 - m) / s) + math.erf(m / s))


def _g1_dm(m, s):
    return math.exp(-((0 - m) / s) ** 2) - math.exp(-((1 - m) / s) ** 2)


def _g1_ds(m, s):
    # d/ds of s*sqrt(pi)/2*(erf(a/s)+erf(b/s)), a=1-m, b=m
    a, b = 1 - m, m
    t = math.sqrt(math.pi) / 2 * (math.erf(a / s) + math.erf(b / s))
    t2 = -(a / s) * math.exp(-(a / s) ** 2) - (b / s) * math.exp(-(b / s) ** 2)
    return t + t2


def mixture(theta, dim):
    """theta = [w1, w2, s1, s2, mu1(dim), mu2(dim)]"""
    th = np.asarray(theta, dtype=np.float64)
    val = 0.0
    for k in range(2):
        w, s = th[k], th[2 + k]
        mu = th[4 + k * dim: 4 + (k + 1) * dim]
        val += w * np.prod([_g1(m, s) for m in mu])
    return val


def mixture_grad(theta, dim):
    th = np.asarray(theta, dtype=np.float64)
    g = np.zeros_like(th)
    for k in range(2):
        w, s = th[k], th[2 + k]
        mu = th[4 + k * dim: 4 + (k + 1) * dim]
        f = [_g1(m, s) for m in mu]
        P = np.prod(f)
        g[k] = P
        ds = 0.0
        for d in range(dim):
            others = np.prod([f[e] for e in range(dim) if e != d])
            ds += _g1_ds(mu[d], s) * others
            g[4 + k * dim + d] = w * _g1_dm(mu[d], s) * others
        g[2 + k] = w * ds
    return g


def product_peak(c, u):
    c = np.asarray(c, dtype=np.float64)
    u = np.asarray(u, dtype=np.float64)
    return float(np.prod(c * (np.arctan(c * (1 - u)) + np.arctan(c * u))))


def corner_peak(c):
    c = [float(v) for v in c]
    d = len(c)
    try:
        import mpmath as mp
        mp.mp.dps = 120
        cs = [mp.mpf(v) for v in c]
        sums = [mp.mpf(0)]
        signs = [1]
        for v in cs:                         # enumerate subsets incrementally
            sums = sums + [s + v for s in sums]
            signs = signs + [-g for g in signs]
        tot = mp.fsum(g / (1 + s) for g, s in zip(signs, sums))
        pc = mp.fprod(cs)
        return float(tot / (mp.factorial(d) * pc))
    except ImportError:
        # exact: divided differences of 1/(1+t) over the points c_i with signs
        fr = [Fraction(v) for v in c]
        sums = [Fraction(0)]
        signs = [1]
        for v in fr:
            sums = sums + [s + v for s in sums]
            signs = signs + [-g for g in signs]
        tot = sum(Fraction(g) / (1 + s) for g, s in zip(signs, sums))
        pc = Fraction(1)
        for v in fr:
            pc *= v
        return float(tot / (math.factorial(d) * pc))
