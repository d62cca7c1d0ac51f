"""Derivation of the polynomial coefficients of the FP32 inverse normal (rg_common.cuh,
rg_ninv32_lower).  Run with numpy and scipy: ``python probit32_fit.py``.  Not used at build or run
time; it reproduces the constants in the source.

For the lower-tail probability p <= 1/2 write s = 1 - 2p and w = -ln(4 p (1 - p)) = -ln(1 - s^2).
Then -Phi^-1(p) = s * g(w) with g(w) = sqrt(2) * erfinv(s) / s, a smooth function of w (g(0) =
sqrt(pi/2)).  g is fitted with near-minimax relative error (Lawson iterations on a weighted
Chebyshev least-squares fit, targets from scipy's double-precision ndtri):

* central branch, w in [0, 5] (p >= 0.0017, 99.6% of draws): degree 8 in t = w - 2.5;
* tail branch, w in [5, 27] (p down to 1e-12): degree 11 in v = sqrt(w) - (sqrt(5) + sqrt(27)) / 2.

The fits' relative errors are 9.4e-8 and 1.1e-8; evaluated in FP32 from the 32-bit Sobol integer
(w from p2 = 2p and s as -ln(p2 (1 + s))) the result is within 4e-7 relative of the exact
inverse normal, which the FP64 lane's Acklam approximation matches to 1.15e-9.
"""
import numpy as np
from numpy.polynomial import chebyshev as Ch
from scipy.special import ndtri


def g_exact(w):
    e = np.exp(-w)
    s = np.sqrt(-np.expm1(-w))        # s = 1 - 2p
    p = e / (2.0 * (1.0 + s))          # 4p(1-p) = e^-w, formed without cancellation
    return -ndtri(p) / s


def fit(a, b, deg, to_w, iters=400, n=30000):
    t = np.cos(np.pi * (np.arange(n) + 0.5) / n)
    x = (a + b) / 2 + (b - a) / 2 * t
    f = g_exact(to_w(x))
    c = Ch.chebfit(t, f, deg, w=1 / f)
    wt = np.ones_like(t)
    for _ in range(iters):
        r = Ch.chebval(t, c) / f - 1
        wt = wt * np.abs(r)
        wt /= wt.sum()
        c = Ch.chebfit(t, f, deg, w=np.sqrt(wt) / f)
    err = np.abs(Ch.chebval(t, c) / f - 1).max()
    # monomial coefficients in the centred variable x - (a + b) / 2
    h = (b - a) / 2
    mono = Ch.cheb2poly(c) / h ** np.arange(deg + 1)
    return mono, err


if __name__ == "__main__":
    central, e1 = fit(0.0, 5.0, 8, lambda x: x)
    tail, e2 = fit(np.sqrt(5.0), np.sqrt(27.0), 11, lambda v: v * v)
    print("centre of the tail variable:", (np.sqrt(5.0) + np.sqrt(27.0)) / 2)
    print("central, ascending powers of (w - 2.5), rel. err %.2e:" % e1)
    print(", ".join("%.9ef" % c for c in central))
    print("tail, ascending powers of (sqrt(w) - centre), rel. err %.2e:" % e2)
    print(", ".join("%.9ef" % c for c in tail))
