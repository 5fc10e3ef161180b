"""Derives the FP32 erfc approximation used by the real-space pair kernel.

erfc(x) = exp(-x^2) * g(x) with g = erfcx, the scaled complementary error
function.  On x in [0, 4] (alpha*r up to 4 covers Ewald tolerances down to
~1e-7 at the cutoff) g is smooth in t = 1 / (1 + 0.4 x), t in [0.385, 1],
so a degree-6 polynomial in t, least-squares fitted on Chebyshev nodes of t
(a near-minimax fit), holds g to ~3e-7 relative in exact arithmetic and
~5e-7 when evaluated by Horner's rule in FP32 (degree 8: 1e-8 and 2.5e-7,
two more multiply-adds per pair for no gain that FP32 keeps).  Run this
file to print the coefficients pasted into nxm_common.cuh.
"""
import numpy as np
from scipy.special import erfcx

P, X, DEG = 0.4, 4.0, 6


def fit():
    lo, hi = 1.0 / (1.0 + P * X), 1.0
    k = np.arange(4000)
    tn = 0.5 * (hi + lo) + 0.5 * (hi - lo) * np.cos(np.pi * (k + 0.5) / len(k))
    xn = (1.0 / tn - 1.0) / P
    return np.polynomial.polynomial.polyfit(tn, erfcx(xn), DEG)


if __name__ == "__main__":
    c = fit()
    x = np.linspace(0, X, 100001)
    t = 1.0 / (1.0 + P * x)
    print("max rel err (fp64 eval): %.2e" % np.abs(np.polynomial.polynomial.polyval(t, c) / erfcx(x) - 1).max())
    for i, v in enumerate(c):
        print("    %.9ef,  // t^%d" % (v, i))
