"""Coefficients of poly_sincos (cp3_device.cuh): near-minimax polynomials for sin and cos on
[0, pi/2] in the forms

    sin x = x + x^3 P(x^2),   cos x = 1 + x^2 Q(x^2),   P, Q of degree 4,

fitted by Lawson's iteratively reweighted least squares on Chebyshev nodes (a discrete
approximation of the minimax fit), with the targets evaluated in 40-digit arithmetic
(mpmath, shipped with sympy).  Prints the coefficients and the truncation error of the
float-rounded coefficients: the angle of (s, c) is what the kernels use, since they
renormalise (s, c) to unit modulus.

    python cudaprob3_gb300/csrc/fit_sincos.py
"""
import mpmath as mp
import numpy as np

mp.mp.dps = 40


def fit(kind, deg, n=4000, iters=60):
    x = np.pi / 4 * (1 + np.cos(np.pi * (np.arange(n) + 0.5) / n))
    xs = [mp.mpf(float(v)) for v in x]
    if kind == "sin":
        target = np.array([float(mp.sin(v) - v) for v in xs])
        A = np.stack([x ** (2 * k + 3) for k in range(deg)], 1)
    else:
        target = np.array([float(mp.cos(v) - 1) for v in xs])
        A = np.stack([x ** (2 * k + 2) for k in range(deg)], 1)
    w = np.ones(n)
    for _ in range(iters):
        c, *_ = np.linalg.lstsq(A * w[:, None], target * w, rcond=None)
        w = w * np.sqrt(np.abs(A @ c - target))
        w /= w.max()
    return c.astype(np.float32)


def horner(coef, v2):
    acc = mp.mpf(float(coef[-1]))
    for k in range(len(coef) - 2, -1, -1):
        acc = acc * v2 + mp.mpf(float(coef[k]))
    return acc


if __name__ == "__main__":
    S, C = fit("sin", 5), fit("cos", 5)
    print("kSin3..kSin11:", ", ".join("%.9e" % v for v in S))
    print("kCos2..kCos10:", ", ".join("%.9e" % v for v in C))
    es = ec = ea = mp.mpf(0)
    for v in np.linspace(0, np.pi / 2, 2001):
        v = mp.mpf(v)
        s = v + v ** 3 * horner(S, v * v)
        c = 1 + v * v * horner(C, v * v)
        es, ec = max(es, abs(s - mp.sin(v))), max(ec, abs(c - mp.cos(v)))
        ea = max(ea, abs(mp.atan2(s, c) - v))
    print("max error with float coefficients: sin %.2e, cos %.2e, angle %.2e" % (es, ec, ea))
