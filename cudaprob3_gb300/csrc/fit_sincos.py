"""Coefficients of poly_sincos_turns (cp3_device.cuh): near-minimax polynomials for
sin(2 pi x) and cos(2 pi x) on [0, 1/4] (x in turns) in the forms

    sin(2 pi x) = x (S1 + x^2 P(x^2)),   cos(2 pi x) = 1 + x^2 (C2 + x^2 Q(x^2)),

with S1 = 2 pi and C2 = -2 pi^2 as float pairs (hi + lo) and P, Q of degree 3, fitted by
Lawson's iteratively reweighted least squares on Chebyshev nodes (a discrete approximation
of the minimax fit), with the targets evaluated in 40-digit arithmetic (mpmath, shipped
with sympy).  Prints the constants and the truncation error with every coefficient rounded
to float: the angle of (s, c) is what the kernels use, since they renormalise (s, c) to unit
modulus.  Also prints kLoEFac / (2 pi) as a float pair (the phase rates are in turns).

    python cudaprob3_gb300/csrc/fit_sincos.py
"""
import mpmath as mp
import numpy as np

mp.mp.dps = 40
TWO_PI = 2 * mp.pi


def split(v):
    hi = np.float32(float(v))
    return hi, np.float32(float(v - mp.mpf(float(hi))))


S1, C2 = split(TWO_PI), split(-TWO_PI ** 2 / 2)


def fit(kind, deg, n=3000, iters=80):
    x = 0.125 * (1 + np.cos(np.pi * (np.arange(n) + 0.5) / n))  # Chebyshev nodes on [0, 1/4]
    xs = [mp.mpf(float(v)) for v in x]
    if kind == "sin":
        s1 = mp.mpf(float(S1[0])) + mp.mpf(float(S1[1]))
        target = np.array([float(mp.sin(TWO_PI * v) - s1 * v) for v in xs])
        A = np.stack([x ** (2 * k + 3) for k in range(deg)], 1)
    else:
        c2 = mp.mpf(float(C2[0])) + mp.mpf(float(C2[1]))
        target = np.array([float(mp.cos(TWO_PI * v) - 1 - c2 * v * v) for v in xs])
        A = np.stack([x ** (2 * k + 4) for k in range(deg)], 1)
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
    P, Q = fit("sin", 4), fit("cos", 4)
    print("kS1Hi, kS1Lo: %.9e, %.9e" % S1)
    print("kC2Hi, kC2Lo: %.9e, %.9e" % C2)
    print("kP3..kP9:", ", ".join("%.9e" % v for v in P))
    print("kQ4..kQ10:", ", ".join("%.9e" % v for v in Q))
    print("kLoEFac / (2 pi): %.9e, %.9e" % split(mp.mpf("2.534") / TWO_PI))
    ea = mp.mpf(0)
    for v in np.linspace(0, 0.25, 2001):
        v = mp.mpf(v)
        v2 = v * v
        s = v * (mp.mpf(float(S1[0])) + mp.mpf(float(S1[1])) + v2 * horner(P, v2))
        c = 1 + v2 * (mp.mpf(float(C2[0])) + mp.mpf(float(C2[1])) + v2 * horner(Q, v2))
        ea = max(ea, abs(mp.atan2(s, c) - TWO_PI * v))
    print("max angle error with float coefficients: %.2e rad" % ea)
