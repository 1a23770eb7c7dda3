"""The mathematics behind the mixed eigen-solver's eigenvectors and its fallback test, checked
in float64 on the CPU (the device code is the FP32 / double-float form of the same formulas,
compared with the oracle by the GPU tests).

* Rank-one update of the vacuum system: with H0 = O diag(mu) O^T (O = R13 R12, mu_k =
  DM(k,0)) and H = H0 + V e0 e0^T, the eigenvector of an eigenvalue l is u = O d with
  d_j = a_j prod_{i != j} (mu_i - l), a = O^T e0; |u| = |d|.  It vanishes for a state with no
  electron component (a_j = 0) at the decoupled eigenvalue, which is what sends such
  parameter sets to the FP64 path.
* The starting-root gap test: for the trigonometric roots t_k = 2 rt cos(th - 2 pi k / 3),
  th in [0, pi/3], the gaps are 2 sqrt3 rt sin(pi/3 - th) and 2 sqrt3 rt sin(th), and the
  spread 2 sqrt3 rt sin(th + pi/3), so gap < 5e-3 spread is th (or pi/3 - th) < ~4.33e-3.
"""
import numpy as np


def vacuum_system(t12, t13, dm21, dm31):
    c12, s12, c13, s13 = np.cos(t12), np.sin(t12), np.cos(t13), np.sin(t13)
    O = np.array([[c13 * c12, c13 * s12, s13], [-s12, c12, 0.0], [-s13 * c12, -s13 * s12, c13]])
    mu = np.array([0.0, dm21, dm31])
    return O, mu


def rank_one_vector(O, mu, lam):
    dl = mu - lam
    a = O[0]
    d = np.array([a[0] * dl[1] * dl[2], a[1] * dl[0] * dl[2], a[2] * dl[0] * dl[1]])
    return O @ d, d


def test_rank_one_eigenvectors_match_eigh():
    rng = np.random.default_rng(11)
    worst = 0.0
    for _ in range(2000):
        t12, t13 = rng.uniform(0.2, 1.3), rng.uniform(0.05, 0.3)
        dm21 = rng.uniform(5e-5, 1e-4)
        dm31 = rng.choice([-1, 1]) * rng.uniform(2e-3, 3e-3)
        V = rng.choice([-1, 1]) * 10 ** rng.uniform(-9, -1)  # vacuum-like up to the core at 100 GeV
        O, mu = vacuum_system(t12, t13, dm21, dm31)
        H = O @ np.diag(mu) @ O.T
        H[0, 0] += V
        w, U = np.linalg.eigh(H)
        for k in range(3):
            u, d = rank_one_vector(O, mu, w[k])
            assert abs(np.dot(u, u) - np.dot(d, d)) <= 1e-12 * np.dot(d, d)  # O orthogonal
            P = np.outer(u, u) / np.dot(u, u)
            worst = max(worst, np.abs(P - np.outer(U[:, k], U[:, k])).max())
    assert worst < 1e-8, worst


def test_rank_one_formula_vanishes_for_a_decoupled_state():
    """theta13 = 0: the third vacuum state has no electron component and stays an eigenvector
    at mu_2; there d -> 0 (relative to spread^2) and the kernels take the FP64 path, while the
    other two eigenvalues keep a well-conditioned formula."""
    O, mu = vacuum_system(0.5843, 0.0, 7.53e-5, 2.5e-3)
    H = O @ np.diag(mu) @ O.T
    H[0, 0] += 3e-4
    w, U = np.linalg.eigh(H)
    spread = w.max() - w.min()
    norms = [np.dot(*(2 * [rank_one_vector(O, mu, x)[1]])) / spread ** 4 for x in w]
    k = int(np.argmin(np.abs(w - mu[2])))
    assert norms[k] < 1e-16
    assert all(n > 1e-12 for i, n in enumerate(norms) if i != k)


def test_start_gap_identities_and_angle_threshold():
    rng = np.random.default_rng(12)
    for _ in range(5000):
        rt = 10 ** rng.uniform(-4, -1)
        th = rng.uniform(0.0, np.pi / 3)
        t = [2 * rt * np.cos(th - 2 * np.pi * k / 3) for k in range(3)]
        l0, l1, l2 = t[0], t[1], t[2]
        assert l0 >= l1 >= l2
        s3 = np.sqrt(3.0)
        assert np.isclose(l0 - l1, 2 * s3 * rt * np.sin(np.pi / 3 - th), rtol=1e-9, atol=1e-15 * rt)
        assert np.isclose(l1 - l2, 2 * s3 * rt * np.sin(th), rtol=1e-9, atol=1e-15 * rt)
        assert np.isclose(l0 - l2, 2 * s3 * rt * np.sin(th + np.pi / 3), rtol=1e-9)
        ratio = min(l0 - l1, l1 - l2) / (l0 - l2)
        near = not (4.33e-3 < th < np.pi / 3 - 4.33e-3)
        # the angle test and the gap test agree away from the 5e-3 boundary itself
        if ratio < 4.9e-3:
            assert near
        if ratio > 5.1e-3:
            assert not near
