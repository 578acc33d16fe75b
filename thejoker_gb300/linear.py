"""Linear-parameter posterior for accepted samples (host, FP64).

Restates CJokerHelper.batch_get_posterior_samples
(thejoker/src/fast_likelihood.pyx:471-545): for each nonlinear sample,
a = (Lambda^-1 + M C^-1 M^T)^-1 (M C^-1 y + Lambda^-1 mu) and
A = (Lambda^-1 + M C^-1 M^T)^-1, then
rng.multivariate_normal(a, A, size=n_linear_samples_per), drawn from the
caller's generator in the same order as the reference so that the draws match.
As in the reference, the jitter is not applied here (:516 computes it, nothing
reads it) and the FixedCompanionMass variance is not clipped at max_K
(:519-521).  This runs only on the accepted samples; it is not the hot path.
"""
import numpy as np

__all__ = ["rv_unit_columns", "posterior_linear_samples"]


def _kepler_E(M, e):
    """Eccentric anomaly, Markley (1995) starter + fifth-order correction, FP64."""
    M = np.mod(M, 2 * np.pi)
    M = np.where(M > np.pi, M - 2 * np.pi, M)
    sgn = np.where(M < 0, -1.0, 1.0)
    x = np.abs(M)
    pi = np.pi
    alpha = (3 * pi * pi + 1.6 * pi * (pi - x) / (1 + e)) / (pi * pi - 6)
    d = 3 * (1 - e) + alpha * e
    q = 2 * alpha * d * (1 - e) - x * x
    r = 3 * alpha * d * (d - 1 + e) * x + x ** 3
    w = np.cbrt(np.abs(r) + np.sqrt(q ** 3 + r * r)) ** 2
    E1 = (2 * r * w / (w * w + w * q + q * q) + x) / d
    s1, c1 = np.sin(E1), np.cos(E1)
    f0 = E1 - e * s1 - x
    f1 = 1 - e * c1
    f2 = e * s1
    f3 = 1 - f1
    f4 = -f2
    d3 = -f0 / (f1 - 0.5 * f0 * f2 / f1)
    d4 = -f0 / (f1 + 0.5 * d3 * f2 + d3 * d3 * f3 / 6)
    d5 = -f0 / (f1 + 0.5 * d4 * f2 + d4 * d4 * f3 / 6 + d4 ** 3 * f4 / 24)
    return sgn * (E1 + d5)


def rv_unit_columns(t, t_ref, P, e, omega, M0):
    """Unit-K RV column cos(omega + f) + e cos(omega), shape (n_samples, n_times)."""
    P, e, omega, M0 = (np.asarray(v, dtype=np.float64)[:, None] for v in (P, e, omega, M0))
    M = 2 * np.pi * (np.asarray(t)[None, :] - t_ref) / P - M0
    E = _kepler_E(M, e)
    f = 2 * np.arctan2(np.sqrt(1 + e) * np.sin(E / 2), np.sqrt(1 - e) * np.cos(E / 2))
    return np.cos(omega + f) + e * np.cos(omega)


def posterior_linear_samples(chunk, n_per, rng, t, rv, ivar, t_ref, trend_M, mu, lam, k_prior):
    """Reference-order posterior draws; returns (samples (S*n, 5+L), a, A)."""
    chunk = np.asarray(chunk, dtype=np.float64)
    S = chunk.shape[0]
    L = len(mu)
    cols = rv_unit_columns(t, t_ref, chunk[:, 0], chunk[:, 1], chunk[:, 2], chunk[:, 3])
    out = np.zeros((S, n_per, 5 + L))
    a_all = np.zeros((S, L))
    A_all = np.zeros((S, L, L))
    lam = np.array(lam, dtype=np.float64)
    for n in range(S):
        P, e = chunk[n, 0], chunk[n, 1]
        if k_prior[0]:
            lam[0] = k_prior[1] ** 2 / (1 - e ** 2) * (P / k_prior[2]) ** (-2 / 3)
        M = np.vstack([cols[n][None, :], np.asarray(trend_M).T]) if L > 1 else cols[n][None, :]
        Ainv = np.diag(1.0 / lam) + (M * ivar) @ M.T
        rhs = (M * ivar) @ rv + mu / lam
        a = np.linalg.solve(Ainv, rhs)
        A = np.linalg.inv(Ainv)
        draws = rng.multivariate_normal(a, A, size=n_per)
        out[n, :, :5] = chunk[n]
        out[n, :, 5:] = draws
        a_all[n], A_all[n] = a, A
    return out.reshape(S * n_per, 5 + L), a_all, A_all
