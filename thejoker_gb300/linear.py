"""Host helpers around the linear parameters.

* ``rv_unit_columns``: the unit-K Kepler RV column in NumPy FP64 (Markley's
  solver), for building synthetic data sets.
* ``multivariate_normal_draws``: the draws of
  CJokerHelper.batch_get_posterior_samples (thejoker/src/fast_likelihood.pyx
  :529-530), rng.multivariate_normal(a, A, size=n) for each accepted sample in
  turn, batched over the samples.  They stay on the host so that they come
  from the caller's numpy generator in the reference's order; the means and
  covariances come from the device (joker_linear_posterior).
"""
import numpy as np

__all__ = ["rv_unit_columns", "multivariate_normal_draws"]


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


def multivariate_normal_draws(rng, a, A, n_per):
    """rng.multivariate_normal(a[i], A[i], size=n_per) for every i in turn,
    batched: the same standard normals in the same order (one block of
    n_per * L per sample) and numpy's default SVD factor of each covariance,
    x = z @ (sqrt(s)[:, None] * vh) + a.  Returns (S, n_per, L)."""
    a = np.asarray(a, dtype=np.float64)
    A = np.asarray(A, dtype=np.float64)
    S, L = a.shape
    z = rng.standard_normal((S, n_per, L))
    if S == 0:
        return z
    _, sv, vh = np.linalg.svd(A)
    factor = np.sqrt(sv)[:, :, None] * vh
    return np.matmul(z, factor) + a[:, None, :]
