"""Python entry points of the CPU oracle (test infrastructure only).

* ``batch_marginal_ln_likelihood``: ctypes call into the plain-C restatement
  (joker_oracle.c) of CJokerHelper.batch_marginal_ln_likelihood
  (thejoker/src/fast_likelihood.pyx:428-469).
* ``py_marginal_ln_likelihood``: a NumPy restatement of the reference's test
  oracle thejoker/src/tests/py_likelihood.py:32-107 and :134-205 (jitter
  applied, slogdet in place of astroML's log_multivariate_gaussian).
* ``accept_mask``: the acceptance rule of likelihood_helpers.py:107-109 /
  multiproc_helpers.py:256-258, ``exp(lls - lls.max()) > uu``.
* ``rv_unit``: the unit-K Kepler RV column (kepler.c).
* ``posterior_linear_samples``: batch_get_posterior_samples restated in NumPy.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_LIB = None
_dp = ctypes.POINTER(ctypes.c_double)


def _lib():
    global _LIB
    if _LIB is None:
        so = _build.build_oracle()
        lib = ctypes.CDLL(so)
        lib.oracle_batch_marginal_ln_likelihood.restype = ctypes.c_int
        lib.oracle_batch_marginal_ln_likelihood.argtypes = [
            ctypes.c_int, ctypes.c_int, ctypes.c_double, _dp, _dp, _dp, _dp, _dp, _dp,
            ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
            ctypes.c_int, _dp, ctypes.c_long, _dp]
        lib.oracle_rv_unit_batch.restype = None
        lib.oracle_rv_unit_batch.argtypes = [ctypes.c_int, ctypes.c_double, _dp, _dp,
                                             ctypes.c_long, _dp]
        lib.oracle_eccentric_anomaly.restype = ctypes.c_double
        lib.oracle_eccentric_anomaly.argtypes = [ctypes.c_double, ctypes.c_double]
        _LIB = lib
    return _LIB


def _ptr(a):
    return a.ctypes.data_as(_dp)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def batch_marginal_ln_likelihood(t, rv, ivar, t_ref, trend_M, mu, Lambda, chunk,
                                 k_prior_scaled=False, sigma_K0=0.0, P0=365.25,
                                 max_K=500.0, jitter=False):
    """FP64 ln L per row of ``chunk`` (S x 5: P, e, omega, M0, s), reference algorithm.

    ``trend_M`` is N x (L-1); ``mu`` / ``Lambda`` have L entries in
    CJokerHelper's order (K, v0, offsets..., v1, ...).  ``Lambda[0]`` is
    replaced per sample when ``k_prior_scaled``.
    """
    t, rv, ivar = _f64(t), _f64(rv), _f64(ivar)
    trend_M = _f64(trend_M)
    mu, Lambda, chunk = _f64(mu), _f64(Lambda), _f64(chunk)
    N = t.shape[0]
    L = Lambda.shape[0]
    assert trend_M.shape == (N, L - 1) and mu.shape == (L,)
    assert chunk.ndim == 2 and chunk.shape[1] == 5
    out = np.full(chunk.shape[0], np.nan)
    if L - 1 == 0:
        trend_M = np.zeros((N, 1))
    rc = _lib().oracle_batch_marginal_ln_likelihood(
        N, L, float(t_ref), _ptr(t), _ptr(rv), _ptr(ivar), _ptr(trend_M), _ptr(mu),
        _ptr(Lambda), int(bool(k_prior_scaled)), float(sigma_K0), float(P0),
        float(max_K), int(bool(jitter)), _ptr(chunk), chunk.shape[0], _ptr(out))
    if rc != 0:
        raise MemoryError("oracle allocation failed")
    return out


def rv_unit(t, t_ref, chunk):
    """Unit-K RV column, shape (S, N)."""
    t, chunk = _f64(t), _f64(chunk)
    out = np.empty((chunk.shape[0], t.shape[0]))
    _lib().oracle_rv_unit_batch(t.shape[0], float(t_ref), _ptr(t), _ptr(chunk),
                                chunk.shape[0], _ptr(out))
    return out


def eccentric_anomaly(M, e):
    return _lib().oracle_eccentric_anomaly(float(M), float(e))


def py_marginal_ln_likelihood(t, rv, ivar, t_ref, chunk, poly_trend, Lambda_lin,
                              k_prior_scaled=False, sigma_K0=0.0, P0=365.25,
                              max_K=500.0):
    """NumPy restatement of py_likelihood.marginal_ln_likelihood (jitter applied).

    Follows py_likelihood.py:110-131 (design matrix [rv_unit, vander(t - t_ref,
    poly_trend)]), :134-172 (Lambda, max_K clip, ivar / (1 + s^2 ivar)), and
    :32-107 (B = C + M Lambda M^T, Binv by Woodbury, Gaussian log density with
    zero prior mean).  ``Lambda_lin`` holds the L variances (K first; ignored
    for K when ``k_prior_scaled``).
    """
    t, rv, ivar = _f64(t), _f64(rv), _f64(ivar)
    chunk = _f64(chunk)
    N = t.shape[0]
    cols = rv_unit(t, t_ref, chunk)
    V = np.vander(t - t_ref, N=poly_trend, increasing=True)
    out = np.empty(chunk.shape[0])
    for n in range(chunk.shape[0]):
        P, e, _, _, s = chunk[n]
        Lam = np.array(Lambda_lin, dtype=np.float64)
        if k_prior_scaled:
            Lam[0] = min(max_K ** 2, sigma_K0 ** 2 / (1 - e ** 2) * (P / P0) ** (-2 / 3))
        iv = ivar / (1 + s ** 2 * ivar)
        M = np.hstack((cols[n][:, None], V))
        Cinv = np.diag(iv)
        B = np.diag(1.0 / iv) + M @ np.diag(Lam) @ M.T
        Ainv = np.diag(1.0 / Lam) + M.T @ Cinv @ M
        A = np.linalg.inv(Ainv)
        Binv = Cinv - Cinv @ M @ A @ M.T @ Cinv
        sign, logdet = np.linalg.slogdet(B)
        r = rv
        out[n] = -0.5 * (N * np.log(2 * np.pi) + logdet + r @ Binv @ r)
    return out


def accept_mask(lls, uu):
    """``np.exp(lls - lls.max()) > uu`` exactly as the reference evaluates it."""
    lls = np.asarray(lls, dtype=np.float64)
    return np.exp(lls - lls.max()) > uu


def posterior_linear_samples(chunk, n_per, rng, t, rv, ivar, t_ref, trend_M, mu, lam, k_prior):
    """CJokerHelper.batch_get_posterior_samples (fast_likelihood.pyx:471-545)
    restated: per sample a = Ainv^-1 (M C^-1 y + Lambda^-1 mu), A = Ainv^-1 with
    Ainv = Lambda^-1 + M C^-1 M^T, then rng.multivariate_normal(a, A, size=n_per)
    in the reference's order.  No jitter and no max_K clip, as there (:516,
    :519-521).  Returns (samples (S*n, 5+L), a, A)."""
    chunk = np.asarray(chunk, dtype=np.float64)
    S = chunk.shape[0]
    L = len(mu)
    cols = rv_unit(t, t_ref, chunk)
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
