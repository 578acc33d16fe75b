"""Seeded synthetic surveys and prior caches.

These stand in for survey data and for the reference's prior-cache files
(``JokerPrior.sample`` written to HDF5, thejoker/prior.py:297-407).  The prior
cache follows the default prior: P log-uniform, e ~ Beta(0.867, 3.03), omega
and M0 ~ U[0, 2 pi), and s either 0 or log-normal.
"""
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from .linear import rv_unit_columns

__all__ = ["fill_prior_cache", "survey_stars", "default_prior_arrays"]


def fill_prior_cache(out, seed, P_min=2.0, P_max=1024.0, jitter=None, threads=16):
    """Fill ``out`` (n x 5 float64: P, e, omega, M0, s) with prior samples,
    drawn in parallel blocks from independent numpy generators.  ``jitter`` is
    None (s = 0) or (mu, sigma) of ln s."""
    n = out.shape[0]
    nblk = max(1, min(threads * 4, n // 65536))
    bounds = np.linspace(0, n, nblk + 1).astype(np.int64)
    seqs = np.random.SeedSequence(seed).spawn(nblk)

    def work(i):
        a, b = bounds[i], bounds[i + 1]
        r = np.random.default_rng(seqs[i])
        m = b - a
        out[a:b, 0] = np.exp(r.uniform(np.log(P_min), np.log(P_max), m))
        out[a:b, 1] = r.beta(0.867, 3.03, m)
        out[a:b, 2] = r.uniform(0, 2 * np.pi, m)
        out[a:b, 3] = r.uniform(0, 2 * np.pi, m)
        out[a:b, 4] = 0.0 if jitter is None else np.exp(r.normal(jitter[0], jitter[1], m))

    with ThreadPoolExecutor(threads) as ex:
        list(ex.map(work, range(nblk)))
    return out


def default_prior_arrays(poly_trend=1, sigma_v=(100.0, 1.0, 0.01), sigma_K0=30.0, P0=365.25,
                         max_K=500.0):
    """mu, lam, k_prior of the default prior (FixedCompanionMass K prior,
    Normal trend terms) in the CJokerHelper index order."""
    L = 1 + poly_trend
    mu = np.zeros(L)
    lam = np.zeros(L)
    for j in range(poly_trend):
        lam[1 + j] = sigma_v[j] ** 2
    return mu, lam, np.array([1.0, sigma_K0, P0, max_K])


def survey_stars(n_stars, seed, n_min=3, n_max=256, base=(100.0, 4000.0), sig=(0.1, 1.0),
                 companion_frac=0.3, K_range=(1.0, 50.0), poly_trend=1,
                 sigma_v=(100.0, 1.0, 0.01), t0=2456000.0):
    """Stars with log-uniform epoch counts in [n_min, n_max], baselines
    uniform in ``base`` days, errors uniform in ``sig``; a fraction
    ``companion_frac`` carries a Keplerian companion drawn from the prior with
    K ~ U(K_range), the others are constant (plus a polynomial trend when
    poly_trend > 1).  Returns the list of StarTable dicts."""
    rng = np.random.default_rng(seed)
    mu, lam, kp = default_prior_arrays(poly_trend, sigma_v)
    stars = []
    for _ in range(n_stars):
        N = int(np.clip(np.round(np.exp(rng.uniform(np.log(n_min), np.log(n_max)))), n_min, n_max))
        t = np.sort(t0 + rng.uniform(0, rng.uniform(*base), N))
        err = rng.uniform(*sig, N)
        rv = rng.normal(0, 30.0) + rng.normal(0, err)
        if rng.uniform() < companion_frac:
            P = np.exp(rng.uniform(np.log(2.0), np.log(1024.0)))
            e = rng.beta(0.867, 3.03)
            om, M0 = rng.uniform(0, 2 * np.pi, 2)
            K = rng.uniform(*K_range)
            rv = rv + K * rv_unit_columns(t, t.min(), [P], [e], [om], [M0])[0]
        dt = t - t.min()
        for j in range(1, poly_trend):
            rv = rv + rng.normal(0, sigma_v[j] * 0.1) * dt ** j
        trend = np.vander(dt, N=poly_trend, increasing=True)
        stars.append(dict(t=t, rv=rv, ivar=1 / err ** 2, t_ref=t.min(), trend_M=trend,
                          mu=mu.copy(), lam=lam.copy(), k_prior=kp.copy()))
    return stars
