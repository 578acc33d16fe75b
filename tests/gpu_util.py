"""Helpers shared by the GPU tests."""
import numpy as np


def star_from_fixture(z):
    return dict(t=z["t"], rv=z["rv"], ivar=z["ivar"], t_ref=float(z["t_ref"]),
                trend_M=z["trend_M"], mu=z["mu"], lam=z["lam"], k_prior=z["k_prior"])


def synth_star(rng, N, base=1000.0, sig=(0.1, 1.0), poly=1, noff=0, K=None, t0=2456000.0,
               sigma_K0=30.0, sigma_v=(100.0, 1.0, 0.01)):
    from thejoker_gb300.linear import rv_unit_columns
    t = np.sort(rng.uniform(0, base, N)) + t0
    err = rng.uniform(*sig, N)
    if K is None:
        K = rng.uniform(1, 50)
    P, e = np.exp(rng.uniform(np.log(2), np.log(1024))), rng.beta(0.867, 3.03)
    om, M0 = rng.uniform(0, 2 * np.pi), rng.uniform(0, 2 * np.pi)
    rv = K * rv_unit_columns(t, t.min(), [P], [e], [om], [M0])[0] + rng.normal(0, 10) \
        + rng.normal(0, err)
    ids = np.zeros(N, dtype=int)
    if noff:
        ids[rng.permutation(N)[: N // 2]] = 1
    const = np.zeros((N, 1 + noff))
    const[:, 0] = 1.0
    for j in range(noff):
        const[ids == j + 1, j + 1] = 1.0
    dt = t - t.min()
    trend = np.hstack([const, np.vander(dt, N=poly, increasing=True)[:, 1:]])
    L = 1 + poly + noff
    lam = np.zeros(L)
    lam[1] = sigma_v[0] ** 2
    for j in range(noff):
        lam[2 + j] = 4.0
    for j in range(1, poly):
        lam[1 + noff + j] = sigma_v[j] ** 2
    return dict(t=t, rv=rv, ivar=1 / err ** 2, t_ref=t.min(), trend_M=trend, mu=np.zeros(L),
                lam=lam, k_prior=np.array([1.0, sigma_K0, 365.25, 500.0]))


def synth_chunk(rng, S, P_min=2.0, P_max=1024.0, jitter=False):
    P = np.exp(rng.uniform(np.log(P_min), np.log(P_max), S))
    e = rng.beta(0.867, 3.03, S)
    om = rng.uniform(0, 2 * np.pi, S)
    M0 = rng.uniform(0, 2 * np.pi, S)
    s = np.exp(rng.normal(np.log(0.5), 1.0, S)) if jitter else np.zeros(S)
    return np.ascontiguousarray(np.stack([P, e, om, M0, s], 1))


def oracle_lnl(star, chunk, jitter=False):
    from oracle import oracle
    return oracle.batch_marginal_ln_likelihood(
        star["t"], star["rv"], star["ivar"], star["t_ref"], star["trend_M"], star["mu"],
        star["lam"], chunk, bool(star["k_prior"][0]), *star["k_prior"][1:], jitter=jitter)


def rel_err(a, b):
    return np.abs(a - b) / np.maximum(1.0, np.abs(b))
