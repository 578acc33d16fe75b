"""After acceptance (GB300 only): the device posterior of the linear
parameters (joker_linear_posterior) behind
GPUJokerHelper.batch_get_posterior_samples reproduces the reference's
batch_get_posterior_samples (fast_likelihood.pyx:471-545) as restated by the
oracle -- same draws from the same generator -- and the device unmarginalized
likelihood matches JokerSamples.ln_unmarginalized_likelihood
(samples.py:611-632) restated in NumPy."""
import numpy as np
import pytest
import torch

from gpu_util import synth_chunk, synth_star

pytestmark = pytest.mark.gpu


def _direct_posterior(star, row, s=0.0, clip=False):
    """a and A of one sample (NumPy FP64) and its ln L from the N x N
    Gaussian in 40-digit arithmetic."""
    from thejoker_gb300.linear import rv_unit_columns
    P, e, om, M0 = row[:4]
    m = rv_unit_columns(star["t"], star["t_ref"], [P], [e], [om], [M0])[0]
    M = np.vstack([m[None, :], np.asarray(star["trend_M"]).T])
    lam = np.array(star["lam"], dtype=np.float64)
    kp = star["k_prior"]
    if kp[0]:
        lam[0] = kp[1] ** 2 / (1 - e ** 2) * (P / kp[2]) ** (-2 / 3)
        if clip:
            lam[0] = min(lam[0], kp[3] ** 2)
    w = 1.0 / (1.0 / star["ivar"] + s * s)
    Ainv = np.diag(1 / lam) + (M * w) @ M.T
    A = np.linalg.inv(Ainv)
    a = A @ ((M * w) @ star["rv"] + star["mu"] / lam)
    # ln N(y | M^T mu, W^-1 + M^T Lambda M) in 40-digit arithmetic: with a
    # quadratic trend this N x N system is too ill-conditioned for FP64
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    N = len(w)
    Mm = [[mp.mpf(float(x)) for x in row_] for row_ in M]
    B = mp.matrix(N, N)
    for i in range(N):
        for j in range(N):
            v = mp.fsum(Mm[k][i] * mp.mpf(float(lam[k])) * Mm[k][j] for k in range(len(Mm)))
            B[i, j] = v + (1 / mp.mpf(float(w[i])) if i == j else 0)
    r = mp.matrix([mp.mpf(float(v)) for v in star["rv"] - M.T @ star["mu"]])
    ll = float(-0.5 * ((r.T * mp.lu_solve(B, r))[0] + mp.log(mp.det(2 * mp.pi * B))))
    return a, A, ll


@pytest.mark.parametrize("poly,jitter", [(1, "reference"), (3, "reference"), (2, "applied")])
def test_linear_posterior_against_direct(cuda, poly, jitter):
    from thejoker_gb300 import device as dev
    rng = np.random.default_rng(31)
    star = synth_star(rng, 23, poly=poly)
    chunk = synth_chunk(rng, 64, jitter=(jitter == "applied"))
    chunk[0] = [0.05, 0.9995, 1.0, 2.0, 0.3]        # scaled K variance above max_K^2
    table = dev.StarTable([star], jitter=jitter)
    cache = dev.PriorCache.from_samples(chunk)
    rows = torch.tensor([0, 5, 17, 63, 5], dtype=torch.int64)
    for clip in (False, True):
        a, A, ll = (x.cpu().numpy() for x in dev.linear_posterior(table, cache, 0, rows,
                                                                  k_clip=clip))
        expect = {}
        for i, r in enumerate(rows.tolist()):
            s = chunk[r, 4] if jitter == "applied" else 0.0
            if r not in expect:
                expect[r] = _direct_posterior(star, chunk[r], s=s, clip=clip)
            ea, eA, ell = expect[r]
            np.testing.assert_allclose(a[i], ea, rtol=1e-8, atol=1e-8 * np.abs(ea).max())
            np.testing.assert_allclose(A[i], eA, rtol=1e-8, atol=1e-10 * np.abs(eA).max())
            assert abs(ll[i] - ell) <= 1e-9 * max(1.0, abs(ell))


def test_batch_get_posterior_samples_matches_reference_order(cuda):
    from oracle.oracle import posterior_linear_samples
    from thejoker_gb300 import JokerPrior, RVData
    from thejoker_gb300.data import get_trend_design_matrix
    from thejoker_gb300.helper import GPUJokerHelper
    rng = np.random.default_rng(5)
    st = synth_star(rng, 19, K=8.0, poly=2)
    prior = JokerPrior.default(P_min=2, P_max=1024, sigma_K0=30.0, sigma_v=[100.0, 1.0],
                               poly_trend=2)
    data = RVData(st["t"], st["rv"], 1 / np.sqrt(st["ivar"]))
    trend = get_trend_design_matrix(data, None, prior.poly_trend)
    helper = GPUJokerHelper(data, prior, trend)
    chunk = prior.sample(40, rng=np.random.default_rng(9)).pack()[0]
    r1, r2 = np.random.default_rng(77), np.random.default_rng(77)
    samples, ll = helper.batch_get_posterior_samples(chunk, 6, r1)
    mu, lam, kp = prior.linear_prior_arrays()
    ref, _, _ = posterior_linear_samples(chunk, 6, r2, data._t_bmjd, data.rv, data.ivar,
                                         data._t_ref_bmjd, trend, mu, lam, kp)
    assert samples.shape == ref.shape == (240, 5 + prior.n_linear)
    np.testing.assert_array_equal(samples[:, :5], ref[:, :5])
    np.testing.assert_allclose(samples[:, 5:], ref[:, 5:], rtol=1e-8, atol=1e-8)
    assert r1.bit_generator.state == r2.bit_generator.state
    assert ll.shape == (240,) and np.all(np.isfinite(ll))
    np.testing.assert_array_equal(ll[::6], ll[5::6])


@pytest.mark.parametrize("poly", [1, 3])
def test_ln_unmarginalized_likelihood(cuda, poly):
    from thejoker_gb300 import RVData
    from thejoker_gb300.linear import rv_unit_columns
    from thejoker_gb300.samples import JokerSamples
    rng = np.random.default_rng(12)
    st = synth_star(rng, 31, poly=1)
    data = RVData(st["t"], st["rv"], 1 / np.sqrt(st["ivar"]))
    n = 500
    chunk = synth_chunk(rng, n, jitter=True)
    cols = dict(P=chunk[:, 0], e=chunk[:, 1], omega=chunk[:, 2], M0=chunk[:, 3], s=chunk[:, 4],
                K=rng.normal(0, 20, n))
    for j in range(poly):
        cols[f"v{j}"] = rng.normal(0, 10.0 ** -j, n)
    t_ref = data._t_ref_bmjd + 3.25                    # samples with their own t_ref
    smp = JokerSamples(cols, t_ref=t_ref, poly_trend=poly)
    got = smp.ln_unmarginalized_likelihood(data)
    m = rv_unit_columns(data._t_bmjd, t_ref, chunk[:, 0], chunk[:, 1], chunk[:, 2], chunk[:, 3])
    dt = data._t_bmjd - t_ref
    model = cols["K"][:, None] * m + sum(cols[f"v{j}"][:, None] * dt[None, :] ** j
                                         for j in range(poly))
    var = 1 / data.ivar[None, :] + chunk[:, 4:5] ** 2
    expect = (-0.5 * (np.log(2 * np.pi * var) + (model - data.rv[None, :]) ** 2 / var)).sum(1)
    np.testing.assert_allclose(got, expect, rtol=1e-10, atol=1e-8)
