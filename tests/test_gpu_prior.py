"""Prior samples drawn on the device (GB300 only): Philox4x32-10 streams
checked bit for bit against a plain statement of the algorithm, the
marginals against their distributions (Kolmogorov-Smirnov), independence
from the launch split, and agreement of the prepared cache with a cache
loaded from the same packed samples."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

_M0, _M1, _W0, _W1 = 0xD2511F53, 0xCD9E8D57, 0x9E3779B9, 0xBB67AE85
_TAG = 0x4A6F6B72


def _philox(ctr, key):
    c, k = list(ctr), list(key)
    for _ in range(10):
        p0, p1 = _M0 * c[0], _M1 * c[2]
        c = [(p1 >> 32) ^ c[1] ^ k[0], p1 & 0xFFFFFFFF, (p0 >> 32) ^ c[3] ^ k[1], p0 & 0xFFFFFFFF]
        k = [(k[0] + _W0) & 0xFFFFFFFF, (k[1] + _W1) & 0xFFFFFFFF]
    return c


def _uniforms(seed, g, block):
    c = _philox([g & 0xFFFFFFFF, g >> 32, block, _TAG], [seed & 0xFFFFFFFF, seed >> 32])
    x0, x1 = (c[1] << 32) | c[0], (c[3] << 32) | c[2]
    return (x0 >> 11) * 2.0 ** -53, (x1 >> 11) * 2.0 ** -53


def test_philox_known_answer():
    # Random123's published vector for zero counter and key
    assert _philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]


def _spec(s_kind="lognormal"):
    from thejoker_gb300 import _native as nat
    d = dict(P_min=2.0, P_max=1024.0, e_alpha=0.867, e_beta=3.03)
    if s_kind == "lognormal":
        d.update(s_kind=nat.JOKER_S_LOGNORMAL, s_mu=np.log(0.5), s_sigma=1.0)
    else:
        d.update(s_kind=nat.JOKER_S_FIXED, s_value=0.0)
    return d


def test_streams_and_distributions(cuda):
    from scipy import stats
    from thejoker_gb300 import device as dev
    n, seed = 1 << 20, 0x1234_5678_9ABC
    cache = dev.PriorCache(n)
    packed = torch.empty((n, 5), dtype=torch.float64, device="cuda")
    cache.sample_prior(_spec(), n, seed=seed, first_index=1000, packed=packed)
    x = packed.cpu().numpy()
    # angles bit for bit from the Philox statement (u_P, u_omega | u_M0, ...)
    for i in (0, 1, 77, 4095, n - 1):
        g = 1000 + i
        u_p, u_om = _uniforms(seed, g, 0)
        u_m0, _ = _uniforms(seed, g, 1)
        assert x[i, 2] == u_om * (2 * np.pi)
        assert x[i, 3] == u_m0 * (2 * np.pi)
        np.testing.assert_allclose(x[i, 0], np.exp(np.log(2.0) + u_p * np.log(512.0)),
                                   rtol=1e-14)
    # marginals
    lp = (np.log(x[:, 0]) - np.log(2.0)) / np.log(512.0)
    for col, cdf in ((lp, stats.uniform.cdf), (x[:, 2] / (2 * np.pi), stats.uniform.cdf),
                     (x[:, 3] / (2 * np.pi), stats.uniform.cdf),
                     (x[:, 1], stats.beta(0.867, 3.03).cdf),
                     (x[:, 4], stats.lognorm(s=1.0, scale=0.5).cdf)):
        assert stats.kstest(col, cdf).pvalue > 1e-4
    assert np.all((x[:, 1] >= 0) & (x[:, 1] < 1)) and np.all(x[:, 4] > 0)


def test_split_independent_and_cache_consistent(cuda):
    from thejoker_gb300 import device as dev
    from gpu_util import synth_star
    n, seed = 300_000, 42
    whole = dev.PriorCache(n)
    pw = torch.empty((n, 5), dtype=torch.float64, device="cuda")
    whole.sample_prior(_spec("fixed"), n, seed=seed, packed=pw)
    parts = dev.PriorCache(n)
    pa = torch.empty((100_000, 5), dtype=torch.float64, device="cuda")
    pb = torch.empty((n - 100_000, 5), dtype=torch.float64, device="cuda")
    parts.sample_prior(_spec("fixed"), 100_000, seed=seed, row0=0, first_index=0, packed=pa)
    parts.sample_prior(_spec("fixed"), n - 100_000, seed=seed, row0=100_000,
                       first_index=100_000, packed=pb)
    torch.testing.assert_close(torch.cat([pa, pb]), pw, rtol=0, atol=0)
    # the sampled cache gives the same ln L as a cache loaded from its samples
    star = synth_star(np.random.default_rng(3), 21)
    table = dev.StarTable([star])
    loaded = dev.PriorCache.from_samples(pw)
    outs = []
    for c in (whole, parts, loaded):
        for prec in ("mixed", "fp64"):
            o = torch.empty((1, n), dtype=torch.float64, device="cuda")
            dev.lnl(table, c, o, precision=prec)
            outs.append(o.cpu().numpy())
    np.testing.assert_array_equal(outs[0], outs[2])
    np.testing.assert_array_equal(outs[0], outs[4])
    np.testing.assert_array_equal(outs[1], outs[3])
    np.testing.assert_array_equal(outs[1], outs[5])


def test_prior_sample_errors(cuda):
    from thejoker_gb300 import JokerPrior, device as dev
    from thejoker_gb300._native import JokerError
    c = dev.PriorCache(1000)
    bad = _spec()
    bad["P_min"] = -1.0
    with pytest.raises(JokerError):
        c.sample_prior(bad, 10)
    with pytest.raises(JokerError):
        c.sample_prior(_spec(), 2000)                       # beyond the capacity
    view = dev.PriorCache.view(torch.zeros((10, 5), dtype=torch.float64, device="cuda"))
    with pytest.raises(JokerError):
        view.sample_prior(_spec(), 10)
    prior = JokerPrior.default(P_min=2, P_max=1024, sigma_K0=30.0, sigma_v=100.0)
    c.sample_prior(prior, 1000, seed=1)                     # from a JokerPrior
