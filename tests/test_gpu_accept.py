"""GPU acceptance pass and the sampler API against the reference's rules
(likelihood_helpers.py:91-229) restated with NumPy (GB300 only)."""
import numpy as np
import pytest
import torch

from gpu_util import oracle_lnl, synth_chunk, synth_star

pytestmark = pytest.mark.gpu


def _keys_for(values):
    from thejoker_gb300 import device as dev
    import struct
    mk = dev.MaxKeys(len(values))
    keys = []
    for m in values:
        b = struct.unpack("<q", struct.pack("<d", m))[0]
        k = (~b) & 0xFFFFFFFFFFFFFFFF if b < 0 else (b | (1 << 63))
        keys.append(np.array(k, dtype=np.uint64).view(np.int64))
    mk.t.copy_(torch.tensor(np.array(keys, dtype=np.int64)))
    return mk


@pytest.mark.parametrize("n", [1, 31, 32, 1000, 8192, 8193, 100000])
def test_pcg64_stream_matches_numpy_uniform(cuda, n):
    """With lnl = log(x) and max 0 the pass keeps exactly x > u: the device
    regenerates rng.uniform(size=n) bit for bit."""
    from thejoker_gb300 import device as dev
    rng = np.random.default_rng(1234 + n)
    x = rng.uniform(size=n)
    lnl = np.log(x)
    lnl[0] = 0.0
    gen = np.random.default_rng(99)
    gen.uniform(size=17)                       # arbitrary position in the stream
    st, inc = dev.pcg64_state(gen)
    uu = np.random.Generator(np.random.PCG64())
    uu.bit_generator.state = gen.bit_generator.state
    expect = np.where(np.exp(lnl - lnl.max()) > uu.uniform(size=n))[0]
    d = torch.from_numpy(lnl).cuda()
    idx, out_lnl, counts = dev.accept(d, _keys_for([0.0]), [dict(
        lnl_off=0, n=n, out_off=0, max_out=n, max_slot=0, pcg=(st, inc, 0))],
        out_lnl=torch.empty(n, dtype=torch.float64, device="cuda"))
    c = int(counts[0])
    assert c == len(expect)
    np.testing.assert_array_equal(idx[:c].cpu().numpy(), expect)
    np.testing.assert_array_equal(out_lnl[:c].cpu().numpy(), lnl[expect])


def test_array_source_truncation_and_segments(cuda):
    from thejoker_gb300 import device as dev
    rng = np.random.default_rng(5)
    lnl = np.concatenate([rng.normal(0, 3, 20000), rng.normal(-2, 1, 9000)])
    u = rng.uniform(size=lnl.size)
    segs = [dict(lnl_off=0, n=20000, idx_base=0, out_off=0, max_out=50, max_slot=0, u_off=0),
            dict(lnl_off=20000, n=9000, idx_base=100, out_off=50, max_out=10000, max_slot=1,
                 u_off=20000)]
    m0, m1 = lnl[:20000].max(), lnl[20000:].max()
    idx, _, counts = dev.accept(torch.from_numpy(lnl).cuda(), _keys_for([m0, m1]), segs,
                                u_source="array", u=torch.from_numpy(u).cuda())
    idx = idx.cpu().numpy()
    e0 = np.where(np.exp(lnl[:20000] - m0) > u[:20000])[0]
    e1 = np.where(np.exp(lnl[20000:] - m1) > u[20000:])[0]
    assert int(counts[0]) == len(e0) and int(counts[1]) == len(e1)
    np.testing.assert_array_equal(idx[:min(50, len(e0))], e0[:50])
    np.testing.assert_array_equal(idx[50:50 + len(e1)], e1 + 100)


def test_accept_extremes(cuda):
    """u == 0 accepts anything above exp underflow; NaN max keeps nothing."""
    from thejoker_gb300 import device as dev
    lnl = np.array([0.0, -100.0, -700.0, -800.0, -5.0])
    u = np.array([0.5, 0.0, 0.0, 0.0, 0.999999])
    idx, _, counts = dev.accept(torch.from_numpy(lnl).cuda(), _keys_for([0.0]),
                                [dict(lnl_off=0, n=5, out_off=0, max_out=5, max_slot=0, u_off=0)],
                                u_source="array", u=torch.from_numpy(u).cuda())
    expect = np.where(np.exp(lnl) > u)[0]
    np.testing.assert_array_equal(idx[:int(counts[0])].cpu().numpy(), expect)
    idx, _, counts = dev.accept(torch.from_numpy(lnl).cuda(), _keys_for([float("nan")]),
                                [dict(lnl_off=0, n=5, out_off=0, max_out=5, max_slot=0, u_off=0)],
                                u_source="array", u=torch.from_numpy(u).cuda())
    assert int(counts[0]) == 0


def _reference_rejection(star, chunk, rng, max_post, n_lin, prior):
    """likelihood_helpers.rejection_sample_inmem restated with the oracle."""
    from oracle.oracle import posterior_linear_samples
    lls = oracle_lnl(star, chunk)
    uu = rng.uniform(size=len(lls))
    good = np.where(np.exp(lls - lls.max()) > uu)[0][:max_post]
    raw, _, _ = posterior_linear_samples(chunk[good], n_lin, rng, star["t"], star["rv"],
                                         star["ivar"], star["t_ref"], star["trend_M"],
                                         star["mu"], star["lam"], star["k_prior"])
    return good, raw, lls


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_thejoker_rejection_sample_matches_reference_pipeline(cuda, precision):
    from thejoker_gb300 import JokerPrior, RVData, TheJoker
    rng = np.random.default_rng(21)
    st = synth_star(rng, 12, K=5.0)
    prior = JokerPrior.default(P_min=2, P_max=1024, sigma_K0=30.0, sigma_v=100.0)
    data = RVData(st["t"], st["rv"], 1 / np.sqrt(st["ivar"]))
    samples = prior.sample(20000, rng=np.random.default_rng(3), return_logprobs=True)
    chunk = samples.pack()[0]
    joker = TheJoker(prior, rng=np.random.default_rng(42), precision=precision)
    out = joker.rejection_sample(data, samples, max_posterior_samples=300, return_logprobs=True,
                                 in_memory=True)
    good, raw, lls = _reference_rejection(st, chunk, np.random.default_rng(42), 300, 1, prior)
    assert len(out) == len(good) > 0
    np.testing.assert_array_equal(out["P"], chunk[good, 0])
    np.testing.assert_array_equal(out["ln_prior"], samples["ln_prior"][good])
    np.testing.assert_allclose(out["ln_likelihood"], lls[good], rtol=0,
                               atol=1e-4 if precision == "mixed" else 1e-8)
    np.testing.assert_allclose(out["K"], raw[:, 5], rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(out["v0"], raw[:, 6], rtol=1e-6, atol=1e-6)
    # the generator ends in the same state as the reference's
    r2 = np.random.default_rng(42)
    _reference_rejection(st, chunk, r2, 300, 1, prior)
    assert joker.rng.bit_generator.state == r2.bit_generator.state


def test_thejoker_iterative_matches_reference_loop(cuda):
    from thejoker_gb300 import JokerPrior, RVData, TheJoker
    rng = np.random.default_rng(22)
    st = synth_star(rng, 10, K=20.0)
    prior = JokerPrior.default(P_min=2, P_max=1024, sigma_K0=30.0, sigma_v=100.0)
    data = RVData(st["t"], st["rv"], 1 / np.sqrt(st["ivar"]))
    chunk = prior.sample(200000, rng=np.random.default_rng(4)).pack()[0]
    joker = TheJoker(prior, rng=np.random.default_rng(7), precision="fp64")
    out = joker.iterative_rejection_sample(data, chunk, n_requested_samples=8,
                                           init_batch_size=2000, in_memory=True)
    # likelihood_helpers.iterative_rejection_inmem restated
    r = np.random.default_rng(7)
    lls_all = oracle_lnl(st, chunk[:200000])
    n_process, start, allm = 2000, 0, np.array([])
    for _ in range(128):
        allm = np.concatenate([allm, lls_all[start:start + n_process]])
        uu = r.uniform(size=len(allm))
        good = np.where(np.exp(allm - allm.max()) > uu)[0]
        if len(good) >= 8:
            break
        start += n_process
        n_process = int(1 * (8 - len(good)) / len(good) * len(allm))
        n_process = min(n_process, 200000 - start)
    np.testing.assert_array_equal(out["P"], chunk[good[:8], 0])


@pytest.mark.parametrize("precision", ["mixed", "mixed_fast"])
@pytest.mark.parametrize("n_ep,K,jitter", [(3, 1.0, "reference"), (12, 5.0, "reference"),
                                           (40, 30.0, "applied"), (8, 0.5, "applied")])
def test_refined_accept_equals_fp64_accept(cuda, n_ep, K, jitter, precision):
    """Acceptance over mixed ln L with refinement keeps exactly what the FP64
    path keeps (same uniforms), while re-evaluating few samples in FP64."""
    from thejoker_gb300 import device as dev
    rng = np.random.default_rng(300 + n_ep)
    st = synth_star(rng, n_ep, K=K)
    S = 1 << 18
    chunk = synth_chunk(rng, S, jitter=(jitter == "applied"))
    table = dev.StarTable([st], jitter=jitter)
    cache = dev.PriorCache.from_samples(chunk)
    lnl64 = torch.empty((1, S), dtype=torch.float64, device="cuda")
    k64 = dev.MaxKeys(1)
    dev.lnl(table, cache, lnl64, precision="fp64", max_keys=k64)
    lnlm = torch.empty((1, S), dtype=torch.float64, device="cuda")
    err = torch.empty((1, S), dtype=torch.float32, device="cuda")
    km, bk = dev.MaxKeys(1), dev.MaxKeys(2)
    dev.lnl(table, cache, lnlm, precision=precision, max_keys=km, err=err, bound_keys=bk)
    gen = np.random.default_rng(5)
    pcg = dev.pcg64_state(gen)
    seg = dict(lnl_off=0, n=S, out_off=0, max_out=S, max_slot=0, star=0, row0=0,
               pcg=(pcg[0], pcg[1], 0))
    i64, _, c64 = dev.accept(lnl64.view(-1), k64, [seg])
    im, _, cm, exact, nref = dev.accept_refined(table, cache, lnlm.view(-1), err.view(-1), bk,
                                                [seg])
    n64, nm = int(c64[0]), int(cm[0])
    print(n_ep, K, jitter, precision, "accepted", n64, "refined in FP64", int(nref[0]))
    assert n64 == nm
    np.testing.assert_array_equal(i64[:n64].cpu().numpy(), im[:nm].cpu().numpy())
    # the refinement re-evaluates in FP64 through a separately compiled call
    # site; its maximum matches the FP64 kernel's to rounding
    np.testing.assert_allclose(exact.values()[0], k64.values()[0], rtol=1e-13)
    assert int(nref[0]) < S // 50


@pytest.mark.parametrize("precision", ["mixed", "mixed_fast"])
@pytest.mark.parametrize("K,sig", [(198.0, (0.1, 1.0)), (0.0, (2.0, 5.0))])
def test_refined_kept_lnl_within_tolerance(cuda, K, sig, precision):
    """Every kept sample's ln L (out_lnl) is within JOKER_MIXED_LNL_TOL of the FP64
    value: kept samples whose bound is looser are re-evaluated in FP64.  The
    first star is so well constrained that the best prior sample still has
    chi2 ~ 4e4 (mixed error ~1e-3 there); the second is constant with broad
    errors (many kept samples)."""
    from thejoker_gb300 import device as dev
    from thejoker_gb300.synthetic import fill_prior_cache
    rng = np.random.default_rng(0)
    st = synth_star(rng, 16, K=K, sig=sig)
    S = 1 << 20
    chunk = fill_prior_cache(np.empty((S, 5)), 0)
    cache = dev.PriorCache.from_samples(chunk)
    table = dev.StarTable([st])
    f64 = torch.empty((1, S), dtype=torch.float64, device="cuda")
    dev.lnl(table, cache, f64, precision="fp64")
    mix = torch.empty((1, S), dtype=torch.float64, device="cuda")
    err = torch.empty((1, S), dtype=torch.float32, device="cuda")
    bk = dev.MaxKeys(2)
    dev.lnl(table, cache, mix, precision=precision, err=err, bound_keys=bk)
    st_, inc = dev.pcg64_state(np.random.default_rng(5))
    seg = dict(lnl_off=0, n=S, idx_base=0, out_off=0, max_out=S, max_slot=0, star=0, row0=0,
               pcg=(st_, inc, 0))
    out_lnl = torch.empty(S, dtype=torch.float64, device="cuda")
    idx, _, cnt, _, _ = dev.accept_refined(table, cache, mix.view(-1), err.view(-1), bk, [seg],
                                           out_lnl=out_lnl)
    c = int(cnt[0])
    assert c > 0
    kept = idx[:c].cpu().numpy()
    ref = f64[0].cpu().numpy()
    got = out_lnl[:c].cpu().numpy()
    assert np.max(np.abs(got - ref[kept])) <= 1e-4
    # the FP64 acceptance keeps the same samples
    idx64, _, cnt64 = dev.accept(f64.view(-1), _keys_for([float(ref.max())]), [seg])
    np.testing.assert_array_equal(kept, idx64[:int(cnt64[0])].cpu().numpy())
