"""The reference's default sampling path (in_memory=False; GB300 only).

TheJoker.rejection_sample and iterative_rejection_sample default to the
file/pool path of thejoker/multiproc_helpers.py:185-427.  Against the in-memory
path it differs in four ways, each restated here with the CPU oracle and
numpy and compared with TheJoker's results:

* an optional random prefix order, rng.choice(n_total, size, replace=False),
  drawn from the caller's generator before the uniforms (:350-354, :247-250);
* safety factor 4 in the iterative growth rule (:334);
* no non-finite check in the iterative loop;
* the linear parameters drawn per pool task from generators spawned off the
  caller's seed sequence, the accepted rows split as utils.batch_tasks splits
  them (multiproc_helpers.py:17-60, 123-182).

Accepted indices and prior rows must be identical, the linear draws equal to
FP64 rounding, and the caller's generator must end in the same state with the
same number of spawned children.
"""
import numpy as np
import pytest

from gpu_util import oracle_lnl, synth_star

pytestmark = pytest.mark.gpu


def _tasks(arr, n_batches):
    # utils.batch_tasks (:22-72): n_batches runs, the first n % n_batches one
    # longer, or a single run when there are fewer rows than batches
    if n_batches > 0 and len(arr) >= n_batches:
        return np.array_split(arr, n_batches)
    return [arr]


def _full_samples(star, chunk, full_idx, n_lin, rng, n_batches):
    """make_full_samples restated: spawned generators, one per task."""
    from numpy.random import PCG64, Generator
    from oracle.oracle import posterior_linear_samples
    tasks = _tasks(full_idx, n_batches)
    seqs = rng.bit_generator._seed_seq.spawn(len(tasks))
    raws = []
    for idx, sq in zip(tasks, seqs):
        raw, _, _ = posterior_linear_samples(chunk[idx], n_lin, Generator(PCG64(sq)), star["t"],
                                             star["rv"], star["ivar"], star["t_ref"],
                                             star["trend_M"], star["mu"], star["lam"],
                                             star["k_prior"])
        raws.append(raw)
    return np.concatenate(raws)


def _reference_pool_rejection(star, chunk, rng, n_prior, max_post, n_lin, n_batches, randomize):
    """rejection_sample_helper (multiproc_helpers.py:185-286) restated."""
    n_total = len(chunk)
    idx = rng.choice(n_total, size=n_prior, replace=False) if randomize else None
    rows = chunk[idx] if randomize else chunk[:n_prior]
    lls = oracle_lnl(star, rows)
    uu = rng.uniform(size=len(lls))
    good = np.where(np.exp(lls - lls.max()) > uu)[0][:max_post]
    full = idx[good] if randomize else good
    raw = _full_samples(star, chunk, full, n_lin, rng, n_batches)
    return good, full, raw, lls


def _reference_pool_iterative(star, chunk, rng, n_req, n_lin, n_batches, randomize, init_batch,
                              max_prior=None, growth=128):
    """iterative_rejection_helper (multiproc_helpers.py:289-427) restated."""
    n_total = len(chunk)
    max_prior = n_total if max_prior is None else max_prior
    n_process = growth * n_req if init_batch is None else init_batch
    assert n_process <= max_prior
    all_idx = rng.choice(n_total, size=max_prior, replace=False) if randomize \
        else np.arange(max_prior)
    lls_lib = oracle_lnl(star, chunk[all_idx])
    allm, start = np.array([]), 0
    for _ in range(128):
        allm = np.concatenate([allm, lls_lib[start:start + n_process]])
        uu = rng.uniform(size=len(allm))
        good = np.where(np.exp(allm - allm.max()) > uu)[0]
        assert len(good) > 0
        if len(good) >= n_req:
            break
        start += n_process
        n_process = int(4 * (n_req - len(good)) / len(good) * len(allm))
        if start + n_process > max_prior:
            n_process = max_prior - start
        if n_process <= 0:
            break
    good = good[:n_req]
    full = all_idx[good]
    raw = _full_samples(star, chunk, full, n_lin, rng, n_batches)
    return good, full, raw, allm


def _setup(seed, n_ep, K, S, poly=1):
    from thejoker_gb300 import JokerPrior, RVData
    rng = np.random.default_rng(seed)
    st = synth_star(rng, n_ep, K=K, poly=poly)
    prior = JokerPrior.default(P_min=2, P_max=1024, sigma_K0=30.0,
                               sigma_v=[100.0, 1.0][:poly], poly_trend=poly)
    data = RVData(st["t"], st["rv"], 1 / np.sqrt(st["ivar"]))
    samples = prior.sample(S, rng=np.random.default_rng(seed + 1), return_logprobs=True)
    return st, prior, data, samples


class _Pool:
    """A stand-in processing pool: map and close, and a size."""

    def __init__(self, size):
        self.size = size

    def map(self, fn, tasks):
        return list(map(fn, tasks))

    def close(self):
        pass


@pytest.mark.parametrize("precision,randomize,n_batches,pool_size",
                         [("fp64", False, None, None), ("fp64", True, 3, None),
                          ("mixed", True, None, 4), ("mixed", False, 5, 2)])
def test_pool_rejection_matches_reference_helper(cuda, precision, randomize, n_batches,
                                                 pool_size):
    from thejoker_gb300 import TheJoker
    st, prior, data, samples = _setup(41, 4, 2.0, 30000)
    chunk = samples.pack()[0]
    pool = _Pool(pool_size) if pool_size is not None else None
    joker = TheJoker(prior, pool=pool, rng=np.random.default_rng(42), precision=precision)
    n_prior, max_post, n_lin = 24000, 500, 2
    out, lls = joker.rejection_sample(data, samples, n_prior_samples=n_prior,
                                      max_posterior_samples=max_post, n_linear_samples=n_lin,
                                      return_logprobs=True, return_all_logprobs=True,
                                      n_batches=n_batches, randomize_prior_order=randomize)
    r = np.random.default_rng(42)
    nb = n_batches if n_batches is not None else max(1, pool_size or 0)
    good, full, raw, lls_ref = _reference_pool_rejection(st, chunk, r, n_prior, max_post, n_lin,
                                                         nb, randomize)
    assert len(good) > 10
    assert len(out) == len(full) * n_lin
    np.testing.assert_array_equal(out["P"], np.repeat(chunk[full, 0], n_lin))
    np.testing.assert_array_equal(out["e"], np.repeat(chunk[full, 1], n_lin))
    np.testing.assert_allclose(out["K"], raw[:, 5], rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(out["v0"], raw[:, 6], rtol=1e-6, atol=1e-6)
    np.testing.assert_array_equal(out["ln_prior"], np.repeat(samples["ln_prior"][full], n_lin))
    # all ln L: FP64 to 1e-9; mixed within 1e-4 inside the band of the maximum
    if precision == "fp64":
        np.testing.assert_allclose(lls, lls_ref, rtol=1e-9, atol=1e-9)
    else:
        band = lls_ref >= lls_ref.max() - 40.0
        assert np.max(np.abs(lls - lls_ref)[band]) <= 1e-4
    np.testing.assert_allclose(out["ln_likelihood"], np.repeat(lls_ref[good], n_lin),
                               rtol=0, atol=1e-4 if precision == "mixed" else 1e-8)
    assert joker.rng.bit_generator.state == r.bit_generator.state
    assert joker.rng.bit_generator._seed_seq.n_children_spawned == \
        r.bit_generator._seed_seq.n_children_spawned


@pytest.mark.parametrize("precision,randomize,n_batches", [("fp64", False, None),
                                                           ("fp64", True, 2),
                                                           ("mixed", True, 3)])
def test_pool_iterative_matches_reference_helper(cuda, precision, randomize, n_batches):
    from thejoker_gb300 import TheJoker
    st, prior, data, samples = _setup(52, 10, 20.0, 200000)
    chunk = samples.pack()[0]
    joker = TheJoker(prior, rng=np.random.default_rng(7), precision=precision)
    out = joker.iterative_rejection_sample(data, samples, n_requested_samples=16,
                                           init_batch_size=2000, n_batches=n_batches,
                                           randomize_prior_order=randomize,
                                           return_logprobs=True)
    r = np.random.default_rng(7)
    nb = n_batches if n_batches is not None else 1
    good, full, raw, allm = _reference_pool_iterative(st, chunk, r, 16, 1, nb, randomize, 2000)
    np.testing.assert_array_equal(out["P"], chunk[full, 0])
    np.testing.assert_allclose(out["K"], raw[:, 5], rtol=1e-6, atol=1e-6)
    np.testing.assert_array_equal(out["ln_prior"], samples["ln_prior"][full])
    np.testing.assert_allclose(out["ln_likelihood"], allm[good], rtol=0,
                               atol=1e-4 if precision == "mixed" else 1e-8)
    assert joker.rng.bit_generator.state == r.bit_generator.state


def test_pool_iterative_safety_factor_differs_from_in_memory(cuda):
    """The two paths grow their batches differently (safety factor 4 against
    1), so with the same generator they need not evaluate the same prefix;
    each matches its own restatement."""
    from thejoker_gb300 import TheJoker
    st, prior, data, samples = _setup(63, 4, 3.0, 100000)
    chunk = samples.pack()[0]
    j1 = TheJoker(prior, rng=np.random.default_rng(9))
    j2 = TheJoker(prior, rng=np.random.default_rng(9))
    a = j1.iterative_rejection_sample(data, samples, n_requested_samples=32, init_batch_size=500,
                                      in_memory=True)
    b = j2.iterative_rejection_sample(data, samples, n_requested_samples=32, init_batch_size=500)
    good, full, _, _ = _reference_pool_iterative(st, chunk, np.random.default_rng(9), 32, 1, 1,
                                                 False, 500)
    np.testing.assert_array_equal(b["P"], chunk[full, 0])
    assert len(a) == len(b) == 32


def test_randomize_prior_order_is_deterministic(cuda):
    """test_sampler.py:199-211 of the reference: with a seeded generator the
    iterative path over a randomly ordered prior gives the same samples each
    time (3 epochs, 10,000 prior samples, 4 requested)."""
    from thejoker_gb300 import TheJoker
    st, prior, data, samples = _setup(74, 3, 10.0, 10000)
    Ps, Ks = [], []
    for _ in range(5):
        joker = TheJoker(prior, rng=np.random.default_rng(42))
        s = joker.iterative_rejection_sample(data, samples, n_requested_samples=4,
                                             randomize_prior_order=True)
        Ps.append(s["P"])
        Ks.append(s["K"])
    for i in range(1, len(Ps)):
        np.testing.assert_array_equal(Ps[0], Ps[i])
        np.testing.assert_array_equal(Ks[0], Ks[i])


def test_pool_path_rejects_plain_arrays(cuda):
    """The file/pool path takes a filename or a JokerSamples, as the
    reference's tempfile_decorator does; the in-memory path takes arrays."""
    from thejoker_gb300 import TheJoker
    st, prior, data, samples = _setup(85, 6, 5.0, 4096)
    chunk = samples.pack()[0]
    joker = TheJoker(prior, rng=np.random.default_rng(1))
    with pytest.raises(TypeError):
        joker.rejection_sample(data, chunk)
    with pytest.raises(TypeError):
        joker.marginal_ln_likelihood(data, chunk)
    a = joker.marginal_ln_likelihood(data, chunk, in_memory=True)
    b = joker.marginal_ln_likelihood(data, samples)
    np.testing.assert_array_equal(a, b)
    no_lnp = prior.sample(4096, rng=np.random.default_rng(2))
    with pytest.raises(RuntimeError, match="ln_prior"):
        joker.rejection_sample(data, no_lnp, return_logprobs=True)
