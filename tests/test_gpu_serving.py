"""Serving loop (GB300 only): stars arriving over time, continuously batched
into the device-resident iterative rounds.  A star's result is identical
whether it runs alone or mixed with others (different slots, pool ranges,
admission round), and matches the reference's iterative loop
(likelihood_helpers.py:130-229) on that star alone."""
import numpy as np
import pytest

from gpu_util import oracle_lnl
from test_gpu_iterative import reference_iterative

pytestmark = pytest.mark.gpu


def _requests(stars, rng):
    from thejoker_gb300.serve import Request
    out = []
    for k, st in enumerate(stars):
        n_req = int(rng.choice([4, 8, 16, 32]))
        budget = int(rng.choice([1 << 14, 1 << 15, 1 << 16, 1 << 17]))
        out.append(Request(st, budget=budget, n_requested=n_req, seed=1000 + k,
                           init_batch=min(budget, 128 * n_req)))
    return out


@pytest.fixture(scope="module")
def served():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from thejoker_gb300 import device as dev
    from thejoker_gb300.synthetic import fill_prior_cache, survey_stars
    stars = survey_stars(20, seed=33, n_min=6, n_max=64, poly_trend=2)
    S = 1 << 17
    chunk = fill_prior_cache(np.empty((S, 5)), 12)
    cache = dev.PriorCache.from_samples(chunk)
    return stars, chunk, cache


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_fast"])
def test_alone_equals_mix(cuda, served, precision):
    from thejoker_gb300.serve import ServingEngine
    stars, chunk, cache = served
    L = len(stars[0]["mu"])
    # alone: one slot, requests served one after another (slot and pool reuse)
    alone = ServingEngine(cache, n_slots=1, max_epochs=64, n_linear=L, pool_samples=1 << 17,
                          max_requested=32, precision=precision)
    reqs_a = _requests(stars, np.random.default_rng(5))
    for r in reqs_a:
        alone.submit(r)
        alone.drain()
    alone.close()
    # mix: few slots and a small pool, so admission waits for slots and memory;
    # a small round budget spreads the large batches over several rounds
    mix = ServingEngine(cache, n_slots=6, max_epochs=64, n_linear=L, pool_samples=3 << 16,
                        max_requested=32, precision=precision, round_budget=1 << 14)
    reqs_m = _requests(stars, np.random.default_rng(5))
    for r in reqs_m[:8]:
        mix.submit(r)
    mix.step()
    mix.step()
    for r in reqs_m[8:]:
        mix.submit(r)
    mix.drain()
    assert mix.rounds > 1
    assert mix.pool.available == mix.pool.size
    mix.close()
    for a, m in zip(reqs_a, reqs_m):
        ia, ga, ea, sa = a.result
        im, gm, em, sm = m.result
        assert (ga, ea, sa) == (gm, em, sm)
        np.testing.assert_array_equal(ia, im)


def test_serving_matches_reference_loop(cuda, served):
    from thejoker_gb300.serve import ServingEngine
    stars, chunk, cache = served
    L = len(stars[0]["mu"])
    eng = ServingEngine(cache, n_slots=8, max_epochs=64, n_linear=L, pool_samples=1 << 19,
                        max_requested=32, precision="mixed")
    reqs = _requests(stars[:10], np.random.default_rng(9))
    for r in reqs:
        eng.submit(r)
    eng.drain()
    stats = eng.latency_stats()
    assert stats["n"] == 10 and stats["p99_s"] >= stats["p50_s"] > 0
    eng.close()
    for k, r in enumerate(reqs):
        lls = oracle_lnl(stars[k], chunk[: r.budget])
        good, n_evals = reference_iterative(lls, r.seed, r.n_requested, r.init_batch, r.budget)
        idx, n_good, n_ev, status = r.result
        assert n_ev == n_evals, k
        if good is None:
            assert status == "no samples accepted"
            continue
        assert n_good == len(good), k
        np.testing.assert_array_equal(idx, good[: r.n_requested])


def test_admission_errors(cuda, served):
    from thejoker_gb300.serve import Request, ServingEngine
    stars, chunk, cache = served
    L = len(stars[0]["mu"])
    eng = ServingEngine(cache, n_slots=2, max_epochs=64, n_linear=L, pool_samples=1 << 16,
                        max_requested=8, precision="fp64")
    eng.submit(Request(stars[0], budget=cache.size * 2, n_requested=4, seed=0))
    with pytest.raises(ValueError):
        eng.step()
    eng.queue.clear()
    eng.submit(Request(stars[0], budget=1 << 14, n_requested=64, seed=0))
    with pytest.raises(ValueError):
        eng.step()
    eng.close()
