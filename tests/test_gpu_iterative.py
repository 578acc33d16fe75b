"""Iterative rejection on the device (GB300 only): the rounds, replayed from a
CUDA graph, reproduce the reference's iterative_rejection_inmem
(likelihood_helpers.py:130-229) star by star -- same batch schedule, same
fresh uniforms for the whole prefix every round, same accepted indices."""
import numpy as np
import pytest

from gpu_util import oracle_lnl

pytestmark = pytest.mark.gpu


def reference_iterative(lls_all, seed, n_req, init, n_total, safety=1.0, maxiter=128):
    rng = np.random.default_rng(seed)
    n_process, start, allm = init, 0, np.array([])
    good = None
    for _ in range(maxiter):
        allm = np.concatenate([allm, lls_all[start:start + n_process]])
        uu = rng.uniform(size=len(allm))
        good = np.where(np.exp(allm - allm.max()) > uu)[0]
        if len(good) == 0:
            return None, len(allm)
        if len(good) >= n_req:
            break
        start += n_process
        n_process = int(safety * (n_req - len(good)) / len(good) * len(allm))
        if start + n_process > n_total:
            n_process = n_total - start
        if n_process <= 0:
            break
    return good, len(allm)


@pytest.mark.parametrize("precision,use_graph", [("fp64", False), ("fp64", True),
                                                 ("mixed", True)])
def test_iterative_matches_reference_loop(cuda, precision, use_graph):
    from thejoker_gb300 import device as dev
    from thejoker_gb300.iterative import IterativeBatch
    from thejoker_gb300.synthetic import fill_prior_cache, survey_stars
    stars = survey_stars(12, seed=21, n_min=8, n_max=64, poly_trend=3)
    S = 1 << 17
    chunk = fill_prior_cache(np.empty((S, 5)), 8)
    cache = dev.PriorCache.from_samples(chunk)
    table = dev.StarTable(stars)
    seeds = np.arange(12) + 50
    n_req, init = 16, 2048
    it = IterativeBatch(table, cache, n_req, precision=precision, seeds=seeds,
                        init_batch_size=init)
    it.run(use_graph=use_graph)
    state, idx, nref = it.results()
    for k in range(12):
        lls = oracle_lnl(stars[k], chunk)
        good, n_evals = reference_iterative(lls, int(seeds[k]), n_req, init, S)
        assert state[k, 2] == n_evals, k
        if good is None:
            assert state[k, 4] == 2
            continue
        assert state[k, 3] == len(good), k
        np.testing.assert_array_equal(idx[k], good[:n_req])
