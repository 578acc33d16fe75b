"""Batched rejection sampling of many stars over one shared prior cache
(GB300 only): the result per star equals the reference's rejection step run
star by star (likelihood_helpers.py:91-127, restated with the oracle and
numpy's own uniforms), and the mixed path keeps what the FP64 path keeps."""
import numpy as np
import pytest
import torch

from gpu_util import oracle_lnl

pytestmark = pytest.mark.gpu


def test_batch_matches_per_star_reference(cuda):
    from thejoker_gb300 import device as dev
    from thejoker_gb300.batch import BatchRejection
    from thejoker_gb300.synthetic import fill_prior_cache, survey_stars
    stars = survey_stars(40, seed=9, n_max=64)
    S = 1 << 15
    chunk = fill_prior_cache(np.empty((S, 5)), 4)
    cache = dev.PriorCache.from_samples(chunk)
    seeds = np.arange(40) + 100
    res = {}
    for prec in ("fp64", "mixed"):
        b = BatchRejection(stars, cache, precision=prec, max_out=64, seeds=seeds, group=16)
        b.run()
        res[prec] = b.results()
    c64, i64, l64 = res["fp64"]
    cm, im, lm = res["mixed"]
    np.testing.assert_array_equal(c64, cm)
    for k in range(40):
        np.testing.assert_array_equal(i64[k], im[k])
    for k in range(0, 40, 7):
        lls = oracle_lnl(stars[k], chunk)
        uu = np.random.default_rng(int(seeds[k])).uniform(size=S)
        good = np.where(np.exp(lls - lls.max()) > uu)[0]
        assert c64[k] == len(good), k
        np.testing.assert_array_equal(i64[k], good[:64])
        np.testing.assert_allclose(l64[k], lls[good[:64]], rtol=2e-8)


def test_batch_rows_subrange(cuda):
    from thejoker_gb300 import device as dev
    from thejoker_gb300.batch import BatchRejection
    from thejoker_gb300.synthetic import fill_prior_cache, survey_stars
    stars = survey_stars(5, seed=10, n_max=30)
    S = 1 << 14
    chunk = fill_prior_cache(np.empty((S, 5)), 5)
    cache = dev.PriorCache.from_samples(chunk)
    b = BatchRejection(stars, cache, precision="mixed", max_out=1000, seeds=[1, 2, 3, 4, 5])
    b.run(row0=1000, count=5000)
    counts, idx, _ = b.results()
    for k in range(5):
        lls = oracle_lnl(stars[k], chunk[1000:6000])
        uu = np.random.default_rng(k + 1).uniform(size=5000)
        good = np.where(np.exp(lls - lls.max()) > uu)[0] + 1000
        assert counts[k] == len(good)
        np.testing.assert_array_equal(idx[k], good[:1000])


def test_host_pipeline_matches_batch(cuda):
    """Streaming a host chunk in slices (copies overlapped with ln L) gives the
    same accepted indices as the resident-cache path."""
    from thejoker_gb300 import device as dev
    from thejoker_gb300.batch import BatchRejection
    from thejoker_gb300.pipeline import HostRejection
    from thejoker_gb300.synthetic import fill_prior_cache, survey_stars
    stars = survey_stars(6, seed=12, n_max=40)
    S = 100_000
    chunk = fill_prior_cache(np.empty((S, 5)), 6)
    table = dev.StarTable(stars)
    seeds = [11, 12, 13, 14, 15, 16]
    host = torch.from_numpy(chunk).pin_memory()
    for prec in ("mixed", "fp64"):
        hr = HostRejection(table, S, precision=prec, slice_rows=30_000, max_out=500)
        pcg = [dev.pcg64_state(np.random.default_rng(sd)) for sd in seeds]
        counts, idx = hr.run(host, pcg)
        cache = dev.PriorCache.from_samples(chunk)
        b = BatchRejection(table, cache, precision=prec, max_out=500, seeds=seeds)
        b.run()
        c2, i2, _ = b.results()
        np.testing.assert_array_equal(counts, c2)
        for k in range(6):
            np.testing.assert_array_equal(idx[k], i2[k])


def test_autotune_records_fastest_chunk(cuda, tmp_path):
    from thejoker_gb300 import autotune as at
    from thejoker_gb300 import device as dev
    from thejoker_gb300.batch import BatchRejection
    from thejoker_gb300.synthetic import fill_prior_cache, survey_stars
    stars = survey_stars(8, seed=5, n_min=10, n_max=40)
    cache = dev.PriorCache.from_samples(fill_prior_cache(np.empty((1 << 18, 5)), 3))
    table = dev.StarTable(stars)
    path = str(tmp_path / "tune.json")
    # the engines' default precision, whose tuning times the fused ln L kernel
    best, times = at.tune(table, cache, precision="mixed_fast", candidates=(256, 1024, 4096),
                          reps=1, path=path)
    assert best in (256, 1024, 4096) and times[best] == min(times.values())
    assert at.chunk_for(table.n_linear, table.jitter, "mixed_fast", table.n_epochs,
                        path=path) == best
    # an engine built without a chunk picks the tuned size
    import os
    os.environ["JOKER_AUTOTUNE"] = path
    try:
        assert BatchRejection(table, cache, max_out=4).chunk == best
    finally:
        del os.environ["JOKER_AUTOTUNE"]


@pytest.mark.parametrize("precision", ["mixed", "mixed_fast", "fp64"])
def test_one_call_rejection_equals_engine(cuda, precision):
    """joker_rejection_sample (ln L + maxima + acceptance in one C call) keeps
    the same rows, counts and ln L as the BatchRejection engine, including a
    star longer than one epoch tile."""
    import ctypes
    from gpu_util import synth_chunk, synth_star
    from thejoker_gb300 import _native as nat
    from thejoker_gb300 import device as dev
    from thejoker_gb300._native import JokerError
    from thejoker_gb300.batch import BatchRejection
    rng = np.random.default_rng(17)
    stars = [synth_star(rng, n) for n in (12, 40, 300)]
    S, max_out, seeds = 1 << 18, 512, [11, 22, 33]
    cache = dev.PriorCache.from_samples(synth_chunk(rng, S, jitter=True))
    table = dev.StarTable(stars, jitter="applied")
    counts, idx, ll = BatchRejection(table, cache, precision=precision, max_out=max_out,
                                     seeds=seeds).run().results()
    prec = dev.PRECISIONS[precision]
    mask = (1 << 64) - 1
    words = []
    for sd in seeds:
        st, inc = dev.pcg64_state(np.random.default_rng(sd))
        words += [st >> 64, st & mask, inc >> 64, inc & mask]
    pcg = (ctypes.c_uint64 * len(words))(*words)
    nbytes = nat.lib().joker_rejection_workspace(len(stars), S, max_out, prec)
    work = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    out_idx = torch.empty(len(stars) * max_out, dtype=torch.int64, device="cuda")
    out_lnl = torch.empty(len(stars) * max_out, dtype=torch.float64, device="cuda")
    cnt = torch.empty(len(stars), dtype=torch.int64, device="cuda")
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    nat.check(nat.lib().joker_rejection_sample(table.handle, cache.handle, 0, len(stars), 0, S,
                                               prec, pcg, max_out, p(out_idx), p(out_lnl),
                                               p(cnt), p(work), nbytes, stream),
              "joker_rejection_sample")
    got_c = cnt.cpu().numpy()
    np.testing.assert_array_equal(got_c, counts)
    oi = out_idx.view(len(stars), max_out).cpu().numpy()
    ol = out_lnl.view(len(stars), max_out).cpu().numpy()
    for k in range(len(stars)):
        n = min(int(counts[k]), max_out)
        np.testing.assert_array_equal(oi[k, :n], idx[k])
        np.testing.assert_array_equal(ol[k, :n], ll[k])
    assert counts.sum() > 0
    with pytest.raises(JokerError):
        nat.check(nat.lib().joker_rejection_sample(table.handle, cache.handle, 0, len(stars), 0,
                                                   S, prec, pcg, max_out, p(out_idx), p(out_lnl),
                                                   p(cnt), p(work), nbytes - 256, stream),
                  "joker_rejection_sample")
