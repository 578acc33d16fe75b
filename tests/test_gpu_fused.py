"""The fused first acceptance pass (GB300 only): joker_lnl_fused draws each
sample's uniform inside the ln L kernel and leaves a candidate bit;
joker_accept_fused decides the candidates.  The kept rows must be exactly
those of the FP64 path (the reference's rejection step,
thejoker/likelihood_helpers.py:107-109, on FP64 ln L and the same numpy
uniforms) for every layout: many stars in one launch, stars longer than one
epoch tile, work items of 128 to 8192 samples, sub-ranges of the cache,
slices of a host chunk, packed cache views."""
import ctypes

import numpy as np
import pytest
import torch

from gpu_util import synth_chunk, synth_star

pytestmark = pytest.mark.gpu


def _engine(table, cache, precision, seeds, max_out, **kw):
    from thejoker_gb300.batch import BatchRejection
    b = BatchRejection(table, cache, precision=precision, max_out=max_out, seeds=seeds, **kw)
    b.run()
    return b


def _same(r64, rf, n_stars, lnl_tol=1e-4):
    c64, i64, l64 = r64
    cf, i_f, lf = rf
    np.testing.assert_array_equal(cf, c64)
    for k in range(n_stars):
        np.testing.assert_array_equal(i_f[k], i64[k])
        if len(l64[k]):
            assert np.max(np.abs(lf[k] - l64[k])) <= lnl_tol


STAR_SETS = {
    # few epochs, small K: a broad posterior, thousands of samples kept
    "weak": dict(ns=[3], K=[1.0], jitter="reference", poly=1, noff=0),
    # mixed epoch counts in one launch, one star above the 256-epoch tile
    "group": dict(ns=[3, 12, 40, 300], K=[0.5, 5.0, 30.0, 20.0], jitter="applied", poly=1,
                  noff=0),
    # three linear parameters (an offset) with the jitter applied
    "offset_jitter": dict(ns=[9, 24], K=[2.0, 10.0], jitter="applied", poly=1, noff=1),
    # four linear parameters (a quadratic trend and an offset), no jitter
    "trend": dict(ns=[16, 50], K=[3.0, 40.0], jitter="reference", poly=2, noff=1),
}


@pytest.mark.parametrize("name", sorted(STAR_SETS))
def test_fused_engine_keeps_fp64_rows(cuda, name):
    from thejoker_gb300 import device as dev
    cfg = STAR_SETS[name]
    rng = np.random.default_rng(len(name) * 31 + 7)
    stars = [synth_star(rng, n, K=k, poly=cfg["poly"], noff=cfg["noff"])
             for n, k in zip(cfg["ns"], cfg["K"])]
    S = (1 << 18) + 77                             # a ragged last word and work item
    cache = dev.PriorCache.from_samples(synth_chunk(rng, S, jitter=True))
    table = dev.StarTable(stars, jitter=cfg["jitter"])
    seeds = [101 + k for k in range(len(stars))]
    r64 = _engine(table, cache, "fp64", seeds, 4096).results()
    bf = _engine(table, cache, "mixed_fast", seeds, 4096)
    assert bf.fused
    _same(r64, bf.results(), len(stars))
    assert r64[0].sum() > 0
    print(name, "kept", r64[0], "refined in FP64", bf.n_refined_last)
    assert bf.n_refined_last < S * len(stars) // 50


@pytest.mark.parametrize("chunk", [128, 384, 8192])
def test_fused_work_item_sizes(cuda, chunk):
    """The per-pass generator states of a work item (one per 256 samples)
    and its candidate words for items of 1 to 32 passes, and a last item
    shorter than one pass."""
    from thejoker_gb300 import device as dev
    rng = np.random.default_rng(chunk)
    stars = [synth_star(rng, 5, K=1.0), synth_star(rng, 30, K=8.0)]
    S = 3 * 8192 + 200
    cache = dev.PriorCache.from_samples(synth_chunk(rng, S, jitter=True))
    table = dev.StarTable(stars, jitter="applied")
    r64 = _engine(table, cache, "fp64", [7, 8], S).results()
    rf = _engine(table, cache, "mixed_fast", [7, 8], S, chunk=chunk).results()
    _same(r64, rf, 2)


def test_fused_rows_subrange(cuda):
    """Rows [1000, 6000) of the cache: uniform j of each star is draw j of
    its stream, whatever the first row."""
    from thejoker_gb300 import device as dev
    from thejoker_gb300.batch import BatchRejection
    rng = np.random.default_rng(3)
    stars = [synth_star(rng, n, K=2.0) for n in (4, 10, 33)]
    S = 1 << 14
    cache = dev.PriorCache.from_samples(synth_chunk(rng, S))
    table = dev.StarTable(stars)
    out = {}
    for prec in ("fp64", "mixed_fast"):
        b = BatchRejection(table, cache, precision=prec, max_out=5000, seeds=[1, 2, 3])
        b.run(row0=1000, count=5000)
        out[prec] = b.results()
    _same(out["fp64"], out["mixed_fast"], 3)


def test_candidate_bits_cover_every_kept_sample(cuda):
    """Direct joker_lnl_fused call: every sample the FP64 rule keeps
    (exp(lnL_64 - max) > u, numpy's own uniforms) has its bit; bits past the
    last sample of a word are clear; most samples of an informative star
    have none (all of this small case's work items run in the first wave,
    before the running lower bound has settled)."""
    from thejoker_gb300 import device as dev
    rng = np.random.default_rng(11)
    st = synth_star(rng, 20, K=15.0)
    S = 200_003
    cache = dev.PriorCache.from_samples(synth_chunk(rng, S, jitter=True))
    table = dev.StarTable([st], jitter="applied")
    f64 = torch.empty((1, S), dtype=torch.float64, device="cuda")
    dev.lnl(table, cache, f64, precision="fp64")
    l64 = f64[0].cpu().numpy()
    uu = np.random.default_rng(42).uniform(size=S)
    kept = np.exp(l64 - l64.max()) > uu
    lnl = torch.empty((1, S), dtype=torch.float64, device="cuda")
    err = torch.empty((1, S), dtype=torch.float32, device="cuda")
    bk = dev.MaxKeys(2)
    pcg = dev.pcg_table([dev.pcg64_state(np.random.default_rng(42))])
    ld, cand = dev.cand_words(1, S)
    cand.fill_(-1)
    dev.lnl_fused(table, cache, lnl, err, bk, pcg, cand, ld)
    words = cand[0].cpu().numpy().view(np.uint32)
    bits = np.unpackbits(words.view(np.uint8), bitorder="little")
    assert np.all(bits[:S][kept])
    assert not np.any(bits[S:32 * ((S + 31) // 32)])
    n_cand = int(bits[:S].sum())
    print("kept", int(kept.sum()), "candidates", n_cand)
    assert n_cand >= kept.sum() and n_cand < S // 2


@pytest.mark.parametrize("zero_copy,slice_rows", [(True, 1 << 16), (False, 1 << 15)])
def test_fused_host_pipeline(cuda, zero_copy, slice_rows):
    """HostRejection with the fused pass: one packed-view launch, or slices of
    the host chunk (each slice's first sample a multiple of 32 into the
    stream)."""
    from thejoker_gb300 import device as dev
    from thejoker_gb300.pipeline import HostRejection
    from thejoker_gb300.synthetic import fill_prior_cache, survey_stars
    stars = survey_stars(5, seed=21, n_max=40)
    S = 100_000
    chunk = fill_prior_cache(np.empty((S, 5)), 7)
    table = dev.StarTable(stars)
    seeds = [31, 32, 33, 34, 35]
    host = torch.from_numpy(chunk).pin_memory()
    pcg = [dev.pcg64_state(np.random.default_rng(sd)) for sd in seeds]
    hr = HostRejection(table, S, precision="mixed_fast", slice_rows=slice_rows, max_out=700,
                       zero_copy=zero_copy)
    assert hr.fused
    counts, idx = hr.run(host, pcg)
    cache = dev.PriorCache.from_samples(chunk)
    c64, i64, _ = _engine(table, cache, "fp64", seeds, 700).results()
    np.testing.assert_array_equal(counts, c64)
    for k in range(5):
        np.testing.assert_array_equal(idx[k], i64[k])


def test_fused_arguments_rejected(cuda):
    """Host-side checks of joker_lnl_fused (no kernel runs): work items above
    8192 samples, a first sample off a 32-sample boundary, too few candidate
    words, a jittered table with four linear parameters."""
    from thejoker_gb300 import _native as nat
    from thejoker_gb300 import device as dev
    from thejoker_gb300._native import JokerError
    rng = np.random.default_rng(5)
    S = 4096
    cache = dev.PriorCache.from_samples(synth_chunk(rng, S, jitter=True))
    table = dev.StarTable([synth_star(rng, 10)], jitter="applied")
    lnl = torch.empty((1, S), dtype=torch.float64, device="cuda")
    err = torch.empty((1, S), dtype=torch.float32, device="cuda")
    bk = dev.MaxKeys(2)
    pcg = dev.pcg_table([(1, 3)])
    ld, cand = dev.cand_words(1, S + 64)
    for kw in (dict(chunk=8192 + 128), dict(chunk=200), dict(first=16)):
        with pytest.raises(JokerError):
            dev.lnl_fused(table, cache, lnl, err, bk, pcg, cand, ld, **kw)
    with pytest.raises(JokerError):
        dev.lnl_fused(table, cache, lnl, err, bk, pcg, cand, S // 32 - 1)
    big = dev.StarTable([synth_star(rng, 10, poly=3)], jitter="applied")   # L = 4
    assert not dev.fused_available(big, "mixed_fast")
    with pytest.raises(JokerError):
        dev.lnl_fused(big, cache, lnl, err, bk, pcg, cand, ld)
    assert nat.lib().joker_last_error()


@pytest.mark.parametrize("S", [1, 31, 33, 257])
def test_fused_tiny_and_ragged(cuda, S):
    """Caches of 1, 31, 33 and 257 samples: a partial first word, a work item
    shorter than one pass, and a second pass with a single active sample."""
    from thejoker_gb300 import device as dev
    rng = np.random.default_rng(S)
    stars = [synth_star(rng, 3, K=0.5), synth_star(rng, 12, K=5.0)]
    cache = dev.PriorCache.from_samples(synth_chunk(rng, S, jitter=True))
    table = dev.StarTable(stars, jitter="applied")
    r64 = _engine(table, cache, "fp64", [5, 6], S).results()
    rf = _engine(table, cache, "mixed_fast", [5, 6], S, chunk=128).results()
    _same(r64, rf, 2)


def test_fused_nan_rows_and_max_out_one(cuda):
    """Rows with e >= 1 give NaN ln L, and a NaN maximum keeps nothing (numpy's
    exp(lls - nan) > u is False), in both paths; with max_out = 1 the counts
    are still those of every kept sample."""
    from thejoker_gb300 import device as dev
    rng = np.random.default_rng(77)
    stars = [synth_star(rng, 6, K=1.0), synth_star(rng, 9, K=1.0)]
    S = 5000
    ch = synth_chunk(rng, S)
    cache_ok = dev.PriorCache.from_samples(ch)
    table = dev.StarTable(stars)
    r64 = _engine(table, cache_ok, "fp64", [1, 2], 1).results()
    rf = _engine(table, cache_ok, "mixed_fast", [1, 2], 1).results()
    _same(r64, rf, 2)
    assert r64[0].min() > 1 and all(len(x) == 1 for x in rf[1])
    ch_bad = ch.copy()
    ch_bad[1234, 1] = 1.5                                 # e >= 1: NaN ln L
    cache_bad = dev.PriorCache.from_samples(ch_bad)
    c64 = _engine(table, cache_bad, "fp64", [1, 2], S).results()[0]
    cf = _engine(table, cache_bad, "mixed_fast", [1, 2], S).results()[0]
    np.testing.assert_array_equal(cf, c64)
    assert c64.sum() == 0


EXIT_SETS = {
    # jitter applied, K and v0; an offset column; no jitter with a linear trend
    "jitter_L2": dict(ns=[40, 12], K=[20.0, 2.0], jitter="applied", poly=1, noff=0),
    "jitter_L3": dict(ns=[30, 9], K=[15.0, 3.0], jitter="applied", poly=1, noff=1),
    "plain_L3": dict(ns=[36, 20], K=[25.0, 5.0], jitter="reference", poly=2, noff=0),
    # a star above the 256-epoch tile (no checkpoints) beside one with fewer
    # epochs than the first checkpoint (only the test after the last epoch)
    "long_short": dict(ns=[300, 6], K=[20.0, 30.0], jitter="applied", poly=1, noff=0),
}


@pytest.mark.parametrize("name", sorted(EXIT_SETS))
def test_early_exit_keeps_fp64_rows(cuda, name):
    """With early exit the kept rows (and their ln L) are still the FP64
    path's, on stars informative enough for most warps to stop early."""
    from thejoker_gb300 import device as dev
    cfg = EXIT_SETS[name]
    rng = np.random.default_rng(len(name) * 7 + 1)
    stars = [synth_star(rng, n, K=k, poly=cfg["poly"], noff=cfg["noff"], sig=(0.05, 0.3))
             for n, k in zip(cfg["ns"], cfg["K"])]
    S = 1 << 20
    cache = dev.PriorCache.from_samples(synth_chunk(rng, S, jitter=True))
    table = dev.StarTable(stars, jitter=cfg["jitter"])
    seeds = [201 + k for k in range(len(stars))]
    r64 = _engine(table, cache, "fp64", seeds, 4096).results()
    rx = _engine(table, cache, "mixed_fast", seeds, 4096, early_exit=True).results()
    _same(r64, rx, len(stars))
    assert r64[0].sum() > 0


@pytest.mark.parametrize("early_exit", [True, False])
@pytest.mark.parametrize("jitter", ["applied", "reference"])
def test_early_exit_values_are_upper_bounds(cuda, jitter, early_exit):
    """Direct joker_lnl_fused call: every sample whose error bound is
    infinite (with early exit, its warp stopped at a checkpoint; with or
    without it, its warp was out of reach after its last epoch) holds a
    value at or above its FP64 ln L (up to FP32 rounding after the last
    epoch; without early exit that FP32 ln L itself), lies more than 746
    nats below the maximum, and has no candidate bit; the other samples hold
    their usual values and bounds.  An
    eighth of the orbits (a contiguous block, so that whole warps hold them)
    have e in [0.9, 0.995], where the FP32 column's own error is largest."""
    from thejoker_gb300 import device as dev
    rng = np.random.default_rng(5 if jitter == "applied" else 6)
    st = synth_star(rng, 80, K=100.0, sig=(0.05, 0.2), base=2000.0)   # informative
    # enough work items (512 samples each) for many waves: the warps of the
    # first wave see no settled lower bound and run to the end
    S = 1 << 23
    ch = synth_chunk(rng, S, jitter=True)
    ecc = slice(S // 2, S // 2 + S // 8)                  # eccentric orbits: large column error
    ch[ecc, 1] = rng.uniform(0.9, 0.995, S // 8)
    cache = dev.PriorCache.from_samples(ch)
    table = dev.StarTable([st], jitter=jitter)
    f64 = torch.empty((1, S), dtype=torch.float64, device="cuda")
    dev.lnl(table, cache, f64, precision="fp64")
    l64 = f64[0].cpu().numpy()
    lnl = torch.empty((1, S), dtype=torch.float64, device="cuda")
    err = torch.empty((1, S), dtype=torch.float32, device="cuda")
    bk = dev.MaxKeys(2)
    pcg = dev.pcg_table([dev.pcg64_state(np.random.default_rng(9))])
    ld, cand = dev.cand_words(1, S)
    dev.lnl_fused(table, cache, lnl, err, bk, pcg, cand, ld, chunk=512, early_exit=early_exit)
    v, e = lnl[0].cpu().numpy(), err[0].cpu().numpy()
    out = np.isinf(e)
    print(jitter, early_exit, "samples with an infinite bound", out.mean())
    assert out.mean() > 0.2
    if not early_exit:
        # every epoch evaluated: the stored value is ln L in FP32
        assert np.all(np.abs(v[out] - l64[out]) <= 1e-4 * np.abs(l64[out]) + 100.0)
    # none of them can be kept or be the maximum
    assert np.all(l64[out] < l64.max() - 746.0)
    # an upper bound from the first epochs, or ln L itself in FP32 after the
    # last (whose rounding scales with the cancelling chi2 terms, up to 1e8
    # here, not with ln L)
    assert np.all(v[out] >= l64[out] - 1e-4 * np.abs(l64[out]) - 100.0)
    bits = np.unpackbits(cand[0].cpu().numpy().view(np.uint32).view(np.uint8),
                         bitorder="little")[:S]
    assert not np.any(bits[out])
    keep = ~out
    assert np.all(np.abs(v[keep] - l64[keep]) <= e[keep] + 1e-9 * np.abs(l64[keep]))
