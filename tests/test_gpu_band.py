"""The mixed path's error bound in its worst regimes, and the band
refinement that brings every ln L near the maximum within 1e-4 of FP64
(GB300 only).

The per-sample bound err of the mixed kernels is built from stated terms
(the FP32 column error amplified near pericentre, the float-float rounding
of the sums, the FP32 weights with the jitter applied) whose constants were
fitted on test cases, not derived as a rounding-error bound.  These tests
sweep the regimes where it is tightest at once: many epochs, the jitter
applied, three linear parameters, eccentricities up to 0.9999, periods down
to 2 d over baselines of thousands of days.  Each sample's |lnL_mixed -
lnL_FP64| must stay within its bound, and after joker_refine_band every
value within JOKER_MIXED_LNL_BAND (40) of the maximum must be within
JOKER_MIXED_LNL_TOL (1e-4) of FP64.  The 4096-star survey is checked star by
star: the refined mixed acceptance keeps exactly the FP64 path's samples.
"""
import numpy as np
import pytest
import torch

from gpu_util import synth_chunk, synth_star

pytestmark = pytest.mark.gpu

BAND, TOL = 40.0, 1e-4


def _hard_chunk(rng, S, jitter):
    """Prior samples with a quarter at eccentricities 0.99-0.9999 and a
    quarter at periods 2-3 d."""
    c = synth_chunk(rng, S, jitter=jitter)
    q = S // 4
    c[:q, 1] = 1 - 10 ** rng.uniform(-4, -2, q)
    c[q:2 * q, 0] = rng.uniform(2.0, 3.0, q)
    return c


def _both(table, cache, S, precision="mixed"):
    from thejoker_gb300 import device as dev
    l64 = torch.empty((1, S), dtype=torch.float64, device="cuda")
    dev.lnl(table, cache, l64, precision="fp64")
    lm = torch.empty((1, S), dtype=torch.float64, device="cuda")
    err = torch.empty((1, S), dtype=torch.float32, device="cuda")
    bk = dev.MaxKeys(2)
    dev.lnl(table, cache, lm, precision=precision, err=err, bound_keys=bk)
    return l64, lm, err, bk


@pytest.mark.parametrize("N,poly,jitter,base", [(256, 2, "applied", 4000.0),
                                                (256, 1, "applied", 4000.0),
                                                (200, 2, "reference", 3000.0),
                                                (64, 3, "reference", 4000.0),
                                                (5, 1, "applied", 300.0)])
@pytest.mark.parametrize("precision", ["mixed", "mixed_fast"])
def test_bound_holds_and_band_meets_tolerance(cuda, N, poly, jitter, base, precision):
    from thejoker_gb300 import device as dev
    rng = np.random.default_rng(1000 + N + poly)
    st = synth_star(rng, N, base=base, sig=(0.05, 0.5), K=25.0, poly=poly)
    S = 1 << 18
    chunk = _hard_chunk(rng, S, jitter == "applied")
    table = dev.StarTable([st], jitter=jitter)
    cache = dev.PriorCache.from_samples(chunk)
    l64, lm, err, bk = _both(table, cache, S, precision)
    a64 = l64[0].cpu().numpy()
    am = lm[0].cpu().numpy()
    ev = err[0].cpu().numpy()
    fin = np.isfinite(a64)
    assert fin.mean() > 0.99
    d = np.abs(am - a64)
    # the bound holds for every sample (it is stated against the FP64 path)
    assert np.all(d[fin] <= ev[fin]), f"max |d|/err = {np.max(d[fin] / ev[fin]):.3f}"
    seg = [dict(lnl_off=0, n=S, out_off=0, max_out=0, max_slot=0, star=0, row0=0)]
    exact, n1 = dev.refine_max(table, cache, lm.view(-1), err.view(-1), bk, seg)
    mx = np.nanmax(a64)
    # the refinement's FP64 (one warp per sample) and the FP64 kernel (one
    # thread per sample) sum the epochs in different orders
    assert abs(exact.values()[0] - mx) <= 1e-9 * max(1.0, abs(mx))
    n2 = dev.refine_band(table, cache, lm.view(-1), err.view(-1), exact, seg)
    ab = lm[0].cpu().numpy()
    band = fin & (a64 >= mx - BAND)
    assert np.max(np.abs(ab - a64)[band]) <= TOL
    # values the band refinement re-evaluated are the FP64 values
    eb = err[0].cpu().numpy()
    redone = (eb == 0) & fin
    np.testing.assert_allclose(ab[redone], a64[redone], rtol=1e-9, atol=1e-9)
    # below the band the values keep their mixed bound
    assert np.all(np.abs(ab - a64)[fin & ~band] <= ev[fin & ~band])
    assert int(n2.item()) <= S


def test_helper_mixed_marginal_ln_likelihood_within_tolerance(cuda):
    """GPUJokerHelper(precision="mixed").batch_marginal_ln_likelihood returns
    band-refined values: within 1e-4 of the FP64 helper near the maximum."""
    from thejoker_gb300 import JokerPrior, RVData
    from thejoker_gb300.data import get_trend_design_matrix
    from thejoker_gb300.helper import GPUJokerHelper
    rng = np.random.default_rng(77)
    st = synth_star(rng, 40, base=3000.0, sig=(0.05, 0.5), K=30.0)
    prior = JokerPrior.default(P_min=2, P_max=1024, sigma_K0=30.0, sigma_v=100.0)
    data = RVData(st["t"], st["rv"], 1 / np.sqrt(st["ivar"]))
    trend = get_trend_design_matrix(data, None, 1)
    chunk = _hard_chunk(rng, 1 << 17, False)
    h64 = GPUJokerHelper(data, prior, trend, precision="fp64")
    hm = GPUJokerHelper(data, prior, trend, precision="mixed")
    a = h64.batch_marginal_ln_likelihood(chunk)
    b = hm.batch_marginal_ln_likelihood(chunk)
    band = a >= np.nanmax(a) - BAND
    assert band.sum() >= 1
    assert np.max(np.abs(a - b)[band]) <= TOL


@pytest.mark.parametrize("precision", ["mixed", "mixed_fast"])
def test_refined_accept_equals_fp64_on_the_4096_star_survey(cuda, precision):
    """The batched configuration (4096 stars, epochs log-uniform [3, 256], 30%
    with companions) over a 2^17-sample prior cache: for every star the
    refined mixed acceptance keeps exactly the FP64 path's indices, and every
    kept ln L is within 1e-4 of FP64."""
    from thejoker_gb300 import device as dev
    from thejoker_gb300.batch import BatchRejection
    from thejoker_gb300.synthetic import fill_prior_cache, survey_stars
    stars = survey_stars(4096, seed=3)
    S = 1 << 17
    cache = dev.PriorCache.from_samples(fill_prior_cache(np.empty((S, 5)), 0))
    table = dev.StarTable(stars)
    res = {}
    for prec in ("fp64", precision):
        b = BatchRejection(table, cache, precision=prec, max_out=512, seeds=np.arange(4096))
        b.run()
        res[prec] = b.results()
    c64, i64, l64 = res["fp64"]
    cm, im, lm = res[precision]
    np.testing.assert_array_equal(c64, cm)
    for k in range(4096):
        np.testing.assert_array_equal(i64[k], im[k])
        if len(lm[k]):
            assert np.max(np.abs(lm[k] - l64[k])) <= TOL
