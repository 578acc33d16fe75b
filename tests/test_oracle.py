"""The CPU oracle, pinned against the reference's own outputs (CPU only)."""
import glob
import os

import numpy as np
import pytest

from oracle import oracle, ref_cython


def _cases(golden_dir):
    return sorted(glob.glob(os.path.join(golden_dir, "ref_lnl_*.npz")))


def test_golden_fixtures_present(golden_dir):
    names = {os.path.basename(p) for p in _cases(golden_dir)}
    for case in ("againstpy", "scalevark", "config1", "trend3", "offsets", "jitter"):
        assert f"ref_lnl_{case}.npz" in names


@pytest.mark.parametrize("case", ["againstpy", "scalevark", "config1", "trend3", "offsets",
                                  "jitter"])
def test_c_oracle_matches_reference_cython_outputs(golden_dir, case):
    """joker_oracle.c reproduces CJokerHelper.batch_marginal_ln_likelihood."""
    z = np.load(os.path.join(golden_dir, f"ref_lnl_{case}.npz"))
    lnl = oracle.batch_marginal_ln_likelihood(
        z["t"], z["rv"], z["ivar"], float(z["t_ref"]), z["trend_M"], z["mu"], z["lam"],
        z["chunk"], bool(z["k_prior"][0]), *z["k_prior"][1:], jitter=False)
    ref = z["lnl_ref"]
    assert np.all(np.isfinite(ref))
    # Both follow the same N x N LU algorithm; they differ only in rounding,
    # which the quadratic-trend case (B ill-conditioned) amplifies to ~3e-9.
    rtol = 1e-8 if case == "trend3" else 1e-10
    np.testing.assert_allclose(lnl, ref, rtol=rtol, atol=1e-9)
    # and both sit within that error of the 50-digit value
    hp = z["lnl_hp"]
    np.testing.assert_allclose(lnl[z["idx_hp"]], hp, rtol=rtol, atol=1e-9)
    np.testing.assert_allclose(ref[z["idx_hp"]], hp, rtol=rtol, atol=1e-9)


def test_reference_ignores_jitter(golden_dir):
    """The reference Cython computes the jittered ivar but never reads it
    (fast_likelihood.pyx:458): with s != 0 its output equals the s = 0 result,
    and differs from the jitter-applied NumPy oracle."""
    z = np.load(os.path.join(golden_dir, "ref_lnl_jitter.npz"))
    assert np.any(z["chunk"][:, 4] > 0)
    chunk0 = z["chunk"].copy()
    chunk0[:, 4] = 0.0
    lnl0 = oracle.batch_marginal_ln_likelihood(
        z["t"], z["rv"], z["ivar"], float(z["t_ref"]), z["trend_M"], z["mu"], z["lam"],
        chunk0, True, *z["k_prior"][1:])
    np.testing.assert_allclose(lnl0, z["lnl_ref"], rtol=1e-10)
    assert np.max(np.abs(z["lnl_py_jitter"] - z["lnl_ref"])) > 1.0


def test_py_oracle_agrees_with_c_oracle_with_jitter():
    """Two independent restatements (NumPy py_likelihood.py form and the C
    reference form with jitter applied) agree."""
    rng = np.random.default_rng(7)
    N = 12
    t = np.sort(rng.uniform(0, 500, N)) + 56000
    err = rng.uniform(0.1, 0.5, N)
    rv = 20 * np.sin(t / 9.0) + rng.normal(0, err)
    S = 200
    chunk = np.stack([np.exp(rng.uniform(np.log(2), np.log(1024), S)), rng.beta(0.867, 3.03, S),
                      rng.uniform(0, 2 * np.pi, S), rng.uniform(0, 2 * np.pi, S),
                      np.exp(rng.normal(np.log(0.5), 1, S))], 1)
    lam = np.array([0.0, 100.0 ** 2])
    c = oracle.batch_marginal_ln_likelihood(t, rv, 1 / err ** 2, t.min(), np.ones((N, 1)),
                                            np.zeros(2), lam, chunk, True, 30.0, 365.25, 500.0,
                                            jitter=True)
    p = oracle.py_marginal_ln_likelihood(t, rv, 1 / err ** 2, t.min(), chunk, 1, lam, True, 30.0,
                                         365.25, 500.0)
    np.testing.assert_allclose(c, p, rtol=1e-9)


def test_kepler_known_answer(golden_dir):
    """The oracle's RV model reproduces the reference's noiseless tutorial
    orbit (docs/examples/data.ecsv) with the regenerated true parameters."""
    z = np.load(os.path.join(golden_dir, "kepler_known_answer.npz"))
    chunk = np.array([[z["P"], z["e"], z["omega"], z["M0"], 0.0]])
    col = oracle.rv_unit(z["t"], float(z["t_ref"]), chunk)[0]
    model = float(z["v0"]) + float(z["K"]) * col
    assert np.max(np.abs(model - z["rv"])) < 1e-8
    # the opposite sign of M0 is far off
    chunk[0, 3] = -chunk[0, 3]
    col2 = oracle.rv_unit(z["t"], float(z["t_ref"]), chunk)[0]
    assert np.max(np.abs(float(z["v0"]) + float(z["K"]) * col2 - z["rv"])) > 1.0


@pytest.mark.parametrize("e", [0.0, 1e-6, 0.3, 0.9, 0.99, 0.999])
def test_oracle_kepler_residual(e):
    for M in np.linspace(-20, 20, 97):
        E = oracle.eccentric_anomaly(M, e)
        Mr = np.mod(M + np.pi, 2 * np.pi) - np.pi
        assert abs(E - e * np.sin(E) - Mr) < 1e-13


def test_accept_mask_rule():
    lls = np.array([0.0, -1.0, -50.0, np.log(0.3)])
    uu = np.array([0.999, 0.2, 0.0, 0.31])
    np.testing.assert_array_equal(oracle.accept_mask(lls, uu), [True, True, True, False])


def test_out_of_reach_threshold_rejects_for_every_uniform():
    """The kernels leave a sample without a bound (+inf) once its ln L lies
    more than 746 nats below a lower bound of the maximum: exp(lnL - max)
    then underflows to 0 in FP64, so the rule rejects it for every uniform,
    0 included (numpy's uniforms lie in [0, 1)), while a sample 745 below
    can still be kept with u = 0."""
    d = -746.0 - np.array([0.0, 1e-9, 1.0, 1e3, np.inf])
    assert np.all(np.exp(d) == 0.0)
    lls = np.concatenate([[0.0], d])
    uu = np.zeros(len(lls))
    np.testing.assert_array_equal(oracle.accept_mask(lls, uu), [True] + [False] * len(d))
    assert np.exp(-745.0) > 0.0
    assert oracle.accept_mask(np.array([0.0, -745.0]), np.zeros(2))[1]


@pytest.mark.skipif(not ref_cython.available(), reason="reference Cython module not built here")
def test_reference_module_reproduces_fixture(golden_dir):
    """Re-running the compiled reference gives the committed fixture bit-for-bit."""
    z = np.load(os.path.join(golden_dir, "ref_lnl_offsets.npz"))
    L = len(z["mu"])
    std = np.sqrt(z["lam"])
    h = ref_cython.make_helper(z["t"], z["rv"], z["ivar"], float(z["t_ref"]), z["trend_M"],
                               int(z["poly_trend"]), int(z["n_offsets"]), z["mu"], std,
                               bool(z["k_prior"][0]), *z["k_prior"][1:])
    out = np.array(h.batch_marginal_ln_likelihood(np.ascontiguousarray(z["chunk"][:256])))
    assert L == 4
    np.testing.assert_array_equal(out, z["lnl_ref"][:256])


def _kepler_hp(golden_dir):
    z = np.load(os.path.join(golden_dir, "kepler_rv_hp.npz"))
    # FP64 rounding of the phase (|M| ulps) carried through dm/dM, plus the
    # result's own rounding: the conditioning of the RV model
    scale = 2.0 ** -52 * (1.0 + z["dmdM"] * (z["Mabs"] + 1.0))
    return z, scale


def test_oracle_rv_matches_40_digit_values(golden_dir):
    """The C oracle's Kepler solve and unit RV against 40-digit values
    (tests/golden/make_kepler_golden.py), e up to 1 - 1e-9."""
    z, scale = _kepler_hp(golden_dir)
    el = z["elems"]
    chunk = np.stack([el[:, 0], el[:, 2], el[:, 3], el[:, 4], np.zeros(len(el))], axis=1)
    m = oracle.rv_unit(z["t"], float(z["t0"]), chunk)
    assert np.all(np.abs(m - z["m_hp"]) <= 8.0 * scale)


def test_sincos_table_is_correctly_rounded():
    """The committed table of the FP64 Kepler solver
    (thejoker_gb300/csrc/joker_sincos_table.cuh, written by
    gen_sincos_table.py): sin and cos of k/128 within an ulp of numpy's."""
    import re
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                        "thejoker_gb300", "csrc", "joker_sincos_table.cuh")
    text = open(path).read()
    pairs = re.findall(r"\{(-?0x[0-9a-fp.+-]+), (-?0x[0-9a-fp.+-]+)\},", text)
    assert len(pairs) == 404
    for k, (s, c) in enumerate(pairs):
        a = k / 128.0
        for got, want in ((float.fromhex(s), np.sin(a)), (float.fromhex(c), np.cos(a))):
            assert abs(got - want) <= np.spacing(abs(want)) + 1e-300
