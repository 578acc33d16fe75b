"""The FP64 Kepler solver and unit RV model (GB300 only), through
joker_rv_from_elements, the device counterpart of twobody's
c_rv_from_elements (thejoker/src/fast_likelihood.pyx:27-30, 453-455): the ln L
kernels, the acceptance refinement and the posterior share this arithmetic.

The bound is the conditioning of the RV model: FP64 rounding of the phase
(a few ulps of |M|) carried through |dm/dM|, plus a few ulps of the result."""
import os

import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu


def _scale(dmdM, Mabs):
    return 2.0 ** -52 * (1.0 + dmdM * (Mabs + 1.0))


def test_rv_matches_40_digit_values(cuda, golden_dir):
    from thejoker_gb300 import device as dev
    z = np.load(os.path.join(golden_dir, "kepler_rv_hp.npz"))
    el = z["elems"]
    rv = dev.rv_from_elements(z["t"], el, float(z["t0"])).cpu().numpy()
    K = el[:, 1:2]
    err = np.abs(rv - K * z["m_hp"])
    ratio = err / (K * _scale(z["dmdM"], z["Mabs"]))
    assert ratio.max() <= 8.0, f"worst {ratio.max():.2f} conditioning units"


def _ecc_anomaly(M, e):
    """E of Kepler's equation, vectorised FP64 Newton with a bisection
    safeguard (only for the tolerance's conditioning factor)."""
    Mr = np.remainder(M + np.pi, 2 * np.pi) - np.pi
    x = np.abs(Mr)
    lo, hi = x.copy(), np.minimum(np.pi, x + e)
    E = np.where(e > 0.8, hi, np.clip(x + e * np.sin(x), lo, hi))
    for _ in range(80):
        f = E - e * np.sin(E) - x
        lo = np.where(f < 0, E, lo)
        hi = np.where(f > 0, E, hi)
        En = E - f / (1 - e * np.cos(E))
        E = np.where((En > lo) & (En < hi), En, 0.5 * (lo + hi))
    return np.sign(Mr) * E


def _dmdM(M, e, om):
    """|dm/dM| of m = (A cos E + B sin E - D)/(1 - e cos E) + D."""
    E = _ecc_anomaly(M, e)
    A, B, D = np.cos(om), -np.sin(om) * np.sqrt((1 - e) * (1 + e)), e * np.cos(om)
    c, s = np.cos(E), np.sin(E)
    den = 1 - e * c
    dm_dE = ((-A * s + B * c) * den - (A * c + B * s - D) * (e * s)) / den ** 2
    return np.abs(dm_dE / den)


def test_rv_matches_oracle_near_perihelion(cuda):
    """Eccentricities up to 1 - 1e-9 and times clustered at perihelion
    passages (M near 0 mod 2 pi), where Kepler's equation is hardest."""
    from thejoker_gb300 import device as dev
    rng = np.random.default_rng(11)
    n, n_t, t0 = 4096, 48, 0.0
    e = np.concatenate([rng.beta(0.867, 3.03, n // 2), 1.0 - 10.0 ** rng.uniform(-9, 0, n // 2)])
    rng.shuffle(e)
    el = np.stack([np.exp(rng.uniform(np.log(1.5), np.log(5000.0), n)), np.ones(n), e,
                   rng.uniform(0, 2 * np.pi, n), rng.uniform(0, 2 * np.pi, n)], axis=1)
    worst = 0.0
    for i0 in range(0, n, 512):
        blk = el[i0:i0 + 512]
        # times shared by the block: perihelion passages of its first orbit
        # (to within 1e-4 periods) and uniform times
        P0, M00 = blk[0, 0], blk[0, 4]
        k = rng.integers(-200, 200, n_t // 2)
        tp = (M00 / (2 * np.pi) + k + rng.uniform(-1e-4, 1e-4, n_t // 2)) * P0
        t = np.concatenate([tp, rng.uniform(-2000, 2000, n_t - n_t // 2)])
        rv = dev.rv_from_elements(t, blk, t0).cpu().numpy()
        chunk = np.stack([blk[:, 0], blk[:, 2], blk[:, 3], blk[:, 4], np.zeros(len(blk))], 1)
        ref = oracle.rv_unit(t, t0, chunk)
        M = 2 * np.pi * (t[None, :] - t0) / blk[:, :1] - blk[:, 4:5]
        scale = _scale(_dmdM(M, blk[:, 2:3], blk[:, 3:4]), np.abs(M))
        worst = max(worst, float((np.abs(rv - ref) / scale).max()))
    # each side within 8 conditioning units of the truth
    assert worst <= 16.0, f"worst {worst:.2f} conditioning units"


def test_rv_edge_inputs(cuda):
    from thejoker_gb300 import device as dev
    from thejoker_gb300._native import JokerError
    # t = t0 and M0 = 0: M = 0 exactly, E = f = 0, m = (1 + e) cos(omega).
    # The eccentric-anomaly form (A cos E - D)/(1 - e cos E) + D divides a
    # difference of O(1) terms by 1 - e, so its rounding grows like 1/(1 - e)
    el = np.array([[10.0, 2.0, 0.0, 0.3, 0.0], [10.0, 2.0, 0.6, 0.3, 0.0],
                   [10.0, 2.0, 0.999, 0.3, 0.0], [10.0, 2.0, 1 - 1e-9, 0.3, 0.0]])
    rv = dev.rv_from_elements(np.array([5.0]), el, 5.0).cpu().numpy()[:, 0]
    want = 2.0 * (1 + el[:, 2]) * np.cos(0.3)
    assert np.all(np.abs(rv - want) <= 8 * 2.0 ** -52 * 2.0 / (1 - el[:, 2]))
    # empty inputs are no-ops; bad shapes and negative sizes are errors
    assert dev.rv_from_elements(np.zeros(0), el).shape == (len(el), 0)
    with pytest.raises(ValueError):
        dev.rv_from_elements(np.zeros(3), np.zeros((2, 4)))
    from thejoker_gb300 import _native as nat
    with pytest.raises(JokerError):
        nat.check(nat.lib().joker_rv_from_elements(None, -1, None, 1, 0.0, None, None),
                  "joker_rv_from_elements")


def test_launch_counter(cuda):
    """joker_launch_count counts the library's kernel launches on the host."""
    from thejoker_gb300 import _native as nat
    from thejoker_gb300 import device as dev
    el = np.array([[10.0, 2.0, 0.3, 0.3, 0.0]])
    c0 = nat.lib().joker_launch_count()
    dev.rv_from_elements(np.linspace(0, 5, 7), el)
    assert nat.lib().joker_launch_count() - c0 == 1
    dev.rv_from_elements(np.zeros(0), el)                       # empty: no launch
    assert nat.lib().joker_launch_count() - c0 == 1
