"""Generate tests/golden/kepler_rv_hp.npz: unit-K radial velocities of seeded
Keplerian orbits in 40-digit arithmetic (mpmath), the truth for the FP64
Kepler solver behind joker_rv_from_elements and the FP64 ln L kernels.

Orbits: periods log-uniform in [1, 1e4] d, omega and M0 uniform, e from the
reference's default Beta(0.867, 3.03) prior plus fixed edge values up to
1 - 1e-9 (where the solver's starter and series are stressed).  Times uniform
in [-3000, 3000] d plus t = t0, so M covers many revolutions and the
perihelion neighbourhood.  Each entry also keeps |dm/dM| and |M| so a test can
scale its tolerance by the conditioning of Kepler's equation.

    python tests/golden/make_kepler_golden.py
"""
import os

import mpmath as mp
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _solve(M, e):
    """E with E - e sin E = M (M reduced to [-pi, pi]), by bisection then Newton."""
    twopi = 2 * mp.pi
    Mr = M - twopi * mp.nint(M / twopi)
    sgn = -1 if Mr < 0 else 1
    x = abs(Mr)
    lo, hi = mp.mpf(0), mp.pi
    for _ in range(60):
        mid = (lo + hi) / 2
        if mid - e * mp.sin(mid) - x > 0:
            hi = mid
        else:
            lo = mid
    E = (lo + hi) / 2
    for _ in range(6):
        E = E - (E - e * mp.sin(E) - x) / (1 - e * mp.cos(E))
    return sgn * E


def _m(M, e, om):
    E = _solve(M, e)
    f = 2 * mp.atan2(mp.sqrt(1 + e) * mp.sin(E / 2), mp.sqrt(1 - e) * mp.cos(E / 2))
    return mp.cos(om + f) + e * mp.cos(om)


def main():
    mp.mp.dps = 40
    rng = np.random.default_rng(20240611)
    n_rand, n_t = 48, 40
    edge_e = [0.0, 1e-12, 0.5, 0.9, 0.99, 0.999, 0.9999, 0.99999, 1 - 1e-7, 1 - 1e-9,
              0.3, 0.7, 0.95, 0.995, 0.9995, 0.99995]
    n = n_rand + len(edge_e)
    P = np.exp(rng.uniform(np.log(1.0), np.log(1e4), n))
    K = rng.uniform(0.5, 50.0, n)
    e = np.concatenate([rng.beta(0.867, 3.03, n_rand), edge_e])
    om = rng.uniform(0, 2 * np.pi, n)
    M0 = rng.uniform(0, 2 * np.pi, n)
    t0 = 57000.25
    t = np.concatenate([[t0], t0 + rng.uniform(-3000, 3000, n_t - 1)])
    elems = np.stack([P, K, e, om, M0], axis=1)
    m_hp = np.empty((n, n_t))
    dmdM = np.empty((n, n_t))
    Mabs = np.empty((n, n_t))
    h = mp.mpf(10) ** -18
    for i in range(n):
        Pi, ei, omi, M0i = (mp.mpf(float(v)) for v in (P[i], e[i], om[i], M0[i]))
        for j in range(n_t):
            M = 2 * mp.pi * (mp.mpf(float(t[j])) - mp.mpf(t0)) / Pi - M0i
            m_hp[i, j] = float(_m(M, ei, omi))
            dmdM[i, j] = float(abs((_m(M + h, ei, omi) - _m(M - h, ei, omi)) / (2 * h)))
            Mabs[i, j] = float(abs(M))
    out = os.path.join(HERE, "kepler_rv_hp.npz")
    np.savez_compressed(out, t=t, t0=np.float64(t0), elems=elems, m_hp=m_hp, dmdM=dmdM,
                        Mabs=Mabs)
    print(f"wrote {out}: {n} orbits x {n_t} times")


if __name__ == "__main__":
    main()
