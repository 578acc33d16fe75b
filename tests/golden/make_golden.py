"""Generate the golden fixtures in tests/golden/ (run in a checkout that has
the reference project and Cython; the fixtures are committed).

* kepler_known_answer.npz -- the reference's tutorial dataset
  docs/examples/data.ecsv (noiseless RVs of a twobody KeplerOrbit, written by
  docs/examples/make-data.ipynb from default_rng(123)) with the orbit's true
  parameters regenerated from the same seed.  It pins the Kepler/RV sign
  convention: M = 2 pi (t - t_ref)/P - M0, rv = v0 + K (cos(w + f) + e cos w).
* ref_lnl_<case>.npz -- inputs and outputs of the reference's own Cython
  CJokerHelper.batch_marginal_ln_likelihood (thejoker/src/fast_likelihood.pyx),
  compiled unmodified by oracle/build.py, on seeded synthetic stars, plus
  50-digit (mpmath) values ``lnl_hp`` at the rows ``idx_hp``: the reference's
  own FP64 error reaches a few 1e-9 relative when a quadratic trend makes B
  ill-conditioned, so the truth is kept beside it.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

# the reference checkout: JOKER_REFERENCE_ROOT, else where this container mounts it
REFERENCE_ROOT = os.environ.get("JOKER_REFERENCE_ROOT", "/root/reference")
DATA_ECSV = os.path.join(REFERENCE_ROOT, "docs", "examples", "data.ecsv")


def kepler_known_answer():
    rnd = np.random.default_rng(seed=123)
    rnd.uniform(0.0, 40)                     # t0 offset (cell 2 of make-data.ipynb)
    P = rnd.uniform(40, 80)
    M0 = rnd.uniform(0.0, 2 * np.pi)
    omega = rnd.uniform(0.0, 2 * np.pi)
    e = 0.1
    K = rnd.uniform(5, 15)
    v0 = rnd.uniform(-50, 50)
    rows = [l.split() for l in open(DATA_ECSV) if not l.startswith("#")][1:]
    arr = np.array([[float(v) for v in r] for r in rows])
    bjd, rv, err = arr[:, 0], arr[:, 1], arr[:, 2]
    t = bjd - 2400000.5                      # BMJD
    np.savez(os.path.join(HERE, "kepler_known_answer.npz"), t=t, rv=rv, rv_err=err,
             t_ref=t.min(), P=P, M0=M0, omega=omega, e=e, K=K, v0=v0)


def _chunk(rng, S, P_min, P_max, s_kind="zero"):
    P = np.exp(rng.uniform(np.log(P_min), np.log(P_max), S))
    e = rng.beta(0.867, 3.03, S)
    om = rng.uniform(0, 2 * np.pi, S)
    M0 = rng.uniform(0, 2 * np.pi, S)
    if s_kind == "zero":
        s = np.zeros(S)
    else:
        s = np.exp(rng.normal(np.log(0.5), 1.0, S))
    return np.ascontiguousarray(np.stack([P, e, om, M0, s], 1))


CASES = {
    # (n_epochs, baseline, sig range, poly_trend, n_offsets, K prior, S, P range, s, seed)
    "againstpy": dict(N=3, base=250.0, sig=(0.1, 0.2), poly=1, noff=0, kp=("normal", 10.0),
                      sigma_v=[100.0], S=2048, P=(8, 32768), s="zero", seed=42, t0=56831.324,
                      signal="cos"),
    "scalevark": dict(N=3, base=250.0, sig=(0.1, 0.2), poly=1, noff=0, kp=("scaled", 25.0),
                      sigma_v=[100.0], S=2048, P=(8, 32768), s="zero", seed=42, t0=56831.324,
                      signal="cos"),
    "config1": dict(N=16, base=1000.0, sig=(0.1, 1.0), poly=1, noff=0, kp=("scaled", 30.0),
                    sigma_v=[100.0], S=4096, P=(2, 1024), s="zero", seed=0, t0=2456000.0,
                    signal="kepler"),
    "trend3": dict(N=24, base=2000.0, sig=(0.1, 1.0), poly=3, noff=0, kp=("scaled", 30.0),
                   sigma_v=[100.0, 1.0, 0.01], S=2048, P=(2, 1024), s="zero", seed=4,
                   t0=2456000.0, signal="kepler"),
    "offsets": dict(N=20, base=800.0, sig=(0.1, 0.5), poly=2, noff=1, kp=("scaled", 30.0),
                    sigma_v=[100.0, 0.5], S=2048, P=(2, 1024), s="zero", seed=5, t0=2456000.0,
                    signal="kepler"),
    "jitter": dict(N=40, base=3000.0, sig=(0.05, 0.5), poly=1, noff=0, kp=("scaled", 30.0),
                   sigma_v=[100.0], S=2048, P=(2, 1024), s="lognormal", seed=2,
                   t0=2456000.0, signal="kepler"),
}


def make_star(c, rng):
    from thejoker_gb300.linear import rv_unit_columns
    N = c["N"]
    t = np.sort(rng.uniform(0, c["base"], N)) + c["t0"]
    err = rng.uniform(*c["sig"], N)
    if c["signal"] == "cos":
        rv = np.cos(t)
    else:
        P, e = np.exp(rng.uniform(np.log(2), np.log(1024))), rng.beta(0.867, 3.03)
        om, M0 = rng.uniform(0, 2 * np.pi), rng.uniform(0, 2 * np.pi)
        K = rng.uniform(1, 50)
        rv = K * rv_unit_columns(t, t.min(), [P], [e], [om], [M0])[0] + rng.normal(0, 10) \
            + rng.normal(0, err)
    ids = np.zeros(N, dtype=int)
    if c["noff"]:
        ids[rng.permutation(N)[: N // 2]] = 1
        rv = rv + 4.8 * (ids == 1)
    dt = t - t.min()
    const = np.zeros((N, 1 + c["noff"]))
    const[:, 0] = 1.0
    for j in range(c["noff"]):
        const[ids == j + 1, j + 1] = 1.0
    trend = np.hstack([const, np.vander(dt, N=c["poly"], increasing=True)[:, 1:]])
    L = 1 + c["poly"] + c["noff"]
    mu = np.zeros(L)
    std = np.zeros(L)
    std[1] = c["sigma_v"][0]
    for j in range(c["noff"]):
        std[2 + j] = 2.0
    for j in range(1, c["poly"]):
        std[1 + c["noff"] + j] = c["sigma_v"][j]
    if c["kp"][0] == "normal":
        std[0] = c["kp"][1]
        kprior = np.array([0.0, 0.0, 0.0, 0.0])
    else:
        kprior = np.array([1.0, c["kp"][1], 365.25, 500.0])
    return t, rv, 1 / err ** 2, trend, mu, std, kprior


def hp_lnl(t, rv, ivar, t0, trend, mu, lam, kp, chunk, idx):
    """ln L in 50-digit arithmetic (determinant lemma + Woodbury form)."""
    from mpmath import mp
    from oracle import oracle
    mp.dps = 50
    cols = oracle.rv_unit(t, t0, chunk[idx])
    L = len(mu)
    out = []
    for k, n in enumerate(idx):
        P, e = chunk[n, 0], chunk[n, 1]
        lam_n = np.array(lam, dtype=np.float64)
        if kp[0]:
            lam_n[0] = min(kp[3] ** 2, kp[1] ** 2 / (1 - e ** 2) * (P / kp[2]) ** (-2 / 3))
        G = mp.matrix(L, L)
        q = mp.matrix(L, 1)
        rWr = mp.mpf(0)
        for i in range(len(t)):
            x = [mp.mpf(cols[k][i])] + [mp.mpf(trend[i, j]) for j in range(L - 1)]
            w = mp.mpf(ivar[i])
            r = mp.mpf(rv[i]) - sum(mp.mpf(mu[a]) * x[a] for a in range(L))
            rWr += w * r * r
            for a in range(L):
                q[a] += w * x[a] * r
                for b in range(L):
                    G[a, b] += w * x[a] * x[b]
        for a in range(L):
            G[a, a] += 1 / mp.mpf(lam_n[a])
        quad = (q.T * mp.inverse(G) * q)[0]
        ld = (len(t) * mp.log(2 * mp.pi) - sum(mp.log(mp.mpf(w)) for w in ivar)
              + sum(mp.log(mp.mpf(v)) for v in lam_n) + mp.log(mp.det(G)))
        out.append(float(-(rWr - quad + ld) / 2))
    return np.array(out)


def ref_cases():
    from oracle import oracle, ref_cython
    for name, c in CASES.items():
        rng = np.random.default_rng(c["seed"])
        t, rv, ivar, trend, mu, std, kprior = make_star(c, rng)
        chunk = _chunk(rng, c["S"], *c["P"], s_kind=c["s"])
        h = ref_cython.make_helper(t, rv, ivar, t.min(), trend, c["poly"], c["noff"], mu, std,
                                   bool(kprior[0]), kprior[1], kprior[2], kprior[3])
        lnl_ref = np.array(h.batch_marginal_ln_likelihood(chunk))
        lam = std ** 2
        idx_hp = np.unique(np.concatenate([np.arange(32), np.argsort(lnl_ref)[-16:]]))
        extra = {"idx_hp": idx_hp,
                 "lnl_hp": hp_lnl(t, rv, ivar, t.min(), trend, mu, lam, kprior, chunk, idx_hp)}
        if c["s"] != "zero":
            extra["lnl_py_jitter"] = oracle.batch_marginal_ln_likelihood(
                t, rv, ivar, t.min(), trend, mu, lam, chunk, bool(kprior[0]), kprior[1],
                kprior[2], kprior[3], jitter=True)
        np.savez(os.path.join(HERE, f"ref_lnl_{name}.npz"), t=t, rv=rv, ivar=ivar,
                 t_ref=t.min(), trend_M=trend, mu=mu, lam=lam, k_prior=kprior,
                 poly_trend=c["poly"], n_offsets=c["noff"], chunk=chunk, lnl_ref=lnl_ref,
                 **extra)
        print(name, lnl_ref.min(), lnl_ref.max())


def degenerate_cases():
    """ref_lnl_degenerate.npz: the reference's own output on degenerate
    designs -- an infinite prior variance on an offset column that duplicates
    the constant one, zero errors at most epochs, an infinite v0 variance --
    where its LU-failure branches (fast_likelihood.pyx:283-291, 347-348,
    381-382) would apply.  Each case stores its star and the reference's
    ln L of 16 prior samples."""
    from oracle import ref_cython
    rng = np.random.default_rng(0)
    N = 8
    t = np.sort(rng.uniform(0, 500, N)) + 56000
    err = rng.uniform(0.2, 0.5, N)
    rv = rng.normal(0, 2, N)
    chunk = _chunk(rng, 16, 2.0, 1024.0)
    e0 = err.copy()
    e0[:6] = 0.0
    with np.errstate(divide="ignore"):
        iv0 = 1 / e0 ** 2
    cases = {
        "dup_offset_inf_var": (1 / err ** 2, np.ones((N, 2)), 1, 1, [0, 0, 0], [0, 100.0, np.inf]),
        "zero_errors": (iv0, np.ones((N, 1)), 1, 0, [0, 0], [0, 100.0]),
        "inf_v0_var": (1 / err ** 2, np.ones((N, 1)), 1, 0, [0, 0], [0, np.inf]),
    }
    out = {"t": t, "rv": rv, "chunk": chunk}
    for name, (ivar, trend, poly, noff, mu, std) in cases.items():
        h = ref_cython.make_helper(t, rv, ivar, t.min(), trend, poly, noff, mu, std, True, 30.0,
                                   365.25, 500.0)
        out[f"{name}_ivar"] = ivar
        out[f"{name}_trend_M"] = trend
        out[f"{name}_mu"] = np.asarray(mu, dtype=float)
        out[f"{name}_lam"] = np.asarray(std, dtype=float) ** 2
        out[f"{name}_lnl_ref"] = np.array(h.batch_marginal_ln_likelihood(chunk))
        print(name, out[f"{name}_lnl_ref"][:4])
    np.savez(os.path.join(HERE, "ref_lnl_degenerate.npz"), **out)


if __name__ == "__main__":
    from oracle import build
    build.build_all()
    kepler_known_answer()
    ref_cases()
    degenerate_cases()
