"""Priors of The Joker, restated with NumPy distributions.

The reference builds its priors from pymc random variables
(thejoker/prior.py:40-575, thejoker/distributions.py).  The likelihood path
only needs the numbers CJokerHelper extracts from them
(fast_likelihood.pyx:202-253): the means / variances of the Gaussian linear
parameters and, for the FixedCompanionMass K prior, sigma_K0, P0 and max_K.
This module keeps those numbers and draws prior samples with NumPy from the
same distributions:

* P ~ log-uniform(P_min, P_max)            UniformLog, distributions.py:19-28
* e ~ Beta(0.867, 3.03)                    Kipping13Global, distributions.py:171-176
* omega, M0 ~ U(0, 2 pi)                   pymc_ext angle
* s = constant (default 0) or a given distribution
* K ~ N(mu_K, sigma_K), sigma_K = sigma_K0 (P/P0)^(-1/3) / sqrt(1 - e^2),
  clipped at max_K                          FixedCompanionMass, distributions.py:103-152
* v_i ~ N(0, sigma_v[i]);  offsets ~ N(mu, sigma)

Units are fixed: days, radians and the data's velocity unit (km/s by
default).  P0 defaults to one Julian year, 365.25 d.
"""
import numpy as np

__all__ = ["JokerPrior", "LogUniform", "Beta", "UniformAngle", "Fixed", "LogNormal",
           "Normal", "FixedCompanionMass", "validate_poly_trend", "validate_n_offsets"]


class LogUniform:
    def __init__(self, a, b):
        if not (0 < a < b):
            raise ValueError("a > 0 and a < b")
        self.a, self.b = float(a), float(b)

    def draw(self, rng, size):
        # UniformLogRV.rng_fn, distributions.py:24-28
        fac = np.log(self.b) - np.log(self.a)
        return np.exp(rng.uniform(size=size) * fac + np.log(self.a))

    def logp(self, x):
        return -np.log(x) - np.log(np.log(self.b) - np.log(self.a))


class Beta:
    def __init__(self, alpha, beta):
        self.alpha, self.beta = float(alpha), float(beta)

    def draw(self, rng, size):
        return rng.beta(self.alpha, self.beta, size=size)


class UniformAngle:
    def draw(self, rng, size):
        return rng.uniform(0.0, 2 * np.pi, size=size)


class Fixed:
    def __init__(self, value):
        self.value = float(value)

    def draw(self, rng, size):
        return np.full(size, self.value)


class LogNormal:
    """ln s ~ N(mu, sigma)."""

    def __init__(self, mu, sigma):
        self.mu, self.sigma = float(mu), float(sigma)

    def draw(self, rng, size):
        return np.exp(rng.normal(self.mu, self.sigma, size=size))


class Normal:
    def __init__(self, mu, sigma):
        self.mu, self.sigma = float(mu), float(sigma)

    def draw(self, rng, size):
        return rng.normal(self.mu, self.sigma, size=size)


class FixedCompanionMass:
    """K prior whose width scales with P and e (distributions.py:103-152)."""

    def __init__(self, sigma_K0, P0=365.25, mu=0.0, max_K=500.0):
        self.sigma_K0, self.P0, self.mu, self.max_K = map(float, (sigma_K0, P0, mu, max_K))

    def sigma(self, P, e):
        s = self.sigma_K0 * (P / self.P0) ** (-1 / 3) / np.sqrt(1 - e ** 2)
        return np.clip(s, 0.0, self.max_K)


def validate_poly_trend(poly_trend):
    try:
        poly_trend = int(poly_trend)
    except Exception as exc:
        raise ValueError("poly_trend must be an integer that specifies the number of "
                         "polynomial (in time) trend terms to include in The Joker.") from exc
    return poly_trend, [f"v{i}" for i in range(poly_trend)]


def validate_n_offsets(n_offsets):
    try:
        n_offsets = int(n_offsets)
    except Exception as exc:
        raise ValueError("n_offsets must be an integer") from exc
    return n_offsets, [f"dv0_{i}" for i in range(1, n_offsets + 1)]


class JokerPrior:
    """Prior over The Joker's parameters (thejoker/prior.py:40-178).

    ``pars`` maps parameter names to distribution objects of this module.
    ``v0_offsets`` is a list of (name, Normal) pairs.
    """

    def __init__(self, pars, poly_trend=1, v0_offsets=None):
        self.poly_trend, self._v_trend_names = validate_poly_trend(poly_trend)
        self.v0_offsets = list(v0_offsets or [])
        self.pars = dict(pars)
        for name, dist in self.v0_offsets:
            self.pars[name] = dist
        self._nonlinear_names = ["P", "e", "omega", "M0", "s"]
        self._linear_names = ["K"] + self._v_trend_names
        self._offset_names = [n for n, _ in self.v0_offsets]
        for name in self.par_names:
            if name not in self.pars:
                raise ValueError(f"Missing prior for parameter '{name}': you must specify a "
                                 "prior distribution for all parameters.")
        for name in self._linear_names + self._offset_names:
            if not isinstance(self.pars[name], (Normal, FixedCompanionMass)):
                raise ValueError("Priors on the linear parameters (K, v0, etc.) must be "
                                 f"independent Normal distributions (for {name})")

    @classmethod
    def default(cls, P_min=None, P_max=None, sigma_K0=None, P0=365.25, sigma_v=None, s=None,
                poly_trend=1, v0_offsets=None, pars=None, max_K=500.0):
        """The default prior (prior.py:180-268)."""
        pars = dict(pars or {})
        poly_trend, v_names = validate_poly_trend(poly_trend)
        out = {}
        if "P" not in pars:
            if P_min is None or P_max is None:
                raise ValueError("If you are using the default period prior, you must pass in "
                                 "both P_min and P_max to set the period prior domain.")
            out["P"] = LogUniform(P_min, P_max)
        out.setdefault("e", Beta(0.867, 3.03))
        out.setdefault("omega", UniformAngle())
        out.setdefault("M0", UniformAngle())
        if "s" not in pars:
            out["s"] = s if hasattr(s, "draw") else Fixed(0.0 if s is None else s)
        if "K" not in pars:
            if sigma_K0 is None or P0 is None:
                raise ValueError("If using the default prior form on K, you must pass in a "
                                 "variance scale (sigma_K0) and a reference period (P0)")
            out["K"] = FixedCompanionMass(sigma_K0, P0, max_K=max_K)
        if v_names and "v0" not in pars:
            if np.ndim(sigma_v) == 0:
                if poly_trend != 1 and sigma_v is not None:
                    raise ValueError("You must pass in a single sigma value for each velocity "
                                     f"trend parameter: poly_trend={poly_trend}")
                sigma_v = {"v0": sigma_v}
            elif not hasattr(sigma_v, "keys"):
                if len(sigma_v) != poly_trend:
                    raise ValueError("You must pass in a single sigma value for each velocity "
                                     f"trend parameter: You passed in {len(sigma_v)} values, "
                                     f"but poly_trend={poly_trend}")
                sigma_v = dict(zip(v_names, sigma_v))
            for name in v_names:
                if sigma_v.get(name) is None:
                    raise ValueError(f"sigma_v is required for {name}")
                out[name] = Normal(0.0, sigma_v[name])
        out.update(pars)
        return cls(out, poly_trend=poly_trend, v0_offsets=v0_offsets)

    @property
    def par_names(self):
        return self._nonlinear_names + self._linear_names + self._offset_names

    @property
    def n_offsets(self):
        return len(self.v0_offsets)

    @property
    def n_linear(self):
        return 1 + self.poly_trend + self.n_offsets

    def linear_prior_arrays(self):
        """mu, Lambda (variances) and the K-prior numbers in CJokerHelper's
        index order K, v0, offsets..., v1, ... (fast_likelihood.pyx:202-253).

        Returns (mu, lam, k_prior) with k_prior = [scaled, sigma_K0, P0, max_K].
        """
        L = self.n_linear
        mu = np.zeros(L)
        lam = np.zeros(L)
        K = self.pars["K"]
        if isinstance(K, FixedCompanionMass):
            k_prior = np.array([1.0, K.sigma_K0, K.P0, K.max_K])
            mu[0] = K.mu
        else:
            k_prior = np.array([0.0, 0.0, 0.0, 0.0])
            mu[0], lam[0] = K.mu, K.sigma ** 2
        order = (["v0"] if self.poly_trend >= 1 else []) + self._offset_names + \
            self._v_trend_names[1:]
        for i, name in enumerate(order):
            d = self.pars[name]
            mu[1 + i], lam[1 + i] = d.mu, d.sigma ** 2
        return mu, lam, k_prior

    def sample(self, size=1, generate_linear=False, return_logprobs=False, rng=None,
               dtype=np.float64, **kwargs):
        """Random samples from the prior as a JokerSamples (prior.py:297-407)."""
        from .samples import JokerSamples
        if rng is None:
            rng = np.random.default_rng()
        size = int(size)
        cols = {}
        for name in self._nonlinear_names:
            cols[name] = self.pars[name].draw(rng, size).astype(dtype)
        if generate_linear:
            K = self.pars["K"]
            if isinstance(K, FixedCompanionMass):
                cols["K"] = rng.normal(K.mu, K.sigma(cols["P"], cols["e"])).astype(dtype)
            else:
                cols["K"] = K.draw(rng, size).astype(dtype)
            for name in self._v_trend_names + self._offset_names:
                cols[name] = self.pars[name].draw(rng, size).astype(dtype)
        out = JokerSamples(poly_trend=self.poly_trend, n_offsets=self.n_offsets, **kwargs)
        for k, v in cols.items():
            out[k] = v
        if return_logprobs:
            P = self.pars["P"]
            out["ln_prior"] = P.logp(cols["P"]) if hasattr(P, "logp") else np.zeros(size)
        return out

    def __repr__(self):
        return f'<JokerPrior [{", ".join(self.par_names)}]>'
