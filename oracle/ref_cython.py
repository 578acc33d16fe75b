"""Loader for the reference's own compiled Cython likelihood (test infrastructure).

``oracle/build.py`` compiles thejoker/src/fast_likelihood.pyx unmodified into
``oracle/_ref``.  Loading it needs import-time stand-ins for astropy.units,
thejoker.units, thejoker.utils and thejoker.distributions (``oracle/ref_stubs``)
and duck-typed ``data`` / ``prior`` objects exposing exactly the attributes
``CJokerHelper.__init__`` reads (fast_likelihood.pyx:125-253).
"""
import importlib.util
import os
import sys

import numpy as np

from . import build as _build

_HERE = os.path.dirname(os.path.abspath(__file__))
_MODULE = None


def available():
    return os.path.exists(_build.ref_so_path())


def load():
    """Import the compiled reference module (``thejoker.src.fast_likelihood``)."""
    global _MODULE
    if _MODULE is not None:
        return _MODULE
    so = _build.ref_so_path()
    if not os.path.exists(so):
        raise FileNotFoundError(f"reference Cython module not built: {so}")
    stubs = os.path.join(_HERE, "ref_stubs")
    sys.path.insert(0, stubs)
    try:
        import astropy.units  # noqa: F401  (the stand-in)
        import thejoker.distributions  # noqa: F401
        import thejoker.src  # noqa: F401
        import thejoker.units  # noqa: F401
        import thejoker.utils  # noqa: F401
        spec = importlib.util.spec_from_file_location("thejoker.src.fast_likelihood", so)
        mod = importlib.util.module_from_spec(spec)
        sys.modules["thejoker.src.fast_likelihood"] = mod
        spec.loader.exec_module(mod)
    finally:
        sys.path.remove(stubs)
    _MODULE = mod
    return mod


class _Quantity:
    def __init__(self, value, unit):
        self.value = np.asarray(value, dtype=np.float64)
        self.unit = unit

    def to_value(self, unit=None):
        return self.value


class _Scalar:
    def __init__(self, value):
        self.value = float(value)

    def to_value(self, unit=None):
        return self.value


class _Data:
    """Duck-typed RVData: the attributes read at fast_likelihood.pyx:139, :155, :162-166."""

    def __init__(self, t, rv, ivar, t_ref):
        import astropy.units as u
        self._t_bmjd = np.ascontiguousarray(t, dtype=np.float64)
        self._t_ref_bmjd = float(t_ref)
        self.rv = _Quantity(rv, u.km / u.s)
        self.ivar = _Quantity(ivar, None)

    def __len__(self):
        return len(self._t_bmjd)


class _Op:
    def __init__(self, name):
        self._print_name = (name, "N")


class _Owner:
    def __init__(self, name):
        self.op = _Op(name)


class _Dist:
    def __init__(self, mean, std, kind="Normal"):
        import thejoker.units as xu
        self.mean = mean
        self.std = std
        self.owner = _Owner(kind)
        setattr(self, xu.UNIT_ATTR_NAME, None)


class _Named:
    def __init__(self, name):
        self.name = name


class _Prior:
    """Duck-typed JokerPrior: the attributes read at fast_likelihood.pyx:144-159, :202-253."""

    def __init__(self, poly_trend, n_offsets, mu, std, k_prior_scaled,
                 sigma_K0=0.0, P0=365.25, max_K=500.0):
        import thejoker.units as xu
        self.poly_trend = int(poly_trend)
        self.n_offsets = int(n_offsets)
        self._v_trend_names = [f"v{i}" for i in range(self.poly_trend)]
        self.v0_offsets = [_Named(f"dv0_{i + 1}") for i in range(self.n_offsets)]
        lin = ["K"] + self._v_trend_names
        self._linear_equiv_units = {k: None for k in lin}
        self.par_names = (["P", "e", "omega", "M0", "s"] + lin
                          + [o.name for o in self.v0_offsets])
        # mu / std are given in CJokerHelper's index order:
        # K, v0, offsets..., v1, ...
        order = ["K", "v0"] + [o.name for o in self.v0_offsets] + self._v_trend_names[1:]
        self.model = {}
        for idx, name in enumerate(order):
            kind = "FixedCompanionMass" if (name == "K" and k_prior_scaled) else "Normal"
            self.model[name] = _Dist(mu[idx], std[idx], kind)
        if k_prior_scaled:
            K = self.model["K"]
            K._sigma_K0 = _Scalar(sigma_K0)
            K._P0 = _Scalar(P0)
            K._max_K = _Scalar(max_K)
        Pvar = _Dist(0.0, 1.0)
        setattr(Pvar, xu.UNIT_ATTR_NAME, None)
        self.pars = {"K": self.model["K"], "P": Pvar}


def make_helper(t, rv, ivar, t_ref, trend_M, poly_trend, n_offsets, mu, std,
                k_prior_scaled, sigma_K0=0.0, P0=365.25, max_K=500.0):
    """Construct the reference ``CJokerHelper`` on plain arrays.

    ``mu`` / ``std`` follow CJokerHelper's linear-parameter index order
    (K, v0, offsets..., v1, ...); for a FixedCompanionMass K prior the K entry
    of ``std`` is ignored (the per-sample variance is computed from
    sigma_K0, P0, max_K).
    """
    mod = load()
    data = _Data(t, rv, ivar, t_ref)
    prior = _Prior(poly_trend, n_offsets, mu, std, k_prior_scaled, sigma_K0, P0, max_K)
    return mod.CJokerHelper(data, prior, np.ascontiguousarray(trend_M, dtype=np.float64))
