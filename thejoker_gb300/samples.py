"""JokerSamples: a table of prior or posterior samples (thejoker/samples.py).

Columns are NumPy arrays in fixed internal units (P in days, angles in
radians, velocities in the data's unit, trend terms in unit/day^i).  The packed
layout of the nonlinear parameters, ``P, e, omega, M0, s``, is the one the
reference's CJokerHelper reads (fast_likelihood.pyx:41, samples.py:404-445).
The on-disk format is a NumPy ``.npz`` in place of the reference's HDF5.
"""
import numpy as np

from .prior import validate_n_offsets, validate_poly_trend

__all__ = ["JokerSamples", "PACKED_ORDER"]

PACKED_ORDER = ["P", "e", "omega", "M0", "s"]


class JokerSamples:
    def __init__(self, samples=None, t_ref=None, n_offsets=None, poly_trend=None, **kwargs):
        poly_trend, v_names = validate_poly_trend(1 if poly_trend is None else poly_trend)
        n_offsets, off_names = validate_n_offsets(0 if n_offsets is None else n_offsets)
        self.t_ref = t_ref
        self.poly_trend = poly_trend
        self.n_offsets = n_offsets
        self.meta = dict(kwargs)
        self._valid = set(PACKED_ORDER + ["K"] + v_names + off_names +
                          ["ln_prior", "ln_likelihood", "ln_posterior"])
        self._cols = {}
        if samples is not None:
            for k, v in dict(samples).items():
                self[k] = v

    @property
    def par_names(self):
        return [k for k in self._cols if k not in ("ln_prior", "ln_likelihood", "ln_posterior")]

    def __setitem__(self, key, val):
        if key not in self._valid:
            raise ValueError(f"Invalid parameter name '{key}'")
        val = np.atleast_1d(np.asarray(val, dtype=np.float64))
        if self._cols and len(val) != len(self):
            raise ValueError("all columns must have the same length")
        self._cols[key] = val

    def __getitem__(self, key):
        if isinstance(key, str):
            return self._cols[key]
        out = JokerSamples(t_ref=self.t_ref, poly_trend=self.poly_trend,
                           n_offsets=self.n_offsets, **self.meta)
        for k, v in self._cols.items():
            out._cols[k] = np.atleast_1d(v[key])
        return out

    def __contains__(self, key):
        return key in self._cols

    def keys(self):
        return self._cols.keys()

    def __len__(self):
        if not self._cols:
            return 0
        return len(next(iter(self._cols.values())))

    def pack(self, units=None, names=None, nonlinear_only=True):
        """(n, k) float64 array of the columns in ``names`` (default the packed
        nonlinear order) and the names used.  Values are already in internal
        units; ``units`` is accepted for interface parity and ignored."""
        if names is None:
            names = PACKED_ORDER if nonlinear_only else self.par_names
        arr = np.stack([self._cols[n] for n in names], axis=1)
        return np.ascontiguousarray(arr, dtype=np.float64), list(names)

    @classmethod
    def unpack(cls, packed_samples, units, **kwargs):
        """Inverse of ``pack``; ``units`` gives the column names in order."""
        packed = np.asarray(packed_samples)
        names = list(units.keys()) if hasattr(units, "keys") else list(units)
        out = cls(**kwargs)
        for i, k in enumerate(names[:packed.shape[1]]):
            out[k] = packed[:, i]
        return out

    def write(self, path, overwrite=False):
        import os
        if os.path.exists(path) and not overwrite:
            raise OSError(f"{path} exists")
        np.savez(path, t_ref=np.nan if self.t_ref is None else self.t_ref,
                 poly_trend=self.poly_trend, n_offsets=self.n_offsets,
                 **{f"col_{k}": v for k, v in self._cols.items()})

    @classmethod
    def read(cls, path):
        z = np.load(path)
        t_ref = float(z["t_ref"])
        out = cls(t_ref=None if np.isnan(t_ref) else t_ref, poly_trend=int(z["poly_trend"]),
                  n_offsets=int(z["n_offsets"]))
        for k in z.files:
            if k.startswith("col_"):
                out[k[4:]] = z[k]
        return out

    def ln_unmarginalized_likelihood(self, data):
        """ln of the unmarginalized likelihood of ``data`` (an RVData) for each
        sample (samples.py:611-632 of the reference): the sum over epochs of
        ln N(rv | K m(t) + sum_k v_k (t - t_ref)^k, rv_err^2 + s^2), with the
        Keplerian and trend of each sample and no offset terms, as the
        reference's get_orbit builds them.  Evaluated on the GPU
        (joker_unmarginalized_lnl)."""
        from . import device as dev
        n = len(self)
        if n == 0:
            return np.zeros(0)
        nt = self.poly_trend
        pars = np.zeros((n, 6 + nt))
        for i, k in enumerate(["P", "e", "omega", "M0"]):
            pars[:, i] = self[k]
        if "s" in self:
            pars[:, 4] = self["s"]
        pars[:, 5] = self["K"]
        for j in range(nt):
            pars[:, 6 + j] = self[f"v{j}"]
        star = dict(t=data._t_bmjd, rv=data.rv, ivar=data.ivar, t_ref=data._t_ref_bmjd,
                    trend_M=np.zeros((len(data), 0)), mu=np.zeros(1), lam=np.ones(1),
                    k_prior=np.zeros(4))
        table = dev.StarTable([star])
        t_ref = data._t_ref_bmjd if self.t_ref is None else float(self.t_ref)
        out = dev.unmarginalized_lnl(table, 0, pars, nt, dt_shift=t_ref - data._t_ref_bmjd)
        return out.cpu().numpy()

    def __repr__(self):
        return f"<JokerSamples [{', '.join(self._cols)}] ({len(self)} samples)>"
