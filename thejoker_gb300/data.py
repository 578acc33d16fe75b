"""Radial-velocity data and the linear design matrix.

Mirrors the parts of the reference's ``RVData`` (thejoker/data.py:16-152) and
``validate_prepare_data`` (thejoker/data_helpers.py:56-133) that the
likelihood consumes.  Quantities are plain floats in fixed units: times are
Barycentric MJD days (the reference's internal ``_t_bmjd``), velocities and
errors share one velocity unit (km/s unless stated otherwise).
"""
import numpy as np

__all__ = ["RVData", "validate_prepare_data", "get_constant_term_design_matrix",
           "get_trend_design_matrix"]


class RVData:
    """Time-domain RV measurements of one target.

    Like the reference (data.py:75-122): non-finite points are dropped when
    ``clean``, points are sorted in time, and ``t_ref`` defaults to the
    earliest time (``t_ref=False`` means 0).
    """

    def __init__(self, t, rv, rv_err, t_ref=None, clean=True, rv_unit="km/s"):
        t = np.atleast_1d(np.asarray(t, dtype=np.float64))
        rv = np.atleast_1d(np.asarray(rv, dtype=np.float64))
        rv_err = np.atleast_1d(np.asarray(rv_err, dtype=np.float64))
        if rv_err.ndim != 1:
            raise NotImplementedError("a full covariance matrix is not supported by this path")
        if rv_err.shape != rv.shape:
            raise ValueError(f"Invalid shape for input RV error {rv_err.shape}. "
                             f"Should be ({rv.size},)")
        if t.shape != rv.shape:
            raise ValueError(f"Shape of input times and RVs must be consistent "
                             f"({t.shape} vs {rv.shape})")
        if clean:
            idx = np.isfinite(t) & np.isfinite(rv) & np.isfinite(rv_err)
            t, rv, rv_err = t[idx], rv[idx], rv_err[idx]
        idx = np.argsort(t, kind="stable")
        self._t_bmjd = t[idx]
        self.rv = rv[idx]
        self.rv_err = rv_err[idx]
        self.rv_unit = rv_unit
        if t_ref is False:
            self.t_ref = None
            self._t_ref_bmjd = 0.0
        else:
            if t_ref is None:
                t_ref = float(self._t_bmjd.min())
            self.t_ref = float(t_ref)
            self._t_ref_bmjd = float(t_ref)

    @property
    def t(self):
        return self._t_bmjd

    @property
    def ivar(self):
        """Inverse variance 1 / rv_err^2 (data.py:146-152)."""
        return 1.0 / self.rv_err ** 2

    def __len__(self):
        return len(self.rv)


def get_constant_term_design_matrix(data, ids=None):
    """Constant term plus one indicator column per extra data source
    (likelihood_helpers.py:8-25)."""
    if ids is None:
        ids = np.zeros(len(data), dtype=int)
    ids = np.asarray(ids)
    unq = np.unique(ids)
    out = np.zeros((len(data), len(unq)))
    out[:, 0] = 1.0
    for j, id_ in enumerate(unq[1:]):
        out[ids == id_, j + 1] = 1.0
    return out


def get_trend_design_matrix(data, ids, poly_trend):
    """Design matrix of the linear parameters other than K
    (likelihood_helpers.py:28-37): [const/offset columns, dt^1, ..., dt^(p-1)]."""
    const = get_constant_term_design_matrix(data, ids)
    dt = data._t_bmjd - data._t_ref_bmjd
    trend = np.vander(dt, N=poly_trend, increasing=True)[:, 1:]
    return np.hstack((const, trend))


def validate_prepare_data(data, poly_trend, n_offsets, ref_ids_order=True):
    """Concatenate one or several data sources (data_helpers.py:56-133).

    Returns (all_data, ids, trend_M).  Several sources share the reference time
    of the concatenated data, as in the reference.

    ``RVData`` sorts the concatenated epochs by time (data.py:97-104), but the
    reference builds the offset columns from the source ids in concatenation
    order (data_helpers.py:115-133).  With ``ref_ids_order`` (the default,
    for parity) the same happens here: when the sources' times interleave,
    an epoch's offset column is that of the epoch at its position before the
    sort.  ``ref_ids_order=False`` sorts the ids with the epochs, so that each
    epoch gets its own source's column.
    """
    if isinstance(data, RVData):
        if n_offsets != 0:
            raise ValueError("If sampling over velocity offsets between data sources, you "
                             "must pass in multiple data sources. To do this, pass in a "
                             "list of RVData instances or a dictionary with RVData "
                             "instances as values.")
        return data, np.zeros(len(data), dtype=int), get_trend_design_matrix(data, None, poly_trend)
    if not hasattr(data, "keys"):
        try:
            data = {i: d for i, d in enumerate(data)}
        except Exception as exc:
            raise TypeError("Failed to parse input data: data must either be an RVData "
                            "instance, an iterable of RVData instances, or a dictionary "
                            f"with RVData instances as values. Received: {type(data)}") from exc
    t, rv, err, ids = [], [], [], []
    for k in data.keys():
        d = data[k]
        if not isinstance(d, RVData):
            raise TypeError(f"All data must be specified as RVData instances: Object at key "
                            f"'{k}' is a '{type(d)}' instead.")
        t.append(d._t_bmjd)
        rv.append(d.rv)
        err.append(d.rv_err)
        ids.append([k] * len(d))
    t = np.concatenate(t)
    rv = np.concatenate(rv)
    err = np.concatenate(err)
    ids = np.concatenate(ids)
    if len(np.unique(ids)) - 1 != n_offsets:
        raise ValueError("Number of data IDs + 1 must equal the number of priors on constant "
                         "offsets specified (i.e. v0_offsets)")
    all_data = RVData(t, rv, err)
    if not ref_ids_order:
        ids = ids[np.argsort(t, kind="stable")]
    return all_data, ids, get_trend_design_matrix(all_data, ids, poly_trend)
