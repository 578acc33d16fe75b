"""Degenerate designs (CPU only): the reference against this library.

The reference's likelihood has failure branches for an exactly singular
linear system: +INF when the LU of the L x L matrix Ainv finds a zero pivot
(fast_likelihood.pyx:283-291, 381-382) and -INF through an infinite
log-determinant when the LU of the N x N matrix B does (:347-348).  With
finite prior variances and errors both matrices are positive definite, so
those branches need degenerate inputs; on the ones that reach them -- an
infinite prior variance on an offset column that duplicates the constant
column, zero errors at most epochs, an infinite v0 variance -- the compiled
reference returns NaN for every sample (rounding leaves no exact zero pivot;
the infinities reach B).  The fixture ref_lnl_degenerate.npz records that
output.  This library rejects the same inputs when the star table is built
(JOKER_EINVAL with a message), before any device work: a deliberate
deviation, a loud error in place of a likelihood of NaN everywhere.
"""
import ctypes
import os

import numpy as np
import pytest

CASES = ["dup_offset_inf_var", "zero_errors", "inf_v0_var"]


@pytest.mark.parametrize("case", CASES)
def test_reference_returns_nan_on_degenerate_designs(golden_dir, case):
    z = np.load(os.path.join(golden_dir, "ref_lnl_degenerate.npz"))
    assert np.all(np.isnan(z[f"{case}_lnl_ref"]))


@pytest.mark.parametrize("case", CASES)
def test_star_table_rejects_degenerate_designs(native_lib, golden_dir, case):
    from thejoker_gb300 import _native as nat
    z = np.load(os.path.join(golden_dir, "ref_lnl_degenerate.npz"))
    t, rv = z["t"], z["rv"]
    ivar = np.ascontiguousarray(z[f"{case}_ivar"])
    trend = np.ascontiguousarray(z[f"{case}_trend_M"])
    mu = np.ascontiguousarray(z[f"{case}_mu"])
    lam = np.ascontiguousarray(z[f"{case}_lam"])
    L = len(mu)
    off = np.array([0, len(t)], dtype=np.int64)
    kp = np.array([1.0, 30.0, 365.25, 500.0])
    tref = np.array([t.min()])
    h = ctypes.c_void_p()
    st = native_lib.joker_stars_create(ctypes.byref(h), 1, L, nat.lptr(off), nat.dptr(t),
                                       nat.dptr(rv), nat.dptr(ivar), nat.dptr(tref),
                                       nat.dptr(trend), nat.dptr(mu), nat.dptr(lam),
                                       nat.dptr(kp), nat.JOKER_JITTER_REFERENCE)
    assert st == 1, "expected JOKER_EINVAL"
    assert not h.value
    assert native_lib.joker_last_error()
