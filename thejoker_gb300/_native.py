"""ctypes binding of libjoker_gb300.so (the C ABI in include/joker_gb300.h).

The library is loaded from the package's ``_lib`` directory; if it is missing
the import fails loudly -- there is no fallback path.
"""
import ctypes
import os

from .build import LIB_PATH

JOKER_OK = 0
JOKER_FP64 = 0
JOKER_MIXED = 1
JOKER_MIXED_ACCURATE = 2
JOKER_MIXED_FP64_TAIL = 3
JOKER_MIXED_FAST = 4
JOKER_JITTER_REFERENCE = 0
JOKER_JITTER_APPLIED = 1
JOKER_U_ARRAY = 0
JOKER_U_PCG64 = 1
JOKER_S_FIXED = 0
JOKER_S_LOGNORMAL = 1
JOKER_MAX_LINEAR = 6
JOKER_MIXED_LNL_TOL = 1e-4
JOKER_MIXED_LNL_BAND = 40.0

# every extern "C" symbol of include/joker_gb300.h
EXPORTED = (
    "joker_abi_version", "joker_last_error", "joker_launch_count", "joker_stars_create",
    "joker_stars_destroy",
    "joker_stars_info", "joker_stars_create_slots", "joker_stars_set", "joker_cache_create", "joker_cache_destroy", "joker_cache_load",
    "joker_cache_create_view", "joker_cache_bind",
    "joker_cache_capacity", "joker_batch_marginal_ln_likelihood", "joker_lnl",
    "joker_key_to_double", "joker_accept_workspace", "joker_accept", "joker_accept_refined",
    "joker_refine_max", "joker_iter_create", "joker_iter_destroy", "joker_iter_round",
    "joker_iter_outputs", "joker_iter_read", "joker_iter_create_pool", "joker_iter_admit",
    "joker_iter_set_round_budget", "joker_accept_noalloc", "joker_linear_posterior",
    "joker_unmarginalized_lnl", "joker_prior_sample", "joker_rv_from_elements",
    "joker_rejection_workspace", "joker_rejection_sample", "joker_refine_band",
    "joker_iter_read_async", "joker_lnl_fused", "joker_accept_fused",
)


class JokerError(RuntimeError):
    """A libjoker_gb300 call returned a non-zero status."""


class PriorSpec(ctypes.Structure):
    """joker_prior_spec (include/joker_gb300.h)."""
    _fields_ = [("P_min", ctypes.c_double), ("P_max", ctypes.c_double),
                ("e_alpha", ctypes.c_double), ("e_beta", ctypes.c_double),
                ("s_kind", ctypes.c_int32), ("pad", ctypes.c_int32),
                ("s_value", ctypes.c_double), ("s_mu", ctypes.c_double),
                ("s_sigma", ctypes.c_double)]


class AcceptSeg(ctypes.Structure):
    """Mirror of joker_accept_seg."""
    _fields_ = [
        ("lnl_off", ctypes.c_int64), ("n", ctypes.c_int64), ("idx_base", ctypes.c_int64),
        ("out_off", ctypes.c_int64), ("max_out", ctypes.c_int64), ("u_off", ctypes.c_int64),
        ("pcg_state_hi", ctypes.c_uint64), ("pcg_state_lo", ctypes.c_uint64),
        ("pcg_inc_hi", ctypes.c_uint64), ("pcg_inc_lo", ctypes.c_uint64),
        ("max_slot", ctypes.c_int32), ("star", ctypes.c_int32), ("row0", ctypes.c_int64),
    ]


_vp = ctypes.c_void_p
_i64 = ctypes.c_int64
_dp = ctypes.POINTER(ctypes.c_double)
_lp = ctypes.POINTER(ctypes.c_int64)

_SIGS = {
    "joker_abi_version": (ctypes.c_int, []),
    "joker_last_error": (ctypes.c_char_p, []),
    "joker_launch_count": (ctypes.c_uint64, []),
    "joker_stars_create": (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_int, ctypes.c_int, _lp,
                                          _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, ctypes.c_int]),
    "joker_stars_destroy": (ctypes.c_int, [_vp]),
    "joker_stars_info": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int),
                                        ctypes.POINTER(ctypes.c_int), _lp,
                                        ctypes.POINTER(ctypes.c_int)]),
    "joker_stars_create_slots": (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_int, ctypes.c_int,
                                                ctypes.c_int, ctypes.c_int]),
    "joker_stars_set": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _dp, _dp, _dp,
                                       ctypes.c_double, _dp, _dp, _dp, _dp, _vp]),
    "joker_cache_create": (ctypes.c_int, [ctypes.POINTER(_vp), _i64]),
    "joker_cache_destroy": (ctypes.c_int, [_vp]),
    "joker_cache_load": (ctypes.c_int, [_vp, _vp, _i64, _i64, _vp]),
    "joker_cache_capacity": (_i64, [_vp]),
    "joker_batch_marginal_ln_likelihood": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _i64, _vp, _vp]),
    "joker_lnl": (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_int, _i64, _i64, ctypes.c_int,
                                 _vp, _i64, _vp, _vp, _vp, ctypes.c_int, _i64, _vp]),
    "joker_lnl_fused": (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_int, _i64, _i64, _vp,
                                       _i64, _vp, _i64, _vp, _vp, _vp, _vp, _i64, _i64,
                                       ctypes.c_int, _vp]),
    "joker_accept_fused": (ctypes.c_int, [_vp, _vp, ctypes.POINTER(AcceptSeg), ctypes.c_int,
                                          _vp, _vp, _vp, _vp, ctypes.c_int, _vp, _i64, _vp, _vp,
                                          _vp, _vp, _vp, _i64, _vp]),
    "joker_key_to_double": (ctypes.c_double, [ctypes.c_uint64]),
    "joker_accept_workspace": (_i64, [ctypes.POINTER(AcceptSeg), ctypes.c_int]),
    "joker_accept": (ctypes.c_int, [ctypes.POINTER(AcceptSeg), ctypes.c_int, _vp, _vp,
                                    ctypes.c_int, _vp, _vp, _vp, _vp, _vp, _i64, _vp]),
    "joker_accept_refined": (ctypes.c_int, [_vp, _vp, ctypes.POINTER(AcceptSeg), ctypes.c_int,
                                            _vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_int, _vp, _vp, _vp, _vp, _vp, _vp, _i64,
                                            _vp]),
    "joker_refine_max": (ctypes.c_int, [_vp, _vp, ctypes.POINTER(AcceptSeg), ctypes.c_int, _vp,
                                        _vp, _vp, _vp, _vp, _vp, _i64, _vp]),
    "joker_refine_band": (ctypes.c_int, [_vp, _vp, ctypes.POINTER(AcceptSeg), ctypes.c_int, _vp,
                                         _vp, _vp, ctypes.c_double, ctypes.c_double, _vp, _vp,
                                         _i64, _vp]),
    "joker_iter_create": (ctypes.c_int, [ctypes.POINTER(_vp), _vp, _vp, ctypes.c_int, _i64, _i64,
                                         ctypes.c_int, _i64, ctypes.c_double, ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_uint64), ctypes.c_int]),
    "joker_iter_destroy": (ctypes.c_int, [_vp]),
    "joker_iter_round": (ctypes.c_int, [_vp, _vp]),
    "joker_iter_outputs": (ctypes.c_int, [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp),
                                          ctypes.POINTER(_vp), ctypes.POINTER(_vp),
                                          ctypes.POINTER(_vp)]),
    "joker_iter_read": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "joker_iter_read_async": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int, _vp, _vp]),
    "joker_iter_create_pool": (ctypes.c_int, [ctypes.POINTER(_vp), _vp, _vp, ctypes.c_int, _i64,
                                              _i64, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                              ctypes.c_int]),
    "joker_iter_admit": (ctypes.c_int, [_vp, ctypes.c_int, _i64, ctypes.c_int, _i64, _i64,
                                        ctypes.POINTER(ctypes.c_uint64), _vp]),
    "joker_iter_set_round_budget": (ctypes.c_int, [_vp, _i64]),
    "joker_cache_create_view": (ctypes.c_int, [ctypes.POINTER(_vp), _vp, _i64]),
    "joker_cache_bind": (ctypes.c_int, [ctypes.POINTER(_vp), _vp, _vp, _vp, _vp, _vp, _i64]),
    "joker_prior_sample": (ctypes.c_int, [_vp, _i64, _i64, ctypes.POINTER(PriorSpec), ctypes.c_uint64,
                                          _i64, _vp, _vp]),
    "joker_linear_posterior": (ctypes.c_int, [_vp, _vp, ctypes.c_int, _vp, _i64, ctypes.c_int,
                                              _vp, _vp, _vp, _vp]),
    "joker_unmarginalized_lnl": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _i64, ctypes.c_int,
                                                ctypes.c_double, _vp, _vp]),
    "joker_rv_from_elements": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _i64, ctypes.c_double,
                                              _vp, _vp]),
    "joker_rejection_workspace": (_i64, [ctypes.c_int, _i64, _i64, ctypes.c_int]),
    "joker_rejection_sample": (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_int, _i64, _i64,
                                              ctypes.c_int, ctypes.POINTER(ctypes.c_uint64),
                                              _i64, _vp, _vp, _vp, _vp, _i64, _vp]),
    "joker_accept_noalloc": (ctypes.c_int, [ctypes.POINTER(AcceptSeg), ctypes.c_int, _vp, _vp,
                                            ctypes.c_int, _vp, _vp, _vp, _vp, _vp]),
}

_LIB = None


def lib():
    """Load libjoker_gb300.so (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with thejoker_gb300.build.build() "
                "(nvcc, sm_103a); there is no CPU fallback")
        handle = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = handle
    return _LIB


def check(status, what=""):
    if status != JOKER_OK:
        msg = lib().joker_last_error().decode(errors="replace")
        raise JokerError(f"{what}: status {status}: {msg}")


def dptr(x):
    """ctypes pointer to a contiguous float64 numpy array."""
    return x.ctypes.data_as(_dp)


def lptr(x):
    return x.ctypes.data_as(_lp)
