"""The C-ABI library: builds for sm_103a, loads, exports every declared
symbol, and validates arguments before touching a device (CPU only)."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    src = open(os.path.join(ROOT, "include", "joker_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(joker_[a-z0-9_]+)\s*\(", src)))


def test_every_declared_symbol_is_exported(native_lib):
    from thejoker_gb300 import _native
    declared = _declared_symbols()
    assert len(declared) >= 14
    for name in declared:
        assert hasattr(native_lib, name), name
    assert sorted(_native.EXPORTED) == declared


def test_abi_version(native_lib):
    assert native_lib.joker_abi_version() == 1


def test_accept_seg_layout():
    from thejoker_gb300 import _native
    assert ctypes.sizeof(_native.AcceptSeg) == 96


def test_key_roundtrip(native_lib):
    from thejoker_gb300 import _native as nat
    import struct
    vals = [-1e300, -5.5, -0.0, 0.0, 1e-300, 3.25, 1e308, float("inf"), float("-inf")]
    keys = []
    for v in vals:
        b = struct.unpack("<q", struct.pack("<d", v))[0]
        k = (~b) & 0xFFFFFFFFFFFFFFFF if b < 0 else (b | (1 << 63))
        keys.append(k)
        assert nat.lib().joker_key_to_double(k) == v
    # the key order is the value order, strictly, with -0.0 just below 0.0
    for i in range(len(vals)):
        for j in range(len(vals)):
            if vals[i] < vals[j]:
                assert keys[i] < keys[j], (vals[i], vals[j])
    assert keys[2] < keys[3]                                   # -0.0, 0.0
    order = np.argsort(vals, kind="stable")
    assert all(keys[order[i]] <= keys[order[i + 1]] for i in range(len(vals) - 1))


def test_argument_validation_without_device(native_lib):
    """Shape and argument errors are reported before any CUDA call."""
    from thejoker_gb300 import _native as nat
    h = ctypes.c_void_p()
    off = np.array([0, 3], dtype=np.int64)
    t = np.array([0.0, 1.0, 2.0])
    one = np.ones(3)
    mu = np.zeros(2)
    lam = np.array([1.0, 1.0])
    kp = np.zeros(4)
    trend = np.ones(3)
    # n_linear out of range
    st = native_lib.joker_stars_create(ctypes.byref(h), 1, 0, nat.lptr(off), nat.dptr(t),
                                       nat.dptr(one), nat.dptr(one), nat.dptr(t[:1]),
                                       nat.dptr(trend), nat.dptr(mu), nat.dptr(lam),
                                       nat.dptr(kp), 0)
    assert st == 1 and b"n_linear" in native_lib.joker_last_error()
    st = native_lib.joker_stars_create(ctypes.byref(h), 1, 7, nat.lptr(off), nat.dptr(t),
                                       nat.dptr(one), nat.dptr(one), nat.dptr(t[:1]),
                                       nat.dptr(trend), nat.dptr(mu), nat.dptr(lam),
                                       nat.dptr(kp), 0)
    assert st == 1
    # non-positive ivar
    bad = one.copy()
    bad[1] = 0.0
    st = native_lib.joker_stars_create(ctypes.byref(h), 1, 2, nat.lptr(off), nat.dptr(t),
                                       nat.dptr(one), nat.dptr(bad), nat.dptr(t[:1]),
                                       nat.dptr(trend), nat.dptr(mu), nat.dptr(lam),
                                       nat.dptr(kp), 0)
    assert st == 1 and b"ivar" in native_lib.joker_last_error()
    # empty star
    off2 = np.array([0, 0], dtype=np.int64)
    st = native_lib.joker_stars_create(ctypes.byref(h), 1, 2, nat.lptr(off2), nat.dptr(t),
                                       nat.dptr(one), nat.dptr(one), nat.dptr(t[:1]),
                                       nat.dptr(trend), nat.dptr(mu), nat.dptr(lam),
                                       nat.dptr(kp), 0)
    assert st == 1 and b"no epochs" in native_lib.joker_last_error()
    # unknown jitter mode
    st = native_lib.joker_stars_create(ctypes.byref(h), 1, 2, nat.lptr(off), nat.dptr(t),
                                       nat.dptr(one), nat.dptr(one), nat.dptr(t[:1]),
                                       nat.dptr(trend), nat.dptr(mu), nat.dptr(lam),
                                       nat.dptr(kp), 5)
    assert st == 1
    # cache with bad capacity; NULL handles
    assert native_lib.joker_cache_create(ctypes.byref(h), 0) == 1
    assert native_lib.joker_lnl(None, None, 0, 1, 0, 1, 0, None, 1, None, None, None, 0, 0,
                                None) == 1
    assert native_lib.joker_batch_marginal_ln_likelihood(None, 0, None, 1, None, None) == 1
    assert native_lib.joker_accept(None, 0, None, None, 0, None, None, None, None, None, 0, None) == 0
    assert native_lib.joker_cache_capacity(None) == -1


def test_workspace_size(native_lib):
    from thejoker_gb300 import _native as nat
    segs = (nat.AcceptSeg * 2)()
    segs[0].n = 8192 * 3
    segs[1].n = 1
    ws = native_lib.joker_accept_workspace(segs, 2)
    assert ws >= 4 * 256 * 4 + 8 * 4


def test_rejection_workspace_size(native_lib):
    """joker_rejection_workspace is host arithmetic: ln L (8 B) and, for the
    mixed precisions, bounds (4 B) per (star, sample), keys and the acceptance
    workspace, each 256-byte aligned; nothing for an empty batch."""
    from thejoker_gb300 import _native as nat
    ws = nat.lib().joker_rejection_workspace
    assert ws(0, 1000, 16, nat.JOKER_MIXED) == 0 and ws(3, 0, 16, nat.JOKER_MIXED) == 0
    m = ws(3, 1 << 20, 256, nat.JOKER_MIXED)
    f = ws(3, 1 << 20, 256, nat.JOKER_FP64)
    assert m % 256 == 0 and f % 256 == 0
    assert m - f == 3 * 4 * (1 << 20)                      # the FP32 bounds
    assert f >= 3 * 8 * (1 << 20) + 4 * 8 * 3              # ln L and the keys
    assert ws(3, 1 << 21, 256, nat.JOKER_MIXED) > m
