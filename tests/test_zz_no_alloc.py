"""joker_accept_noalloc -- the acceptance pass for callers that cannot
allocate device memory -- against joker_accept (GB300 only).

Some callers of this library cannot call cudaMalloc: a serving loop with
per-request deadlines (cudaMalloc may synchronise the device) or a plugin
inside a framework whose allocator already holds the free device memory.
For them the pass keeps its scratch space in a fixed array inside the library.
This test makes the start-up call (no segments), then calls that entry point
through the C ABI twice in a row, with different inputs, and checks each
result against the ordinary entry point, which uses a caller-supplied
workspace, and that the device's free memory is the same after each call as
before it.  Indices and counts are integers and
must match exactly; the gathered ln L values are copies and must match
bit for bit.  The file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _keys(values):
    import struct
    out = []
    for m in values:
        b = struct.unpack("<q", struct.pack("<d", m))[0]
        k = (~b) & 0xFFFFFFFFFFFFFFFF if b < 0 else (b | (1 << 63))
        out.append(np.array(k, dtype=np.uint64).view(np.int64))
    return torch.tensor(np.array(out, dtype=np.int64), device="cuda")


def _segments(rng, sizes, pcg):
    from thejoker_gb300 import _native as nat
    from thejoker_gb300.device import pcg64_fields
    arr = (nat.AcceptSeg * len(sizes))()
    off = 0
    out_off = 0
    for i, n in enumerate(sizes):
        a = arr[i]
        a.lnl_off, a.n, a.idx_base = off, n, 1000 * i
        a.out_off, a.max_out = out_off, max(1, n // 3)
        a.u_off = off
        a.max_slot = i
        a.pcg_state_hi, a.pcg_state_lo, a.pcg_inc_hi, a.pcg_inc_lo = pcg64_fields(*pcg, offset=off)
        off += n
        out_off += a.max_out
    return arr, off, out_off


def _warm_up():
    """The start-up call with no segments: looks up the fixed array on this
    device and loads the pass's kernels, so no later call loads anything."""
    from thejoker_gb300 import _native as nat
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    nat.check(nat.lib().joker_accept_noalloc(None, 0, None, None, 1, None, None, None, None,
                                             stream), "joker_accept_noalloc warm-up")
    torch.cuda.synchronize()


def _run(fn_name, arr, n_segs, lnl, keys, u_source, u, n_out):
    from thejoker_gb300 import _native as nat
    lib = nat.lib()
    idx = torch.full((n_out,), -7, dtype=torch.int64, device="cuda")
    olnl = torch.full((n_out,), float("nan"), dtype=torch.float64, device="cuda")
    cnt = torch.full((n_segs,), -1, dtype=torch.int64, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    uptr = ctypes.c_void_p(u.data_ptr()) if u is not None else None
    if fn_name == "joker_accept":
        ws = lib.joker_accept_workspace(arr, n_segs)
        work = torch.empty(int(ws), dtype=torch.uint8, device="cuda")
        st = lib.joker_accept(arr, n_segs, ctypes.c_void_p(lnl.data_ptr()),
                              ctypes.c_void_p(keys.data_ptr()), u_source, uptr,
                              ctypes.c_void_p(idx.data_ptr()), ctypes.c_void_p(olnl.data_ptr()),
                              ctypes.c_void_p(cnt.data_ptr()), ctypes.c_void_p(work.data_ptr()),
                              int(ws), stream)
    else:
        st = lib.joker_accept_noalloc(arr, n_segs, ctypes.c_void_p(lnl.data_ptr()),
                                      ctypes.c_void_p(keys.data_ptr()), u_source, uptr,
                                      ctypes.c_void_p(idx.data_ptr()),
                                      ctypes.c_void_p(olnl.data_ptr()),
                                      ctypes.c_void_p(cnt.data_ptr()), stream)
    nat.check(st, fn_name)
    torch.cuda.synchronize()
    if fn_name == "joker_accept_noalloc":
        # after the warm-up the call takes no device memory: free memory is
        # unchanged across it (its outputs were allocated before)
        assert torch.cuda.mem_get_info()[0] == free0
    return idx.cpu().numpy(), olnl.cpu().numpy(), cnt.cpu().numpy()


@pytest.mark.parametrize("u_source", [0, 1])
def test_noalloc_matches_workspace_version_twice(u_source):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from thejoker_gb300 import build
    build.build()
    _warm_up()
    rng = np.random.default_rng(2024 + u_source)
    gen = np.random.default_rng(77)
    pcg = (int(gen.bit_generator.state["state"]["state"]),
           int(gen.bit_generator.state["state"]["inc"]))
    # two calls in a row with different segment layouts and values; the second
    # is smaller, so stale contents of the shared array would show up
    for sizes in ([40000, 8192, 3, 70001], [5000, 12]):
        arr, total, n_out = _segments(rng, sizes, pcg)
        lnl_h = rng.normal(-3.0, 2.0, total)
        lnl = torch.from_numpy(lnl_h).cuda()
        maxes, off = [], 0
        for n in sizes:
            maxes.append(lnl_h[off:off + n].max())
            off += n
        keys = _keys(maxes)
        u = torch.from_numpy(rng.uniform(size=total)).cuda() if u_source == 0 else None
        a = _run("joker_accept", arr, len(sizes), lnl, keys, u_source, u, n_out)
        b = _run("joker_accept_noalloc", arr, len(sizes), lnl, keys, u_source, u, n_out)
        np.testing.assert_array_equal(a[2], b[2])
        assert np.all(b[2] > 0)
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])


def test_noalloc_rejects_sizes_above_its_limit():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from thejoker_gb300 import _native as nat
    lib = nat.lib()
    arr = (nat.AcceptSeg * 1)()
    arr[0].n = 2049 * 8192            # one block more than JOKER_NOALLOC_MAX_BLOCKS
    arr[0].max_out = 1
    dummy = torch.zeros(1, dtype=torch.float64, device="cuda")
    st = lib.joker_accept_noalloc(arr, 1, ctypes.c_void_p(dummy.data_ptr()),
                                  ctypes.c_void_p(dummy.data_ptr()), 1, None,
                                  ctypes.c_void_p(dummy.data_ptr()), None,
                                  ctypes.c_void_p(dummy.data_ptr()), None)
    assert st == 4 and b"JOKER_NOALLOC_MAX_BLOCKS" in lib.joker_last_error()
    many = (nat.AcceptSeg * 1025)()
    st = lib.joker_accept_noalloc(many, 1025, ctypes.c_void_p(dummy.data_ptr()),
                                  ctypes.c_void_p(dummy.data_ptr()), 1, None,
                                  ctypes.c_void_p(dummy.data_ptr()), None,
                                  ctypes.c_void_p(dummy.data_ptr()), None)
    assert st == 4
