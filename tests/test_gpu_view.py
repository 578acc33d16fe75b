"""Cache views (GB300 only): the mixed kernel reading the reference's packed
(S, 5) chunk directly, or five separate columns (joker_cache_bind) -- from
device memory or from pinned host memory over the host link -- gives
bit-identical ln L, error bounds and accepted samples to the prepared device
cache, and the zero-copy host pipeline equals the staged one."""
import numpy as np
import pytest
import torch

from gpu_util import synth_chunk, synth_star

pytestmark = pytest.mark.gpu


def _lnl(table, cache, S, precision):
    from thejoker_gb300 import device as dev
    out = torch.empty((1, S), dtype=torch.float64, device="cuda")
    keys = dev.MaxKeys(1)
    err = torch.empty((1, S), dtype=torch.float32, device="cuda") if precision != "fp64" else None
    bk = dev.MaxKeys(2) if err is not None else None
    dev.lnl(table, cache, out, precision=precision, max_keys=keys, err=err, bound_keys=bk)
    torch.cuda.synchronize()
    return (out[0].cpu().numpy(), None if err is None else err[0].cpu().numpy(),
            keys.t.cpu().numpy(), None if bk is None else bk.t.cpu().numpy())


@pytest.mark.parametrize("jitter,poly", [("reference", 1), ("applied", 1), ("applied", 3),
                                          ("reference", 3)])
@pytest.mark.parametrize("precision", ["mixed", "mixed_accurate", "fp64"])
def test_view_equals_cache(cuda, jitter, poly, precision):
    from thejoker_gb300 import device as dev
    rng = np.random.default_rng(7)
    star = synth_star(rng, 37, poly=poly)
    S = 50000
    chunk = synth_chunk(rng, S, jitter=(jitter == "applied"))
    chunk[:5, 3] = [0.0, 2 * np.pi - 1e-12, 1e-30, 40.0, -3.0]       # M0 edge cases
    chunk[5:8, 1] = [0.0, 0.999, 1e-9]                                 # e edge cases
    table = dev.StarTable([star], jitter=jitter)
    ref = _lnl(table, dev.PriorCache.from_samples(chunk), S, precision)
    d_chunk = torch.from_numpy(chunk).cuda()
    h_chunk = torch.from_numpy(chunk).pin_memory()
    caches = [dev.PriorCache.view(d_chunk), dev.PriorCache.view(h_chunk)]
    # the column form (joker_cache_bind), device and pinned host columns
    d_cols = [d_chunk[:, k].contiguous() for k in range(5)]
    h_cols = [torch.from_numpy(np.ascontiguousarray(chunk[:, k])).pin_memory() for k in range(5)]
    caches += [dev.PriorCache.bind(*d_cols), dev.PriorCache.bind(*h_cols)]
    for cache in caches:
        got = _lnl(table, cache, S, precision)
        for a, b in zip(ref, got):
            if a is not None:
                np.testing.assert_array_equal(a, b)


def test_view_refined_accept_and_errors(cuda):
    from thejoker_gb300 import device as dev
    rng = np.random.default_rng(8)
    star = synth_star(rng, 24)
    S = 1 << 18
    chunk = synth_chunk(rng, S, jitter=True)
    table = dev.StarTable([star], jitter="applied")
    res = []
    h_chunk = torch.from_numpy(chunk).pin_memory()
    for cache in (dev.PriorCache.from_samples(chunk), dev.PriorCache.view(h_chunk)):
        out = torch.empty((1, S), dtype=torch.float64, device="cuda")
        err = torch.empty((1, S), dtype=torch.float32, device="cuda")
        bk = dev.MaxKeys(2)
        dev.lnl(table, cache, out, precision="mixed", err=err, bound_keys=bk)
        st, inc = dev.pcg64_state(np.random.default_rng(3))
        seg = dict(lnl_off=0, n=S, idx_base=0, out_off=0, max_out=S, max_slot=0, star=0, row0=0,
                   pcg=(st, inc, 0))
        idx, _, cnt, exact, _ = dev.accept_refined(table, cache, out.view(-1), err.view(-1), bk,
                                                   [seg])
        c = int(cnt[0])
        res.append((c, idx[:c].cpu().numpy(), exact.t.cpu().numpy()))
    assert res[0][0] == res[1][0] > 0
    np.testing.assert_array_equal(res[0][1], res[1][1])
    np.testing.assert_array_equal(res[0][2], res[1][2])
    view = dev.PriorCache.view(h_chunk)
    with pytest.raises(Exception):
        view.load(torch.from_numpy(chunk[:10]).cuda())
    with pytest.raises(ValueError):
        dev.PriorCache.view(torch.from_numpy(chunk))            # pageable CPU tensor
    cols = [torch.from_numpy(np.ascontiguousarray(chunk[:, k])).cuda() for k in range(5)]
    with pytest.raises(ValueError):
        dev.PriorCache.bind(*cols[:4], cols[4][:-1])            # ragged columns
    with pytest.raises(ValueError):
        dev.PriorCache.bind(*cols[:4], torch.from_numpy(chunk[:, 4].copy()))   # pageable
    from thejoker_gb300 import _native as nat
    from thejoker_gb300._native import JokerError
    import ctypes
    h = ctypes.c_void_p()
    with pytest.raises(JokerError):
        nat.check(nat.lib().joker_cache_bind(ctypes.byref(h), ctypes.c_void_p(cols[0].data_ptr()),
                                             None, None, None, None, S), "joker_cache_bind")
    # a bound cache feeds the refined acceptance like the others
    bound = dev.PriorCache.bind(*cols)
    out = torch.empty((1, S), dtype=torch.float64, device="cuda")
    err = torch.empty((1, S), dtype=torch.float32, device="cuda")
    bk = dev.MaxKeys(2)
    dev.lnl(table, bound, out, precision="mixed", err=err, bound_keys=bk)
    st, inc = dev.pcg64_state(np.random.default_rng(3))
    seg = dict(lnl_off=0, n=S, idx_base=0, out_off=0, max_out=S, max_slot=0, star=0, row0=0,
               pcg=(st, inc, 0))
    idx, _, cnt, _, _ = dev.accept_refined(table, bound, out.view(-1), err.view(-1), bk, [seg])
    np.testing.assert_array_equal(idx[:int(cnt[0])].cpu().numpy(), res[0][1])


def test_zero_copy_pipeline_equals_staged(cuda):
    from thejoker_gb300 import device as dev
    from thejoker_gb300.pipeline import HostRejection
    rng = np.random.default_rng(9)
    stars = [synth_star(rng, n) for n in (12, 40, 7)]
    S = (1 << 18) + 777
    host = torch.from_numpy(synth_chunk(rng, S, jitter=True)).pin_memory()
    table = dev.StarTable(stars, jitter="applied")
    pcg = [dev.pcg64_state(np.random.default_rng(100 + k)) for k in range(3)]
    out = []
    for zc in (True, False):
        hr = HostRejection(table, S, precision="mixed", slice_rows=1 << 16, max_out=512,
                           zero_copy=zc)
        out.append(hr.run(host, pcg))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    for a, b in zip(out[0][1], out[1][1]):
        np.testing.assert_array_equal(a, b)
