"""Autotuner for the launch shapes of the ln L kernels.

The persistent ln L kernels take work items of ``chunk`` samples of one star
(joker_lnl's ``chunk``; the CTA size is fixed at 128 by the kernels' launch
bounds).  Small chunks balance the tail of a launch over the SMs; large ones
spend less on staging a star's epochs and on the per-item work-queue atomics.
The best size depends on the GPU, the number of linear parameters, the jitter
mode, the precision and the epoch counts, so it is measured: ``tune`` times
``joker_lnl`` for each candidate on the caller's own stars and cache (CUDA
events, after a warm-up launch) and records the fastest in a JSON table keyed
by those properties.  ``chunk_for`` looks a workload up (default 1024 when it
was never tuned); BatchRejection and IterativeBatch use it when no chunk is
given.
"""
import json
import os
import threading

import numpy as np
import torch

from . import device as dev

__all__ = ["CANDIDATE_CHUNKS", "table_path", "load", "save", "key_for", "chunk_for", "tune"]

CANDIDATE_CHUNKS = (256, 512, 1024, 2048, 4096, 8192)
DEFAULT_CHUNK = 1024
_LOCK = threading.Lock()
_CACHE = {}


def table_path():
    """JSON file of tuned shapes: $JOKER_AUTOTUNE, else next to the built
    library."""
    p = os.environ.get("JOKER_AUTOTUNE")
    if p:
        return p
    from .build import OUT_DIR
    return os.path.join(OUT_DIR, "autotune.json")


def load(path=None):
    path = path or table_path()
    with _LOCK:
        if path not in _CACHE:
            try:
                with open(path) as f:
                    _CACHE[path] = json.load(f)
            except (OSError, ValueError):
                _CACHE[path] = {}
        return dict(_CACHE[path])


def save(table, path=None):
    path = path or table_path()
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, path)
    with _LOCK:
        _CACHE[path] = dict(table)


def _epoch_bucket(n_epochs):
    """Epoch-count bucket: 1-16, 17-64, 65-256, >256 (by the median)."""
    if n_epochs is None or len(n_epochs) == 0:
        return "any"
    m = float(np.median(np.asarray(n_epochs)))
    for b in (16, 64, 256):
        if m <= b:
            return f"<={b}"
    return ">256"


def key_for(n_linear, jitter, precision, n_epochs):
    name = torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"
    return f"{name}|L={n_linear}|jitter={jitter}|{precision}|N{_epoch_bucket(n_epochs)}"


def chunk_for(n_linear, jitter, precision, n_epochs, path=None):
    entry = load(path).get(key_for(n_linear, jitter, precision, n_epochs))
    return int(entry["chunk"]) if entry else DEFAULT_CHUNK


def tune(table, cache, precision="mixed_fast", n_epochs=None, star0=0, n_sel=None, count=None,
         candidates=CANDIDATE_CHUNKS, reps=3, path=None, write=True):
    """Time joker_lnl (joker_lnl_fused where "mixed_fast" runs the fused
    acceptance pass) over stars [star0, star0 + n_sel) x cache rows [0, count)
    for every candidate chunk; record and return the fastest (chunk,
    {chunk: ms})."""
    n_sel = table.n_stars - star0 if n_sel is None else int(n_sel)
    count = cache.size if count is None else int(count)
    out = torch.empty((n_sel, count), dtype=torch.float64, device="cuda")
    mixed = precision != "fp64"
    err = torch.empty((n_sel, count), dtype=torch.float32, device="cuda") if mixed else None
    keys = dev.MaxKeys(n_sel)
    bkeys = dev.MaxKeys(2 * n_sel) if mixed else None
    fused = dev.fused_available(table, precision)
    if fused:
        pcg = dev.pcg_table([(int(s), 1 + 2 * int(s)) for s in range(n_sel)])
        cand_ld, cand = dev.cand_words(n_sel, count)
    times = {}
    for ch in candidates:
        if fused:
            run = lambda: dev.lnl_fused(table, cache, out, err, bkeys, pcg, cand, cand_ld,
                                        star0=star0, n_sel=n_sel, count=count, max_keys=keys,
                                        chunk=ch)
        else:
            run = lambda: dev.lnl(table, cache, out, precision=precision, star0=star0,
                                  n_sel=n_sel, count=count, max_keys=keys, err=err,
                                  bound_keys=bkeys, chunk=ch)
        run()
        torch.cuda.synchronize()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        for _ in range(reps):
            run()
        t1.record()
        torch.cuda.synchronize()
        times[int(ch)] = t0.elapsed_time(t1) / reps
    best = min(times, key=times.get)
    if write:
        if n_epochs is None:
            ne = getattr(table, "n_epochs", None)
            n_epochs = ne[star0:star0 + n_sel] if ne is not None else [table.max_epochs]
        t = load(path)
        t[key_for(table.n_linear, table.jitter, precision, n_epochs)] = {
            "chunk": best, "ms": times, "stars": n_sel, "samples": count}
        save(t, path)
    return best, times
