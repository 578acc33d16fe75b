"""Iterative rejection sampling of many stars on the device, rounds replayed
from a CUDA graph.

Each star follows the reference's iterative_rejection_inmem
(thejoker/likelihood_helpers.py:130-229) over a shared prior library; all
per-star state (position in the library, batch size, prefix length,
accepted count, how many uniforms its generator has drawn) lives on the
device, so a round needs no host involvement and is captured once in a CUDA
graph, then replayed until every star has finished.
"""
import ctypes

import numpy as np
import torch

from . import _native as nat
from . import device as dev

__all__ = ["IterativeBatch"]

DONE_CODES = {0: "running", 1: "done", 2: "no samples accepted", 3: "hit maxiter"}


class IterativeBatch:
    """Iterative rejection of ``table``'s stars against cache rows
    [lib_row0, lib_row0 + lib_size).

    seeds: one numpy seed per star (its PCG64 stream gives that star's
    uniforms).  init_batch_size / growth_factor / safety_factor / maxiter as
    the reference (defaults: growth_factor * n_requested, 128, 1, 128).
    """

    def __init__(self, table, cache, n_requested, precision="mixed_fast", lib_row0=0, lib_size=None,
                 seeds=None, init_batch_size=None, growth_factor=128, safety_factor=1.0,
                 maxiter=128, chunk=None, round_budget=0):
        self.table, self.cache = table, cache
        self.n = table.n_stars
        self.n_requested = int(n_requested)
        lib_size = cache.size - lib_row0 if lib_size is None else int(lib_size)
        init = growth_factor * n_requested if init_batch_size is None else int(init_batch_size)
        if init > lib_size:
            raise ValueError("Prior sample library not big enough! For iterative sampling, you "
                             "have to have at least growth_factor * n_requested_samples = "
                             f"{growth_factor * n_requested} samples in the prior samples "
                             f"cache file. You have, or have limited to, {lib_size} samples.")
        if seeds is None:
            seeds = np.arange(self.n)
        if chunk is None:                      # the autotuned work-item size
            from .autotune import chunk_for
            chunk = chunk_for(table.n_linear, table.jitter, precision, table.n_epochs)
        pcg = self._pcg(seeds)
        self.lib_size, self.init = lib_size, init
        h = ctypes.c_void_p()
        nat.check(nat.lib().joker_iter_create(
            ctypes.byref(h), table.handle, cache.handle, dev.PRECISIONS[precision],
            int(lib_row0), lib_size, self.n_requested, init, float(safety_factor), int(maxiter),
            pcg.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), int(chunk)),
            "joker_iter_create")
        self._h = h
        nat.check(nat.lib().joker_iter_set_round_budget(h, int(round_budget)),
                  "joker_iter_set_round_budget")
        self.graph = None
        self.rounds = 0

    def _pcg(self, seeds):
        if len(seeds) != self.n:
            raise ValueError("one seed per star")
        pcg = np.zeros((self.n, 4), dtype=np.uint64)
        for k, sd in enumerate(seeds):
            st, inc = dev.pcg64_state(np.random.default_rng(int(sd)))
            pcg[k] = [st >> 64, st & ((1 << 64) - 1), inc >> 64, inc & ((1 << 64) - 1)]
        return pcg

    def reset(self, seeds):
        """Start every star again with new seeds (joker_iter_admit per star);
        the buffers and a captured round graph stay valid."""
        pcg = self._pcg(seeds)
        st = dev.stream_handle()
        for k in range(self.n):
            nat.check(nat.lib().joker_iter_admit(
                self._h, k, self.lib_size, self.n_requested, self.init, k * self.lib_size,
                pcg[k].ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), st), "joker_iter_admit")
        return self

    def _round(self):
        nat.check(nat.lib().joker_iter_round(self._h, dev.stream_handle()), "joker_iter_round")

    def _done(self):
        out = np.zeros(1, dtype=np.int32)
        nat.check(nat.lib().joker_iter_read(self._h, None, None, None,
                                            out.ctypes.data_as(ctypes.c_void_p), None),
                  "joker_iter_read")
        return int(out[0])

    def run(self, use_graph=True, max_rounds=1 << 20):
        """Run rounds until every star is finished; returns self.  The first
        round runs eagerly (it also loads the kernels); with use_graph the
        next rounds replay one captured round."""
        for _ in range(max_rounds):
            if use_graph and self.rounds >= 1:
                if self.graph is None:
                    g = torch.cuda.CUDAGraph()
                    s = torch.cuda.Stream()
                    s.wait_stream(torch.cuda.current_stream())
                    with torch.cuda.stream(s):
                        with torch.cuda.graph(g, stream=s):
                            self._round()
                    torch.cuda.current_stream().wait_stream(s)
                    self.graph = g
                self.graph.replay()
            else:
                self._round()
            self.rounds += 1
            torch.cuda.synchronize()
            if self._done() >= self.n:
                break
        return self

    def results(self):
        """(state rows (n, 8): start, n_process, n_evals, n_good, done, rounds,
        uniforms drawn, 0), [first n_requested accepted indices per star],
        number of samples re-evaluated in FP64)."""
        state = np.zeros((self.n, 8), dtype=np.int64)
        idx = np.zeros((self.n, self.n_requested), dtype=np.int64)
        nref = np.zeros(1, dtype=np.uint64)
        nat.check(nat.lib().joker_iter_read(self._h, state.ctypes.data_as(ctypes.c_void_p),
                                            idx.ctypes.data_as(ctypes.c_void_p), None, None,
                                            nref.ctypes.data_as(ctypes.c_void_p)),
                  "joker_iter_read")
        k = np.minimum(state[:, 3], self.n_requested)
        return state, [idx[s, :k[s]] for s in range(self.n)], int(nref[0])

    def close(self):
        if getattr(self, "_h", None) is not None:
            self.graph = None
            nat.lib().joker_iter_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
