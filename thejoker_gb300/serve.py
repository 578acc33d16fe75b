"""Serving loop: iterative rejection for stars that arrive over time.

Every request is one star with its own library budget (the first ``budget``
rows of a device-resident prior cache, the reference's
``iterative_rejection_sample(..., max_prior_samples=budget)``), samples
requested, and a numpy seed for its uniforms.  The engine is continuously
batched:
- Requests wait in a queue until a slot and pool space for their ln L prefix
  are free (admission by device memory); then they are admitted between two
  rounds.
- Every round advances all admitted stars at once: one plan, one persistent
  ln L launch over all their work items, one acceptance pass, one update.
  The round after the first is replayed from a CUDA graph.
- Finished stars leave, freeing their slot and pool range for the queue.
Per star the result is the same whether it runs alone or in a mix: its
samples, uniforms and schedule depend only on the star itself.
"""
import ctypes
import time
from collections import deque

import numpy as np
import torch

from . import _native as nat
from . import device as dev

__all__ = ["Request", "ServingEngine", "PoolAllocator"]


class PoolAllocator:
    """First-fit allocator of sample ranges in the engine's ln L pool."""

    def __init__(self, size, align=8192):
        self.size = int(size)
        self.align = int(align)
        self.free = [(0, self.size)]            # sorted (offset, length)

    def alloc(self, n):
        n = (int(n) + self.align - 1) // self.align * self.align
        for k, (o, l) in enumerate(self.free):
            if l >= n:
                if l == n:
                    self.free.pop(k)
                else:
                    self.free[k] = (o + n, l - n)
                return o, n
        return None

    def release(self, off, n):
        self.free.append((off, n))
        self.free.sort()
        merged = []
        for o, l in self.free:
            if merged and merged[-1][0] + merged[-1][1] == o:
                merged[-1] = (merged[-1][0], merged[-1][1] + l)
            else:
                merged.append((o, l))
        self.free = merged

    @property
    def available(self):
        return sum(l for _, l in self.free)


class Request:
    """One star: a StarTable dict, a library budget, samples requested, and a
    seed for its PCG64 uniform stream."""

    def __init__(self, star, budget, n_requested, seed, init_batch=None, growth_factor=128):
        self.star = star
        self.budget = int(budget)
        self.n_requested = int(n_requested)
        self.seed = int(seed)
        self.init_batch = int(growth_factor * n_requested if init_batch is None else init_batch)
        self.init_batch = min(self.init_batch, self.budget)
        self.t_arrival = None
        self.t_admitted = None
        self.t_done = None
        self.slot = None
        self.pool = None
        self.result = None           # (indices, n_good, n_evals, status)


class ServingEngine:
    """Continuously batched iterative rejection over one prior cache.

    round_budget: samples evaluated per round over all active stars (0: no
    limit).  Large batches then take several rounds, which bounds the round
    time, and with it how long a new request waits to start; the results do
    not change."""

    def __init__(self, cache, n_slots=1024, max_epochs=256, n_linear=2, pool_samples=None,
                 max_requested=512, precision="mixed_fast", safety_factor=1.0, maxiter=128,
                 chunk=1024, use_graph=True, pool_fraction=0.5, round_budget=0):
        self.cache = cache
        self.n_slots = int(n_slots)
        self.table = dev.StarTable.slots(n_slots, max_epochs, n_linear)
        if pool_samples is None:
            free, _ = torch.cuda.mem_get_info()
            per = 12 if precision != "fp64" else 8
            pool_samples = int(pool_fraction * free // per)
        self.pool = PoolAllocator(pool_samples)
        self.max_requested = int(max_requested)
        h = ctypes.c_void_p()
        nat.check(nat.lib().joker_iter_create_pool(
            ctypes.byref(h), self.table.handle, cache.handle, dev.PRECISIONS[precision], 0,
            int(pool_samples), self.max_requested, float(safety_factor), int(maxiter),
            int(chunk)), "joker_iter_create_pool")
        self._h = h
        nat.check(nat.lib().joker_iter_set_round_budget(h, int(round_budget)),
                  "joker_iter_set_round_budget")
        self.use_graph = use_graph
        self.graph = None
        self.rounds = 0
        self.stream = torch.cuda.Stream()
        self.queue = deque()
        self.free_slots = list(range(self.n_slots))[::-1]
        self.active = {}
        self.done = []
        self.samples_evaluated = 0
        # after every round its state table (n_slots x 8) comes back into one of
        # two pinned buffers; the host retires round k - 1 while round k runs
        self._state_h = [torch.empty((self.n_slots, 8), dtype=torch.int64).pin_memory()
                         for _ in range(2)]
        self._state_ev = [torch.cuda.Event() for _ in range(2)]
        self._pending = None              # (buffer, round) of the last round's state copy
        self._idx_h = torch.empty((self.n_slots, self.max_requested),
                                  dtype=torch.int64).pin_memory()
        self._side = torch.cuda.Stream()

    # ------------------------------------------------------------ requests
    def submit(self, req, t=None):
        req.t_arrival = time.perf_counter() if t is None else t
        self.queue.append(req)

    def _admit(self):
        n = 0
        while self.queue and self.free_slots:
            req = self.queue[0]
            if req.budget > self.cache.size:
                raise ValueError("request budget larger than the prior cache")
            if req.n_requested > self.max_requested:
                raise ValueError("request asks for more samples than max_requested")
            rng = self.pool.alloc(req.budget)
            if rng is None:
                break                                # wait for memory to free up
            self.queue.popleft()
            slot = self.free_slots.pop()
            req.slot, req.pool = slot, rng
            self.table.set(slot, req.star, stream=self.stream)
            st, inc = dev.pcg64_state(np.random.default_rng(req.seed))
            pcg = np.array([st >> 64, st & ((1 << 64) - 1), inc >> 64, inc & ((1 << 64) - 1)],
                           dtype=np.uint64)
            nat.check(nat.lib().joker_iter_admit(
                self._h, slot, req.budget, req.n_requested, req.init_batch, rng[0],
                pcg.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                dev.stream_handle(self.stream)), "joker_iter_admit")
            req.t_admitted = time.perf_counter()
            req.admit_round = self.rounds       # the first round that includes it
            self.active[slot] = req
            n += 1
        return n

    def _round(self):
        with torch.cuda.stream(self.stream):
            if self.use_graph and self.rounds >= 1:
                if self.graph is None:
                    g = torch.cuda.CUDAGraph()
                    with torch.cuda.graph(g, stream=self.stream):
                        nat.check(nat.lib().joker_iter_round(self._h, dev.stream_handle(self.stream)),
                                  "joker_iter_round")
                    self.graph = g
                self.graph.replay()
            else:
                nat.check(nat.lib().joker_iter_round(self._h, dev.stream_handle(self.stream)),
                          "joker_iter_round")
            # the round's state table to the host, asynchronously
            b = self.rounds % 2
            nat.check(nat.lib().joker_iter_read_async(
                self._h, ctypes.c_void_p(self._state_h[b].data_ptr()), None, 0, None,
                dev.stream_handle(self.stream)), "joker_iter_read_async")
            self._state_ev[b].record(self.stream)
        pending = (self.rounds % 2, self.rounds)
        self.rounds += 1
        return pending

    def _retire(self, pending):
        """Retire the stars that round `pending` finished: its state copy is
        complete by now (the following round was queued after it), the index
        rows of only the finished slots are copied on a side stream (the
        rounds running meanwhile do not write them)."""
        b, k = pending
        self._state_ev[b].synchronize()
        state = self._state_h[b].numpy()
        finished = [s for s, req in self.active.items()
                    if req.admit_round <= k and state[s, 4] != 0]
        if not finished:
            return 0
        slots = np.array(finished, dtype=np.int32)
        nat.check(nat.lib().joker_iter_read_async(
            self._h, None, slots.ctypes.data_as(ctypes.c_void_p), len(finished),
            ctypes.c_void_p(self._idx_h.data_ptr()), dev.stream_handle(self._side)),
            "joker_iter_read_async")
        self._side.synchronize()
        idx = self._idx_h.numpy()
        now = time.perf_counter()
        for j, s in enumerate(finished):
            req = self.active.pop(s)
            row = state[s]
            n = int(min(row[3], req.n_requested))
            status = {1: "done", 2: "no samples accepted", 3: "hit maxiter"}.get(int(row[4]), "?")
            req.result = (idx[j, :n].copy(), int(row[3]), int(row[2]), status)
            req.t_done = now
            self.samples_evaluated += int(row[2])
            self.pool.release(*req.pool)
            self.free_slots.append(s)
            self.done.append(req)
        return len(finished)

    def step(self):
        """Admit what fits, queue one round for every active star, and retire
        the stars the previous round finished while this one runs.  Returns
        the number of active stars after the step."""
        self._admit()
        prev, self._pending = self._pending, None
        if self.active:
            self._pending = self._round()
        if prev is not None:
            self._retire(prev)
        return len(self.active)

    def drain(self):
        while self.queue or self.active or self._pending is not None:
            self.step()
        return self.done

    def latency_stats(self):
        lat = np.array([r.t_done - r.t_arrival for r in self.done])
        if lat.size == 0:
            return {}
        return {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
                "mean_s": float(lat.mean()), "n": int(lat.size)}

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
