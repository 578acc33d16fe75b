"""Multi-GPU sharding of the rejection path (one process per GPU).

Two shardings, as the work partitions:

* stars across ranks (the batched survey case): every rank holds the whole
  prior cache and its share of the stars.  There is no exchange; the shares
  are balanced by epoch count (longest-processing-time assignment).
* one star's prior samples across ranks (a single star with a huge cache):
  rank r owns rows [row0_r, row0_r + n_r).  The acceptance test needs the
  star's maximum over all samples.  So after the ln L pass the ranks exchange
  maxima in one all-reduce(max), and a second one after the FP64 refinement of
  the maximum.  Each rank then keeps its own samples against that maximum and
  the uniforms u[row0_r + i] of the star's stream.

Maxima travel as order-preserving 64-bit keys (the image of a double whose
unsigned order is the double's order); with the top bit flipped their signed
order is the same, which is what a MAX all-reduce compares.
"""
import heapq

import numpy as np
import torch

__all__ = ["shard_rows", "shard_stars", "key_of", "value_of", "allreduce_max_keys",
           "ShardedRejection", "StarShardedRejection", "gather_indices"]

_TOP = -(1 << 63)


def shard_rows(n_rows, world, rank):
    """(row0, count) of rank's contiguous share of n_rows (remainder to the
    first ranks, as the reference's batch_tasks splits, utils.py:22-72)."""
    base, rem = divmod(int(n_rows), int(world))
    row0 = rank * base + min(rank, rem)
    return row0, base + (1 if rank < rem else 0)


def shard_stars(n_epochs, world):
    """Star indices per rank, balanced by epoch count (LPT)."""
    order = np.argsort(-np.asarray(n_epochs), kind="stable")
    heap = [(0, r) for r in range(world)]
    out = [[] for _ in range(world)]
    for s in order:
        load, r = heapq.heappop(heap)
        out[r].append(int(s))
        heapq.heappush(heap, (load + int(n_epochs[s]), r))
    return [sorted(v) for v in out]


def key_of(x):
    """Order-preserving uint64 key of a double (NaN is the largest key)."""
    x = np.asarray(x, dtype=np.float64)
    b = x.view(np.int64).astype(np.int64)
    k = np.where(b < 0, ~b, b | np.int64(_TOP)).view(np.uint64)
    return np.where(np.isnan(x), np.uint64(0xFFFFFFFFFFFFFFFF), k)


def value_of(k):
    k = np.asarray(k, dtype=np.uint64)
    top = (k & np.uint64(1 << 63)) != 0
    b = np.where(top, k & np.uint64((1 << 63) - 1), ~k)
    return b.astype(np.uint64).view(np.float64)


def _all_reduce(t, op, group=None):
    """In-place all-reduce; a CUDA tensor goes through host memory when the
    group's backend is gloo (its collectives are host-side)."""
    import torch.distributed as dist
    if t.is_cuda and dist.get_backend(group) == "gloo":
        h = t.cpu()
        dist.all_reduce(h, op=op, group=group)
        t.copy_(h)
    else:
        dist.all_reduce(t, op=op, group=group)
    return t


def allreduce_max_keys(keys, group=None):
    """In-place MAX all-reduce of an int64 tensor holding uint64 keys."""
    import torch.distributed as dist
    flip = torch.tensor(_TOP, dtype=torch.int64, device=keys.device)
    m = torch.bitwise_xor(keys, flip)
    _all_reduce(m, dist.ReduceOp.MAX, group)
    keys.copy_(torch.bitwise_xor(m, flip))
    return keys


def gather_indices(local_idx, group=None):
    """Concatenate each rank's (ascending) accepted indices in rank order,
    which is ascending overall because the shards are contiguous row ranges."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    n = torch.tensor([len(local_idx)], dtype=torch.int64)
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, n, group=group)
    mx = int(max(int(s) for s in sizes))
    buf = torch.full((max(mx, 1),), -1, dtype=torch.int64)
    buf[:len(local_idx)] = torch.as_tensor(np.asarray(local_idx, dtype=np.int64))
    bufs = [torch.empty_like(buf) for _ in range(world)]
    dist.all_gather(bufs, buf, group=group)
    return np.concatenate([b[:int(s)].numpy() for b, s in zip(bufs, sizes)])


class ShardedRejection:
    """One star's rejection over a prior cache sharded by rows across ranks.

    Each rank passes its own PriorCache holding rows [row0, row0 + n) of the
    global chunk.  ``run`` evaluates, exchanges the maxima (two all-reduces)
    and accepts; it returns this rank's accepted global indices and the global
    count.
    """

    def __init__(self, table, cache, row0, precision="mixed_fast", max_out=1 << 20, group=None):
        from . import device as dev
        self.dev = dev
        self.table, self.cache, self.row0 = table, cache, int(row0)
        self.precision = precision
        self.group = group
        n = cache.size
        self.lnl = torch.empty((1, n), dtype=torch.float64, device="cuda")
        self.err = torch.empty((1, n), dtype=torch.float32, device="cuda") \
            if precision != "fp64" else None
        self.keys = dev.MaxKeys(1)
        self.bkeys = dev.MaxKeys(2) if self.err is not None else None
        self.max_out = int(max_out)

    def run(self, pcg_state):
        import torch.distributed as dist
        dev = self.dev
        n = self.cache.size
        self.keys.t.zero_()
        if self.bkeys is not None:
            self.bkeys.t.zero_()
        dev.lnl(self.table, self.cache, self.lnl, precision=self.precision, max_keys=self.keys,
                err=self.err, bound_keys=self.bkeys)
        allreduce_max_keys(self.keys.t, self.group)
        st, inc = pcg_state
        seg = dict(lnl_off=0, n=n, idx_base=self.row0, out_off=0, max_out=self.max_out,
                   max_slot=0, star=0, row0=0, pcg=(st, inc, self.row0))
        if self.err is None:
            idx, _, cnt = dev.accept(self.lnl.view(-1), self.keys, [seg])
        else:
            allreduce_max_keys(self.bkeys.t, self.group)
            exact, _ = dev.refine_max(self.table, self.cache, self.lnl.view(-1),
                                      self.err.view(-1), self.bkeys, [seg])
            allreduce_max_keys(exact.t, self.group)
            idx, _, cnt, _, _ = dev.accept_refined(self.table, self.cache, self.lnl.view(-1),
                                                   self.err.view(-1), self.bkeys, [seg],
                                                   exact=exact)
        c = int(cnt[0])
        total = torch.tensor([c], dtype=torch.int64, device="cuda")
        _all_reduce(total, dist.ReduceOp.SUM, self.group)
        return idx[:min(c, self.max_out)].cpu().numpy(), int(total)


class StarShardedRejection:
    """Rejection sampling of many stars sharded across ranks by star, with no
    exchange: every rank holds the whole prior cache and runs a BatchRejection
    over its share of the stars (``shard_stars``, balanced by epoch count).
    Star k uses the PCG64 stream of ``seeds[k]`` whichever rank owns it, so
    the results do not depend on the number of ranks.

    ``stars``: the full list of star dicts (as StarTable takes); ``world`` and
    ``rank`` default to the process group's.  ``results`` returns this rank's
    (global star indices, counts, indices, ln L); ``gather`` collects every
    star's results in star order on every rank (host objects, so any backend).
    """

    def __init__(self, stars, cache, precision="mixed_fast", jitter="reference", max_out=256,
                 seeds=None, world=None, rank=None, group=None, chunk=None):
        import torch.distributed as dist
        from .batch import BatchRejection
        if world is None:
            world = dist.get_world_size(group) if dist.is_initialized() else 1
        if rank is None:
            rank = dist.get_rank(group) if dist.is_initialized() else 0
        self.world, self.rank, self.group = int(world), int(rank), group
        self.n_stars = len(stars)
        n_ep = np.array([len(s["t"]) for s in stars])
        self.mine = shard_stars(n_ep, self.world)[self.rank]
        if seeds is None:
            seeds = np.arange(self.n_stars)
        seeds = np.asarray(seeds)
        self.batch = None
        if self.mine:
            self.batch = BatchRejection([stars[k] for k in self.mine], cache, precision=precision,
                                        jitter=jitter, max_out=max_out, seeds=seeds[self.mine],
                                        chunk=chunk)

    def run(self, row0=0, count=None, stream=None):
        if self.batch is not None:
            self.batch.run(row0=row0, count=count, stream=stream)
        return self

    def results(self):
        """(global star indices, counts, [indices], [ln L]) of this rank's stars."""
        if self.batch is None:
            return [], np.zeros(0, dtype=np.int64), [], []
        counts, idx, ll = self.batch.results()
        return list(self.mine), counts, idx, ll

    def gather(self):
        """(counts, [indices per star], [ln L per star]) of all stars, in star
        order, on every rank."""
        import torch.distributed as dist
        local = self.results()
        if self.world == 1 or not dist.is_initialized():
            parts = [local]
        else:
            parts = [None] * self.world
            dist.all_gather_object(parts, local, group=self.group)
        counts = np.zeros(self.n_stars, dtype=np.int64)
        idx = [None] * self.n_stars
        ll = [None] * self.n_stars
        for ks, c, i, l in parts:
            for j, k in enumerate(ks):
                counts[k] = c[j]
                idx[k] = i[j]
                ll[k] = l[j]
        return counts, idx, ll
