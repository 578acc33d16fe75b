"""Rejection sampling from a prior chunk in host memory.

The reference's entry point takes a packed (S, 5) prior chunk on the host
(``batch_marginal_ln_likelihood(chunk)``, thejoker/src/fast_likelihood.pyx
:428-469, then the acceptance of likelihood_helpers.py:107-109).  Two ways to
bring it to the device:

- ``zero_copy`` (default for a pinned chunk): the ln L kernel reads the packed
  rows directly through the chunk's mapped device address and prepares each
  sample in registers (a cache view, ``PriorCache.view``).  The host link
  streams 40 bytes per sample while the kernel computes; there is no staging
  copy, no preparation pass and no device copy of the chunk.  The FP64
  re-evaluations of the acceptance pass read the few rows they need the same
  way.
- staged: the chunk is copied in slices of ``slice_rows`` rows on a copy
  stream, double-buffered, while the previous slice is prepared into a device
  cache and evaluated on a compute stream.

Either way the acceptance pass runs once, after every sample's ln L, because
it needs each star's maximum over all samples; only the accepted indices (and
the counts) come back to the host.
"""
import numpy as np
import torch

from . import device as dev

__all__ = ["HostRejection"]


class HostRejection:
    """Reusable buffers for rejection sampling of ``table``'s stars against
    host prior chunks of up to ``capacity`` rows."""

    def __init__(self, table, capacity, precision="mixed_fast", slice_rows=1 << 24, max_out=256,
                 zero_copy=True, chunk=None):
        self.table = table
        self.precision = precision
        self.capacity = int(capacity)
        self.slice_rows = int(min(slice_rows, capacity))
        self.max_out = int(max_out)
        self.zero_copy = bool(zero_copy)
        if chunk is None:                      # the autotuned work-item size
            from .autotune import chunk_for
            chunk = chunk_for(table.n_linear, table.jitter, precision, table.n_epochs)
        self.chunk = int(chunk)
        n = table.n_stars
        self.cache = None if self.zero_copy else dev.PriorCache(self.capacity)
        self.stage = [] if self.zero_copy else \
            [torch.empty((self.slice_rows, 5), dtype=torch.float64, device="cuda")
             for _ in range(2)]
        self.lnl = torch.empty((n, self.capacity), dtype=torch.float64, device="cuda")
        mixed = precision != "fp64"
        self.err = torch.empty((n, self.capacity), dtype=torch.float32, device="cuda") \
            if mixed else None
        self.keys = dev.MaxKeys(n)
        self.bkeys = dev.MaxKeys(2 * n) if mixed else None
        # "mixed_fast": the first acceptance pass fused into the ln L kernel
        # (slices must then start on multiples of 32 samples)
        self.fused = dev.fused_available(table, precision) and self.slice_rows % 32 == 0
        if self.fused:
            self.cand_ld, self.cand = dev.cand_words(n, self.capacity)
            self.chunk = min(self.chunk, 8192)
        self.out_idx = torch.empty(n * self.max_out, dtype=torch.int64, device="cuda")
        self.counts = torch.empty(n, dtype=torch.int64, device="cuda")
        self.copy_stream = torch.cuda.Stream()
        self.compute_stream = torch.cuda.Stream()
        self.copied = [torch.cuda.Event() for _ in range(2)]
        self.freed = [torch.cuda.Event() for _ in range(2)]
        self.host_idx = torch.empty(n * self.max_out, dtype=torch.int64).pin_memory()
        self.host_counts = torch.empty(n, dtype=torch.int64).pin_memory()
        self.d2h_bytes = 0

    def _lnl(self, cache, row0, count, pcg, ks):
        if self.fused:
            dev.lnl_fused(self.table, cache, self.lnl, self.err, self.bkeys, pcg, self.cand,
                          self.cand_ld, row0=row0, count=count, first=row0,
                          max_keys=self.keys, chunk=self.chunk, out_offset=row0, stream=ks)
        else:
            dev.lnl(self.table, cache, self.lnl, precision=self.precision, row0=row0,
                    count=count, max_keys=self.keys, err=self.err, bound_keys=self.bkeys,
                    out_offset=row0, chunk=self.chunk, stream=ks)

    def _staged(self, host_chunk, S, ks, pcg):
        cs = self.copy_stream
        n_slices = (S + self.slice_rows - 1) // self.slice_rows
        for k in range(n_slices):
            a = k * self.slice_rows
            b = min(S, a + self.slice_rows)
            buf = self.stage[k % 2]
            with torch.cuda.stream(cs):
                if k >= 2:
                    cs.wait_event(self.freed[k % 2])
                buf[: b - a].copy_(host_chunk[a:b], non_blocking=True)
                self.copied[k % 2].record(cs)
            with torch.cuda.stream(ks):
                ks.wait_event(self.copied[k % 2])
                self.cache.load(buf[: b - a], row0=a, stream=ks)
                self.freed[k % 2].record(ks)
                self._lnl(self.cache, a, b - a, pcg, ks)
        return self.cache

    def run(self, host_chunk, pcg_states):
        """Accepted indices per star for an (S, 5) float64 host tensor (pinned
        for the zero-copy path; pinned here otherwise).

        ``pcg_states``: per star (state, inc) of its numpy PCG64 generator; the
        star's uniforms are that generator's first S draws.  Returns (counts,
        list of index arrays, the first max_out per star in ascending order).
        """
        S = host_chunk.shape[0]
        if S > self.capacity:
            raise ValueError("chunk larger than the capacity")
        if not host_chunk.is_pinned():
            host_chunk = host_chunk.pin_memory()
        ks = self.compute_stream
        ks.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(ks):
            self.keys.t.zero_()
            if self.bkeys is not None:
                self.bkeys.t.zero_()
        n = self.table.n_stars
        pcg = None
        if self.fused:
            with torch.cuda.stream(ks):
                pcg = dev.pcg_table([pcg_states[s] for s in range(n)])
        if self.zero_copy:
            cache = dev.PriorCache.view(host_chunk.contiguous())
            with torch.cuda.stream(ks):
                self._lnl(cache, 0, S, pcg, ks)
        else:
            cache = self._staged(host_chunk, S, ks, pcg)
        segs = []
        for s in range(n):
            st, inc = pcg_states[s]
            segs.append(dict(lnl_off=s * self.capacity, n=S, idx_base=0,
                             out_off=s * self.max_out, max_out=self.max_out, max_slot=s,
                             star=s, row0=0, pcg=(st, inc, 0)))
        with torch.cuda.stream(ks):
            if self.err is None:
                dev.accept(self.lnl.view(-1), self.keys, segs, out_idx=self.out_idx,
                           counts=self.counts, stream=ks)
            elif self.fused:
                dev.accept_fused(self.table, cache, self.lnl.view(-1), self.err.view(-1),
                                 self.bkeys, self.cand, self.cand_ld, segs,
                                 out_idx=self.out_idx, counts=self.counts, stream=ks)
            else:
                dev.accept_refined(self.table, cache, self.lnl.view(-1), self.err.view(-1),
                                   self.bkeys, segs, out_idx=self.out_idx, counts=self.counts,
                                   stream=ks)
            self.host_counts.copy_(self.counts, non_blocking=True)
        ks.synchronize()
        counts = self.host_counts.numpy().copy()
        keep = np.minimum(counts, self.max_out)
        # bring back only the accepted indices
        with torch.cuda.stream(ks):
            if n * self.max_out * 8 <= (64 << 20):
                self.host_idx.copy_(self.out_idx, non_blocking=True)
                self.d2h_bytes = n * self.max_out * 8 + 8 * n
            else:
                for s in range(n):
                    o = s * self.max_out
                    self.host_idx[o:o + keep[s]].copy_(self.out_idx[o:o + keep[s]],
                                                       non_blocking=True)
                self.d2h_bytes = int(keep.sum()) * 8 + 8 * n
        ks.synchronize()
        idx = self.host_idx.numpy().reshape(n, self.max_out)
        return counts, [idx[s, :keep[s]].copy() for s in range(n)]
