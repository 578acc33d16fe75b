"""Batched rejection sampling: many stars against one device-resident prior
cache.

This is the GPU form of running the reference's ``rejection_sample`` once per
star (thejoker/thejoker.py:140-257, likelihood_helpers.py:91-127) over a
shared prior cache.  The reference would loop over stars and map each star's
samples over a process pool (multiproc_helpers.py:17-60).  Here stars are
taken in groups.  Each group is one persistent launch over (star,
sample-chunk) work items, stars ordered by epoch count, largest first. The
acceptance pass follows over the group's ln L buffers, with each star's own
PCG64 uniform stream regenerated on the device.  With mixed precision the
pass is refined to the FP64 decisions.  Per star the result is the number of
accepted samples and the first ``max_out`` accepted indices, in ascending
order, with their ln L.
"""
import numpy as np
import torch

from . import device as dev

__all__ = ["BatchRejection", "star_record"]


def star_record(t, rv, rv_err, prior, t_ref=None):
    """The per-star dict a StarTable takes, for a single data source."""
    from .data import RVData, get_trend_design_matrix
    data = RVData(t, rv, rv_err, t_ref=t_ref)
    mu, lam, kp = prior.linear_prior_arrays()
    return dict(t=data._t_bmjd, rv=data.rv, ivar=data.ivar, t_ref=data._t_ref_bmjd,
                trend_M=get_trend_design_matrix(data, None, prior.poly_trend), mu=mu, lam=lam,
                k_prior=kp)


class BatchRejection:
    """Rejection sampling of ``stars`` (dicts as StarTable takes) against a
    PriorCache.

    precision: "mixed_fast" (default: FP32-sum ln L with the first acceptance
    pass fused into its kernel, refined to the FP64 decisions), "mixed" (the
    float-float kernel and separate acceptance scans, same decisions) or
    "fp64".  group: stars per launch (bounded by device memory: 12 bytes per
    star and sample for the mixed path).  seeds: one seed per star for its
    numpy PCG64 generator (its first ``n`` uniforms are the star's ``uu``).
    chunk: samples per ln L work item (None: the autotuned size, autotune.py).
    early_exit (fused path, at most three linear parameters): warps whose
    samples the partial epoch sums put out of reach stop early; the kept rows
    and their ln L are the same.
    """

    def __init__(self, stars, cache, precision="mixed_fast", jitter="reference", group=None,
                 max_out=256, seeds=None, chunk=None, timing=False, early_exit=False):
        self.table = stars if isinstance(stars, dev.StarTable) else dev.StarTable(stars,
                                                                                  jitter=jitter)
        self.cache = cache
        self.precision = precision
        self.n_stars = self.table.n_stars
        self.max_out = int(max_out)
        if chunk is None:                      # the autotuned work-item size
            from .autotune import chunk_for
            chunk = chunk_for(self.table.n_linear, self.table.jitter, precision,
                              self.table.n_epochs)
        self.chunk = int(chunk)
        S = cache.size
        if group is None:
            per = S * (12 if precision != "fp64" else 8)
            free, _ = torch.cuda.mem_get_info()
            group = max(1, min(self.n_stars, int(0.6 * free // max(per, 1))))
        self.group = int(group)
        if seeds is None:
            seeds = np.arange(self.n_stars)
        self.pcg = []
        for sd in seeds:
            g = np.random.default_rng(int(sd))
            self.pcg.append(dev.pcg64_state(g))
        G = self.group
        self.lnl = torch.empty((G, S), dtype=torch.float64, device="cuda")
        self.err = torch.empty((G, S), dtype=torch.float32, device="cuda") \
            if precision != "fp64" else None
        self.keys = dev.MaxKeys(G)
        self.bkeys = dev.MaxKeys(2 * G) if precision != "fp64" else None
        # "mixed_fast": the first acceptance pass runs inside the ln L kernel
        # (joker_lnl_fused), leaving one candidate bit per sample
        self.fused = dev.fused_available(self.table, precision)
        self.early_exit = bool(early_exit)
        if self.fused:
            self.pcg_dev = dev.pcg_table(self.pcg)
            self.cand_ld, self.cand = dev.cand_words(G, S)
        self.out_idx = torch.empty(self.n_stars * self.max_out, dtype=torch.int64, device="cuda")
        self.out_lnl = torch.empty(self.n_stars * self.max_out, dtype=torch.float64,
                                   device="cuda")
        self.counts = torch.zeros(self.n_stars, dtype=torch.int64, device="cuda")
        self.n_refined = 0
        # CUDA events around each group's ln L launch (for kernel timing)
        self.timing = timing
        self.lnl_events = []

    def run(self, row0=0, count=None, stream=None):
        """Evaluate every star over cache rows [row0, row0 + count) and accept.
        Results stay on the device (``out_idx``, ``out_lnl``, ``counts``)."""
        S = self.cache.size - row0 if count is None else int(count)
        refined = torch.zeros(1, dtype=torch.int64, device="cuda")
        self.lnl_events = []
        for g0 in range(0, self.n_stars, self.group):
            n = min(self.group, self.n_stars - g0)
            self.keys.t.zero_()
            if self.bkeys is not None:
                self.bkeys.t.zero_()
            lnl = self.lnl[:n, :S]
            err = self.err[:n, :S] if self.err is not None else None
            out = self.lnl[:n]
            if self.timing:
                ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                ev[0].record(stream)
            if self.fused:
                dev.lnl_fused(self.table, self.cache, out, self.err[:n], self.bkeys,
                              self.pcg_dev[g0:g0 + n], self.cand, self.cand_ld, star0=g0,
                              n_sel=n, row0=row0, count=S, max_keys=self.keys,
                              chunk=min(self.chunk, 8192), early_exit=self.early_exit,
                              stream=stream)
            else:
                dev.lnl(self.table, self.cache, out, precision=self.precision, star0=g0,
                        n_sel=n, row0=row0, count=S, max_keys=self.keys,
                        err=self.err[:n] if err is not None else None, bound_keys=self.bkeys,
                        chunk=self.chunk, stream=stream)
            if self.timing:
                ev[1].record(stream)
                self.lnl_events.append(ev)
            ld = self.lnl.shape[1]
            segs = []
            for k in range(n):
                st, inc = self.pcg[g0 + k]
                segs.append(dict(lnl_off=k * ld, n=S, idx_base=row0,
                                 out_off=(g0 + k) * self.max_out, max_out=self.max_out,
                                 max_slot=k, star=g0 + k, row0=row0, pcg=(st, inc, 0)))
            cnt = self.counts[g0:g0 + n]
            if self.precision == "fp64":
                dev.accept(self.lnl.view(-1), self.keys, segs, u_source="pcg64",
                           out_idx=self.out_idx, out_lnl=self.out_lnl, counts=cnt,
                           stream=stream)
            elif self.fused:
                _, _, _, _, nref = dev.accept_fused(
                    self.table, self.cache, self.lnl.view(-1), self.err.view(-1), self.bkeys,
                    self.cand, self.cand_ld, segs, out_idx=self.out_idx, out_lnl=self.out_lnl,
                    counts=cnt, stream=stream)
                refined += nref
            else:
                _, _, _, _, nref = dev.accept_refined(
                    self.table, self.cache, self.lnl.view(-1), self.err.view(-1), self.bkeys,
                    segs, u_source="pcg64", out_idx=self.out_idx, out_lnl=self.out_lnl,
                    counts=cnt, stream=stream)
                refined += nref
        self._refined = refined
        return self

    def results(self):
        """(counts, [indices per star], [ln L per star]) on the host."""
        counts = self.counts.cpu().numpy()
        idx = self.out_idx.view(self.n_stars, self.max_out).cpu().numpy()
        ll = self.out_lnl.view(self.n_stars, self.max_out).cpu().numpy()
        k = np.minimum(counts, self.max_out)
        return counts, [idx[i, :k[i]] for i in range(self.n_stars)], \
            [ll[i, :k[i]] for i in range(self.n_stars)]

    def lnl_ms(self):
        """Device time of the last run's ln L launches (needs timing=True)."""
        return sum(a.elapsed_time(b) for a, b in self.lnl_events)

    @property
    def n_refined_last(self):
        """Samples the last run() re-evaluated in FP64 (mixed precisions: the
        candidates for each star's maximum, the undecided samples and the kept
        samples whose bound exceeds JOKER_MIXED_LNL_TOL)."""
        return int(self._refined.item())
