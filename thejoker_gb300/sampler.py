"""TheJoker: the reference's public sampling API over the GPU helper.

Mirrors thejoker/thejoker.py:23-370 and both orchestrations behind it:

* ``in_memory=True``: thejoker/likelihood_helpers.py:40-229 (the prior
  samples in memory, the linear parameters drawn from ``self.rng``);
* ``in_memory=False``, the reference's default: thejoker/multiproc_helpers.py
  :17-427 (the prior samples passed through a cache file and a processing
  pool): an optional random prefix order ``rng.choice(n_total, size,
  replace=False)``, safety factor 4 in the iterative growth rule, and the
  linear parameters drawn per pool task from generators spawned off the
  caller's seed sequence, the tasks split as utils.batch_tasks splits them.

Here both run on one GPU and the samples never leave device memory (no cache
file, no pool); only the schedule, the random streams and the results of each
path are reproduced.  The ln L values stay on the device; the acceptance
test exp(lls - lls.max()) > uu runs on the device against the caller's own
uniform draws (reproduced from the generator's PCG64 state, or uploaded for
other bit generators), and the generator is advanced exactly as
``rng.uniform(size=len(lls))`` would advance it.
"""
import numpy as np
import torch

from . import device as dev
from .data import validate_prepare_data
from .helper import GPUJokerHelper
from .prior import JokerPrior
from .samples import JokerSamples

__all__ = ["TheJoker", "batch_tasks"]


def batch_tasks(n_tasks, n_batches, arr):
    """The slices of ``arr`` the reference's pool tasks get
    (thejoker/utils.py:22-72): ``n_batches`` contiguous runs, the first
    ``n_tasks % n_batches`` one longer; a single run when there are fewer
    tasks than batches."""
    arr = np.asarray(arr)
    if n_batches > 0 and n_tasks >= n_batches:
        base, rmdr = divmod(int(n_tasks), int(n_batches))
        out, i1 = [], 0
        for i in range(n_batches):
            i2 = i1 + base + (1 if i < rmdr else 0)
            out.append(arr[i1:i2])
            i1 = i2
        return out
    return [arr[0:n_tasks]]


class TheJoker:
    """A custom Monte-Carlo sampler for two-body systems (thejoker.py:23-80).

    ``pool``: any object with ``map`` and ``close``, as the reference takes.
    Nothing is mapped over it (the whole batch runs on one GPU); its ``size``
    (0 when absent) sets the default number of tasks of the file/pool path,
    max(1, pool.size), as in multiproc_helpers.py:39-40, and with it how
    the linear parameters' random streams are split.  ``precision`` selects
    the likelihood kernel ("fp64" matches the reference to 1e-9 relative;
    "mixed" is the fast path: its accepted samples are the FP64 path's, and
    every ln L it returns within JOKER_MIXED_LNL_BAND of the maximum is within
    JOKER_MIXED_LNL_TOL of the FP64 value).
    """

    def __init__(self, prior, pool=None, rng=None, tempfile_path=None, precision="fp64",
                 jitter="reference"):
        if pool is not None and (not hasattr(pool, "map") or not hasattr(pool, "close")):
            raise TypeError("Input pool object must have .map() and .close() methods.")
        self.pool = pool
        if rng is None:
            rng = np.random.default_rng()
        elif not isinstance(rng, np.random.Generator):
            raise TypeError("The input random number generator must be a "
                            "numpy.random.Generator instance.")
        self.rng = rng
        if not isinstance(prior, JokerPrior):
            raise TypeError("The input prior must be a JokerPrior instance.")
        self.prior = prior
        self.precision = precision
        self.jitter = jitter
        self.tempfile_path = tempfile_path

    def _make_joker_helper(self, data):
        all_data, ids, trend_M = validate_prepare_data(data, self.prior.poly_trend,
                                                       self.prior.n_offsets)
        return GPUJokerHelper(all_data, self.prior, trend_M, precision=self.precision,
                              jitter=self.jitter)

    @staticmethod
    def _packed(prior_samples, helper):
        if isinstance(prior_samples, JokerSamples):
            chunk, _ = prior_samples.pack(names=helper.packed_order)
            return chunk
        if isinstance(prior_samples, str):
            return JokerSamples.read(prior_samples).pack(names=helper.packed_order)[0]
        return np.ascontiguousarray(prior_samples, dtype=np.float64)

    @staticmethod
    def _file_samples(prior_samples):
        """The prior samples of the file/pool path: a filename or a
        JokerSamples, as the reference's tempfile_decorator accepts
        (utils.py:248-302)."""
        if isinstance(prior_samples, str):
            return JokerSamples.read(prior_samples)
        if not isinstance(prior_samples, JokerSamples):
            raise TypeError("prior_samples_file must either be a string filename specifying "
                            "a cache file contining prior samples, or must be a JokerSamples "
                            f"instance, not: {type(prior_samples)}")
        return prior_samples

    def _n_tasks(self, n_batches):
        if n_batches is not None:
            return int(n_batches)
        return max(1, int(getattr(self.pool, "size", 0) or 0))

    # -------------------------------------------------------------- likelihood
    def marginal_ln_likelihood(self, data, prior_samples, n_batches=None, in_memory=False):
        """Marginal ln-likelihood at each prior sample (thejoker.py:93-138).
        Both paths give the same values (the pool path concatenates its tasks'
        results in order)."""
        helper = self._make_joker_helper(data)
        if not in_memory:
            prior_samples = self._file_samples(prior_samples)
        return helper.batch_marginal_ln_likelihood(self._packed(prior_samples, helper))

    # -------------------------------------------------------------- acceptance
    def _accept_device(self, st, n, max_out):
        """Indices (ascending, at most max_out) with exp(lnl - max) > uu, uu the
        next n uniforms of self.rng; advances self.rng past them.  Mixed ln L
        go through the refined pass, which keeps what the FP64 path keeps, and
        leaves the FP64 maximum in ``st.exact``."""
        pcg = dev.pcg64_state(self.rng)
        seg = dict(lnl_off=0, n=n, idx_base=0, out_off=0, max_out=max_out, max_slot=0, star=0,
                   row0=0)
        kw = {}
        if pcg is not None:
            seg["pcg"] = (pcg[0], pcg[1], 0)
            kw["u_source"] = "pcg64"
        else:
            seg["u_off"] = 0
            kw["u_source"] = "array"
            kw["u"] = torch.from_numpy(self.rng.uniform(size=n)).cuda()
        if st.err is None:
            out_idx, _, counts = dev.accept(st.lnl, st.max_keys, [seg], **kw)
        else:
            out_idx, _, counts, st.exact, _ = dev.accept_refined(
                st.stars, st.cache, st.lnl, st.err, st.bound_keys, [seg], **kw)
        if pcg is not None:
            dev.pcg64_advance_generator(self.rng, n)
        count = int(counts[0].item())
        return out_idx[:min(count, max_out)].cpu().numpy()

    def _all_lnl(self, st, n):
        """The first n ln L values on the host; mixed values band-refined
        against the FP64 maximum the last acceptance found."""
        if st.err is not None and st.exact is not None:
            dev.refine_band(st.stars, st.cache, st.lnl, st.err, st.exact,
                            [dict(lnl_off=0, n=n, out_off=0, max_out=0, max_slot=0, star=0,
                                  row0=0)])
        return st.lnl[:n].cpu().numpy()

    def _full_samples(self, helper, rows, n_linear_samples, rng):
        raw, _ = helper.batch_get_posterior_samples(rows, n_linear_samples, rng)
        return JokerSamples.unpack(raw, helper.internal_units, t_ref=helper.data.t_ref,
                                   poly_trend=self.prior.poly_trend,
                                   n_offsets=self.prior.n_offsets)

    def _full_samples_pool(self, helper, chunk, full_idx, n_linear_samples, n_batches):
        """make_full_samples of the pool path (multiproc_helpers.py:123-182,
        :17-60): the accepted rows split into tasks as batch_tasks splits
        them, each task's linear parameters drawn from its own generator,
        spawned off self.rng's seed sequence (self.rng itself is not
        advanced), the tasks' rows concatenated in order."""
        from numpy.random import PCG64, Generator
        tasks = batch_tasks(len(full_idx), self._n_tasks(n_batches), full_idx)
        seqs = self.rng.bit_generator._seed_seq.spawn(len(tasks))
        raws = []
        for idx, sq in zip(tasks, seqs):
            raw, _ = helper.batch_get_posterior_samples(chunk[idx], n_linear_samples,
                                                        Generator(PCG64(sq)))
            raws.append(raw)
        raw = np.concatenate(raws)
        return JokerSamples.unpack(raw, helper.internal_units, t_ref=helper.data.t_ref,
                                   poly_trend=self.prior.poly_trend,
                                   n_offsets=self.prior.n_offsets)

    def rejection_sample(self, data, prior_samples, n_prior_samples=None,
                         max_posterior_samples=None, n_linear_samples=1, return_logprobs=False,
                         return_all_logprobs=False, n_batches=None, randomize_prior_order=False,
                         in_memory=False):
        """Rejection sampling over prior samples (thejoker.py:140-257;
        likelihood_helpers.py:91-127 in memory, multiproc_helpers.py:185-286
        otherwise)."""
        helper = self._make_joker_helper(data)
        if isinstance(prior_samples, int):
            # drawn from the prior's own default generator, not self.rng, as
            # the reference does (thejoker.py:215-218)
            prior_samples = self.prior.sample(size=prior_samples,
                                              return_logprobs=return_logprobs)
        if in_memory:
            return self._rejection_inmem(helper, prior_samples, max_posterior_samples,
                                         n_linear_samples, return_logprobs, return_all_logprobs)
        return self._rejection_pool(helper, prior_samples, n_prior_samples,
                                    max_posterior_samples, n_linear_samples, return_logprobs,
                                    return_all_logprobs, n_batches, randomize_prior_order)

    def _rejection_inmem(self, helper, prior_samples, max_posterior_samples, n_linear_samples,
                         return_logprobs, return_all_logprobs):
        ln_prior = None
        if isinstance(prior_samples, JokerSamples):
            if return_logprobs:
                ln_prior = prior_samples["ln_prior"]
        elif return_logprobs:
            raise ValueError("return_logprobs=True needs the prior samples as a JokerSamples "
                             "with an ln_prior column")
        chunk = self._packed(prior_samples, helper)
        S = chunk.shape[0]
        if max_posterior_samples is None:
            max_posterior_samples = S
        st = _CallState(helper, torch.from_numpy(chunk).pin_memory().to("cuda",
                                                                          non_blocking=True))
        st.evaluate(0, S)
        good = self._accept_device(st, S, max_posterior_samples)
        samples = self._full_samples(helper, chunk[good], n_linear_samples, self.rng)
        lls = self._all_lnl(st, S) if (return_all_logprobs or ln_prior is not None) else None
        if ln_prior is not None:
            samples["ln_prior"] = np.repeat(ln_prior[good], n_linear_samples)
            samples["ln_likelihood"] = np.repeat(lls[good], n_linear_samples)
        if return_all_logprobs:
            return samples, lls
        return samples

    def _rejection_pool(self, helper, prior_samples, n_prior_samples, max_posterior_samples,
                        n_linear_samples, return_logprobs, return_all_logprobs, n_batches,
                        randomize_prior_order):
        js = self._file_samples(prior_samples)
        n_total = len(js)
        if return_logprobs and "ln_prior" not in js:
            raise RuntimeError("return_logprobs=True but ln_prior values not found in prior "
                               "cache: make sure you generate prior samples with prior.sample "
                               "(..., return_logprobs=True) before saving the prior samples.")
        if n_prior_samples is None:
            n_prior_samples = n_total
        elif n_prior_samples > n_total:
            raise ValueError("Number of prior samples to use is greater than the number of "
                             "prior samples passed, or cached to a filename specified. "
                             f"n_prior_samples={n_prior_samples} vs. "
                             f"n_total_samples={n_total}")
        if max_posterior_samples is None:
            max_posterior_samples = n_prior_samples
        chunk = self._packed(js, helper)
        idx = None
        if randomize_prior_order:
            idx = self.rng.choice(n_total, size=n_prior_samples, replace=False)
            rows = chunk[idx]
        else:
            rows = chunk[:n_prior_samples]
        S = rows.shape[0]
        st = _CallState(helper, torch.from_numpy(np.ascontiguousarray(rows)).pin_memory()
                        .to("cuda", non_blocking=True))
        st.evaluate(0, S)
        good = self._accept_device(st, S, max_posterior_samples)
        full_idx = idx[good] if idx is not None else good
        samples = self._full_samples_pool(helper, chunk, full_idx, n_linear_samples, n_batches)
        lls = self._all_lnl(st, S) if (return_all_logprobs or return_logprobs) else None
        if return_logprobs:
            samples["ln_likelihood"] = np.repeat(lls[good], n_linear_samples)
            samples["ln_prior"] = np.repeat(js["ln_prior"][full_idx], n_linear_samples)
        if return_all_logprobs:
            return samples, lls
        return samples

    def iterative_rejection_sample(self, data, prior_samples, n_requested_samples,
                                   max_prior_samples=None, n_linear_samples=1,
                                   return_logprobs=False, n_batches=None,
                                   randomize_prior_order=False, init_batch_size=None,
                                   growth_factor=128, in_memory=False):
        """Adaptive rejection sampling (thejoker.py:259-370;
        likelihood_helpers.py:130-229 in memory, multiproc_helpers.py:289-427
        otherwise): batches grow until enough samples pass; every round
        redraws the uniforms for all ln L computed so far.  As in the
        reference, the in-memory path ignores ``max_prior_samples``,
        ``n_batches`` and ``randomize_prior_order``."""
        helper = self._make_joker_helper(data)
        if in_memory:
            ln_prior = None
            if isinstance(prior_samples, JokerSamples):
                if return_logprobs:
                    ln_prior = prior_samples["ln_prior"]
            elif return_logprobs:
                raise ValueError("return_logprobs=True needs the prior samples as a "
                                 "JokerSamples with an ln_prior column")
            chunk = self._packed(prior_samples, helper)
            return self._iterative(helper, chunk, None, n_requested_samples, chunk.shape[0],
                                   n_linear_samples, ln_prior, init_batch_size, growth_factor,
                                   pool=False, n_batches=None)
        js = self._file_samples(prior_samples)
        n_total = len(js)
        if return_logprobs and "ln_prior" not in js:
            raise RuntimeError("return_logprobs=True but ln_prior values not found in prior "
                               "cache: make sure you generate prior samples with prior.sample "
                               "(..., return_logprobs=True) before saving the prior samples.")
        if max_prior_samples is None:
            max_prior_samples = n_total
        chunk = self._packed(js, helper)
        n_process = growth_factor * n_requested_samples if init_batch_size is None \
            else init_batch_size
        if n_process > max_prior_samples:
            raise ValueError(self._library_msg(growth_factor, n_requested_samples,
                                               max_prior_samples))
        all_idx = None
        if randomize_prior_order:
            all_idx = self.rng.choice(n_total, size=max_prior_samples, replace=False)
        return self._iterative(helper, chunk, all_idx, n_requested_samples, max_prior_samples,
                               n_linear_samples,
                               js["ln_prior"] if return_logprobs else None, init_batch_size,
                               growth_factor, pool=True, n_batches=n_batches)

    @staticmethod
    def _library_msg(growth_factor, n_requested_samples, n_total):
        return ("Prior sample library not big enough! For iterative sampling, you have to have "
                "at least growth_factor * n_requested_samples = "
                f"{growth_factor * n_requested_samples} samples in the prior samples cache "
                f"file. You have, or have limited to, {n_total} samples.")

    def _iterative(self, helper, chunk, all_idx, n_requested_samples, n_total, n_linear_samples,
                   ln_prior, init_batch_size, growth_factor, pool, n_batches):
        """The loop of iterative_rejection_inmem (pool=False: safety factor 1,
        the non-finite check, linear draws from self.rng) or of
        iterative_rejection_helper (pool=True: safety factor 4, no check,
        linear draws per pool task) over the library rows all_idx (rows
        0..n_total-1 when all_idx is None)."""
        maxiter = 128
        safety_factor = 4 if pool else 1
        n_process = growth_factor * n_requested_samples if init_batch_size is None \
            else init_batch_size
        if n_process > n_total:
            raise ValueError(self._library_msg(growth_factor, n_requested_samples, n_total))
        lib = chunk[all_idx] if all_idx is not None else chunk[:n_total]
        st = _CallState(helper, torch.from_numpy(np.ascontiguousarray(lib)).pin_memory()
                        .to("cuda", non_blocking=True))
        lnl_all = st.lnl
        start = 0
        good = None
        for i in range(maxiter):
            st.evaluate(start, n_process)
            n_evals = start + n_process
            if not pool and not torch.isfinite(lnl_all[:n_evals]).all():
                # the reference returns (does not raise) this error object
                return RuntimeError(f"There are NaN or Inf likelihood values in iteration step {i}!")
            good = self._accept_device(st, n_evals, n_evals)
            if len(good) == 0:
                raise RuntimeError("Failed to find any good samples!")
            n_good = len(good)
            if n_good >= n_requested_samples:
                break
            start += n_process
            n_need = n_requested_samples - n_good
            n_process = int(safety_factor * n_need / n_good * n_evals)
            if start + n_process > n_total:
                n_process = n_total - start
            if n_process <= 0:
                break
        else:
            raise RuntimeError("Hit maximum number of iterations!")
        good = good[:n_requested_samples]
        full_idx = all_idx[good] if all_idx is not None else good
        if pool:
            samples = self._full_samples_pool(helper, chunk, full_idx, n_linear_samples,
                                              n_batches)
        else:
            samples = self._full_samples(helper, chunk[full_idx], n_linear_samples, self.rng)
        if ln_prior is not None:
            lls = self._all_lnl(st, n_evals)
            samples["ln_prior"] = np.repeat(np.asarray(ln_prior)[full_idx], n_linear_samples)
            samples["ln_likelihood"] = np.repeat(lls[good], n_linear_samples)
        return samples


class _CallState:
    """Device state of one sampling call: the prior cache (all rows), the ln L
    buffer, its error bounds (mixed precision), the running maxima, and the
    FP64 maximum the last refined acceptance found."""

    def __init__(self, helper, chunk_dev):
        S = chunk_dev.shape[0]
        self.stars = helper.stars
        self.precision = helper.precision
        self.cache = dev.PriorCache.from_samples(chunk_dev)
        self.lnl = torch.empty(S, dtype=torch.float64, device="cuda")
        self.max_keys = dev.MaxKeys(1)
        self.exact = None
        if self.precision == "fp64" or self.precision == "mixed_fp64_tail":
            self.err = None
            self.bound_keys = None
        else:
            self.err = torch.empty(S, dtype=torch.float32, device="cuda")
            self.bound_keys = dev.MaxKeys(2)

    def evaluate(self, row0, count):
        if count <= 0:
            return
        out = self.lnl[row0:row0 + count].view(1, count)
        err = self.err[row0:row0 + count].view(1, count) if self.err is not None else None
        dev.lnl(self.stars, self.cache, out, precision=self.precision, row0=row0, count=count,
                max_keys=self.max_keys, err=err, bound_keys=self.bound_keys)
