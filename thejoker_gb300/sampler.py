"""TheJoker: the reference's public sampling API over the GPU helper.

Mirrors thejoker/thejoker.py:23-370 and the in-memory orchestration of
thejoker/likelihood_helpers.py:40-229.  The ln L values stay on the device;
the acceptance test exp(lls - lls.max()) > uu runs on the device against the
caller's own uniform draws (reproduced from the generator's PCG64 state, or
uploaded for other bit generators), and the generator is advanced exactly as
``rng.uniform(size=len(lls))`` would advance it.
"""
import numpy as np
import torch

from . import device as dev
from .data import validate_prepare_data
from .helper import GPUJokerHelper
from .prior import JokerPrior
from .samples import JokerSamples

__all__ = ["TheJoker"]


class TheJoker:
    """A custom Monte-Carlo sampler for two-body systems (thejoker.py:23-80).

    ``pool`` is accepted for interface parity and unused: the whole batch runs
    on one GPU.  ``precision`` selects the likelihood kernel ("fp64" matches
    the reference to 1e-9 relative; "mixed" is the fast path).
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

    # -------------------------------------------------------------- likelihood
    def marginal_ln_likelihood(self, data, prior_samples, n_batches=None, in_memory=True):
        """Marginal ln-likelihood at each prior sample (thejoker.py:93-138)."""
        helper = self._make_joker_helper(data)
        return helper.batch_marginal_ln_likelihood(self._packed(prior_samples, helper))

    # -------------------------------------------------------------- acceptance
    def _accept_device(self, st, n, max_out):
        """Indices (ascending, at most max_out) with exp(lnl - max) > uu, uu the
        next n uniforms of self.rng; advances self.rng past them.  Mixed ln L
        go through the refined pass, which keeps what the FP64 path keeps."""
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
            out_idx, _, counts, _, _ = dev.accept_refined(st.stars, st.cache, st.lnl, st.err,
                                                         st.bound_keys, [seg], **kw)
        if pcg is not None:
            dev.pcg64_advance_generator(self.rng, n)
        count = int(counts[0].item())
        return out_idx[:min(count, max_out)].cpu().numpy()

    def _device_state(self, helper, chunk_dev):
        """Prior cache, ln L buffer and running maxima for one call."""
        return _CallState(helper, chunk_dev)

    def _full_samples(self, helper, chunk, n_linear_samples):
        raw, _ = helper.batch_get_posterior_samples(chunk, n_linear_samples, self.rng)
        return JokerSamples.unpack(raw, helper.internal_units, t_ref=helper.data.t_ref,
                                   poly_trend=self.prior.poly_trend,
                                   n_offsets=self.prior.n_offsets)

    def rejection_sample(self, data, prior_samples, n_prior_samples=None,
                         max_posterior_samples=None, n_linear_samples=1, return_logprobs=False,
                         return_all_logprobs=False, n_batches=None, randomize_prior_order=False,
                         in_memory=True):
        """Rejection sampling over prior samples (thejoker.py:140-257,
        likelihood_helpers.py:91-127)."""
        helper = self._make_joker_helper(data)
        if isinstance(prior_samples, int):
            prior_samples = self.prior.sample(size=prior_samples, rng=self.rng,
                                              return_logprobs=return_logprobs)
        ln_prior = None
        if isinstance(prior_samples, JokerSamples) and return_logprobs and \
                "ln_prior" in prior_samples:
            ln_prior = prior_samples["ln_prior"]
        chunk = self._packed(prior_samples, helper)
        if n_prior_samples is not None:
            chunk = chunk[:n_prior_samples]
        S = chunk.shape[0]
        if max_posterior_samples is None:
            max_posterior_samples = S
        d_chunk = torch.from_numpy(chunk).pin_memory().to("cuda", non_blocking=True)
        st = self._device_state(helper, d_chunk)
        st.evaluate(0, S)
        good = self._accept_device(st, S, max_posterior_samples)
        lnl = st.lnl
        samples = self._full_samples(helper, chunk[good], n_linear_samples)
        if return_logprobs:
            lls = lnl.cpu().numpy()
            if ln_prior is not None:
                samples["ln_prior"] = np.repeat(ln_prior[good], n_linear_samples)
            samples["ln_likelihood"] = np.repeat(lls[good], n_linear_samples)
        if return_all_logprobs:
            return samples, lnl.cpu().numpy()
        return samples

    def iterative_rejection_sample(self, data, prior_samples, n_requested_samples,
                                   max_prior_samples=None, n_linear_samples=1,
                                   return_logprobs=False, n_batches=None,
                                   randomize_prior_order=False, init_batch_size=None,
                                   growth_factor=128, in_memory=True):
        """Adaptive rejection sampling (thejoker.py:259-370,
        likelihood_helpers.py:130-229): batches grow until enough samples pass;
        every round redraws the uniforms for all ln L computed so far."""
        helper = self._make_joker_helper(data)
        chunk = self._packed(prior_samples, helper)
        if max_prior_samples is not None:
            chunk = chunk[:max_prior_samples]
        n_total = chunk.shape[0]
        maxiter, safety_factor = 128, 1
        n_process = growth_factor * n_requested_samples if init_batch_size is None \
            else init_batch_size
        if n_process > n_total:
            raise ValueError("Prior sample library not big enough! For iterative sampling, you "
                             "have to have at least growth_factor * n_requested_samples = "
                             f"{growth_factor * n_requested_samples} samples in the prior "
                             f"samples cache file. You have, or have limited to, {n_total} "
                             "samples.")
        d_chunk = torch.from_numpy(chunk).pin_memory().to("cuda", non_blocking=True)
        st = self._device_state(helper, d_chunk)
        lnl_all = st.lnl
        start = 0
        good = None
        for i in range(maxiter):
            st.evaluate(start, n_process)
            n_evals = start + n_process
            if not torch.isfinite(lnl_all[:n_evals]).all():
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
        samples = self._full_samples(helper, chunk[good], n_linear_samples)
        if return_logprobs:
            samples["ln_likelihood"] = np.repeat(lnl_all[good].cpu().numpy(), n_linear_samples)
        return samples



class _CallState:
    """Device state of one sampling call: the prior cache (all rows), the ln L
    buffer, its error bounds (mixed precision) and the running maxima."""

    def __init__(self, helper, chunk_dev):
        S = chunk_dev.shape[0]
        self.stars = helper.stars
        self.precision = helper.precision
        self.cache = dev.PriorCache.from_samples(chunk_dev)
        self.lnl = torch.empty(S, dtype=torch.float64, device="cuda")
        self.max_keys = dev.MaxKeys(1)
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
