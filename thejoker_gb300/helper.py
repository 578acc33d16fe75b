"""GPUJokerHelper: the GB300 drop-in for the reference's CJokerHelper.

It exposes the surface the reference's sampling code uses
(thejoker/src/fast_likelihood.pyx:70-576): ``packed_order``,
``internal_units``, ``data``, ``prior``, ``batch_marginal_ln_likelihood``,
``batch_get_posterior_samples`` and ``test_likelihood_worker``, and it pickles
by its constructor arguments (``__reduce__``, :122-123).  The likelihood runs
in libjoker_gb300 on the GPU; there is no CPU path.
"""
import numpy as np
import torch

from . import device as dev
from .linear import multivariate_normal_draws
from .samples import PACKED_ORDER

__all__ = ["GPUJokerHelper", "band_refined_lnl"]


def band_refined_lnl(stars, cache, out, precision, star=0, stream=None):
    """Mixed-precision ln L of one star over every cache row into ``out`` (a
    float64 CUDA tensor of cache.size values), with the band refinement: the
    samples whose interval reaches within JOKER_MIXED_LNL_BAND of the star's
    FP64 maximum and whose bound exceeds JOKER_MIXED_LNL_TOL are re-evaluated
    in FP64, so every returned value within the band of the maximum is within
    the tolerance of the FP64 path's.  Returns (per-sample bounds, FP64
    maximum keys, number of re-evaluated samples)."""
    S = cache.size
    err = torch.empty((1, S), dtype=torch.float32, device=out.device)
    bkeys = dev.MaxKeys(2)
    dev.lnl(stars, cache, out.view(1, S), precision=precision, star0=star, n_sel=1,
            err=err, bound_keys=bkeys, stream=stream)
    seg = [dict(lnl_off=0, n=S, out_off=0, max_out=0, max_slot=0, star=star, row0=0)]
    exact, n1 = dev.refine_max(stars, cache, out, err.view(-1), bkeys, seg, stream=stream)
    n2 = dev.refine_band(stars, cache, out, err.view(-1), exact, seg, stream=stream)
    return err.view(-1), exact, n1 + n2


class GPUJokerHelper:
    """Per-star likelihood helper.

    Parameters
    ----------
    data : RVData
    prior : JokerPrior
    trend_M : (n_times, n_linear - 1) float64 design matrix of the linear
        parameters other than K (as built by ``validate_prepare_data``).
    precision : "fp64" (default; the drop-in), "mixed" or "mixed_accurate".
    jitter : "reference" (default; s is ignored as in CJokerHelper) or
        "applied" (ivar / (1 + s^2 ivar), as the reference's NumPy test oracle).
    """

    def __init__(self, data, prior, trend_M, precision="fp64", jitter="reference"):
        self.prior = prior
        self.data = data
        self.precision = precision
        self.jitter = jitter
        unit = data.rv_unit
        self.internal_units = {"P": "d", "e": "", "omega": "rad", "M0": "rad", "s": unit,
                               "K": unit, "v0": unit}
        for name in prior._offset_names:
            self.internal_units[name] = unit
        for i, name in enumerate(prior._v_trend_names):
            self.internal_units.setdefault(name, f"{unit} / d^{i}")
        self.packed_order = list(PACKED_ORDER)
        self.n_times = len(data)
        self.n_linear = prior.n_linear
        trend_M = np.ascontiguousarray(trend_M, dtype=np.float64)
        if trend_M.ndim != 2 or trend_M.shape[0] != self.n_times or \
                trend_M.shape[1] != self.n_linear - 1:
            raise ValueError("Invalid design matrix shape: {}, expected: {}".format(
                trend_M.shape, (self.n_times, self.n_linear - 1)))
        self.trend_M = trend_M
        self.mu, self.lam, self.k_prior = prior.linear_prior_arrays()
        self._stars = dev.StarTable([dict(
            t=data._t_bmjd, rv=data.rv, ivar=data.ivar, t_ref=data._t_ref_bmjd,
            trend_M=trend_M, mu=self.mu, lam=self.lam, k_prior=self.k_prior)], jitter=jitter)

    def __reduce__(self):
        return (GPUJokerHelper, (self.data, self.prior, self.trend_M, self.precision, self.jitter))

    @property
    def stars(self):
        return self._stars

    # ------------------------------------------------------------ likelihood
    def batch_marginal_ln_likelihood_device(self, chunk, out=None, stream=None):
        """ln L for a (S, 5) float64 CUDA tensor; returns a CUDA tensor."""
        if chunk.dtype != torch.float64 or chunk.dim() != 2 or chunk.shape[1] != 5:
            raise ValueError("chunk must be float64 with shape (n_samples, 5)")
        chunk = chunk.contiguous()
        S = chunk.shape[0]
        if out is None:
            out = torch.empty(S, dtype=torch.float64, device=chunk.device)
        if self.precision == "fp64":
            import ctypes
            from . import _native as nat
            nat.check(nat.lib().joker_batch_marginal_ln_likelihood(
                self._stars.handle, 0, ctypes.c_void_p(chunk.data_ptr()), S,
                ctypes.c_void_p(out.data_ptr()), dev.stream_handle(stream)),
                "joker_batch_marginal_ln_likelihood")
        else:
            cache = dev.PriorCache.from_samples(chunk, stream=stream)
            if self.precision == "mixed_fp64_tail":
                # this variant states no per-sample bound, so nothing is refined
                dev.lnl(self._stars, cache, out.view(1, S), precision=self.precision,
                        stream=stream)
            else:
                band_refined_lnl(self._stars, cache, out, self.precision, stream=stream)
        return out

    def batch_marginal_ln_likelihood(self, chunk):
        """Marginal ln-likelihood per row of ``chunk`` (S x 5: P, e, omega, M0, s),
        the drop-in for CJokerHelper.batch_marginal_ln_likelihood (:428-469)."""
        chunk = np.ascontiguousarray(chunk, dtype=np.float64)
        if chunk.ndim != 2 or chunk.shape[1] != 5:
            raise ValueError("chunk must have shape (n_samples, 5)")
        if chunk.shape[0] == 0:
            return np.zeros(0)
        d = torch.from_numpy(chunk).pin_memory().to("cuda", non_blocking=True)
        out = self.batch_marginal_ln_likelihood_device(d)
        return out.cpu().numpy()

    def test_likelihood_worker(self, chunk_row):
        """ln L of one packed sample (fast_likelihood.pyx:547-576)."""
        return float(self.batch_marginal_ln_likelihood(np.asarray(chunk_row)[None, :])[0])

    # ------------------------------------------------------ linear parameters
    def batch_get_posterior_samples(self, chunk, n_linear_samples_per, rng):
        """(samples (S*n, 5 + L), ll (S*n)) as fast_likelihood.pyx:471-545: the
        posterior mean and covariance of the linear parameters of every row
        come from the device (joker_linear_posterior, FP64, the K prior
        variance unclipped as there); the draws use ``rng`` in the
        reference's order (one multivariate_normal block per row)."""
        chunk = np.ascontiguousarray(chunk, dtype=np.float64)
        if chunk.ndim != 2 or chunk.shape[1] != 5:
            raise ValueError("chunk must have shape (n_samples, 5)")
        S, L, n = chunk.shape[0], self.n_linear, int(n_linear_samples_per)
        if S == 0:
            return np.zeros((0, 5 + L)), np.zeros(0)
        d = torch.from_numpy(chunk).to("cuda")
        a, A, ll = dev.linear_posterior(self._stars, dev.PriorCache.view(d), 0, k_clip=False)
        draws = multivariate_normal_draws(rng, a.cpu().numpy(), A.cpu().numpy(), n)
        samples = np.empty((S, n, 5 + L))
        samples[:, :, :5] = chunk[:, None, :]
        samples[:, :, 5:] = draws
        return samples.reshape(S * n, 5 + L), np.repeat(ll.cpu().numpy(), n)
