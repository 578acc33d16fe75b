"""The default workload at its full size (GB300 only): one star, 40 epochs
over 3000 d, jitter applied, 2^28 prior samples drawn on the device.  At
this size the oracle cannot run; the properties checked do not depend on
the size:
- the refined mixed acceptance keeps exactly the plain FP64 path's samples
  (indices and count) against the same PCG64 uniforms;
- every kept sample's ln L is within 1e-4 of its FP64 value.
"""
import numpy as np
import pytest
import torch

from gpu_util import synth_star

pytestmark = pytest.mark.gpu

N_SAMPLES = 1 << 28


def test_full_size_mixed_keeps_the_fp64_samples(cuda):
    from thejoker_gb300 import _native as nat
    from thejoker_gb300 import device as dev
    from thejoker_gb300.batch import BatchRejection
    free, _ = torch.cuda.mem_get_info()
    if free < (48 << 30):
        pytest.skip("needs 48 GB of free device memory")
    rng = np.random.default_rng(2024)
    star = synth_star(rng, 40, base=3000.0, sig=(0.05, 0.5))
    cache = dev.PriorCache(N_SAMPLES)
    cache.sample_prior(dict(P_min=2.0, P_max=1024.0, e_alpha=0.867, e_beta=3.03,
                            s_kind=nat.JOKER_S_LOGNORMAL, s_mu=np.log(0.5), s_sigma=1.0),
                       N_SAMPLES, seed=77)
    table = dev.StarTable([star], jitter="applied")
    res = {}
    for prec in ("mixed", "fp64"):
        br = BatchRejection(table, cache, precision=prec, max_out=1 << 16, seeds=[1234])
        br.run()
        counts, idx, ll = br.results()
        res[prec] = (int(counts[0]), idx[0], ll[0])
        del br
        torch.cuda.empty_cache()
    (cm, im, lm), (c64, i64, l64) = res["mixed"], res["fp64"]
    assert cm == c64 > 0
    np.testing.assert_array_equal(im, i64)
    assert np.max(np.abs(lm - l64)) <= 1e-4
