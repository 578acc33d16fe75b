"""The two forms of the mixed kernel (GB300 only): two samples per thread on
the paired FP32 instructions (the default for L <= 3, and for any L without
jitter) and one sample per thread.  Each must keep |ln L - FP64 ln L| within its own per-sample bound, and
the two agree within the sum of their bounds.  The form is fixed per process
(JOKER_MIXED_PAIRED=0 selects one sample per thread), so each runs in a child
process."""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
CHILD = r"""
import sys
sys.path.insert(0, {root!r}); sys.path.insert(0, {tests!r})
import numpy as np, torch
from gpu_util import synth_star, synth_chunk
from thejoker_gb300 import device as dev
rng = np.random.default_rng(17)
out = {{}}
for name, jitter, poly, N, mu0 in (("ref2", "reference", 1, 33, 0.0), ("jit2", "applied", 1, 41, 0.0),
                                   ("jit3", "applied", 2, 150, 0.0), ("ref3", "reference", 2, 300, 0.0),
                                   ("jitmu", "applied", 1, 12, 3.0), ("ref4", "reference", 3, 20, 0.0)):
    star = synth_star(rng, N, poly=poly)
    star["mu"] = star["mu"].copy(); star["mu"][0] = mu0
    S = 70001
    chunk = synth_chunk(rng, S, jitter=(jitter == "applied"))
    table = dev.StarTable([star], jitter=jitter)
    cache = dev.PriorCache.from_samples(chunk)
    o = torch.empty((1, S), dtype=torch.float64, device="cuda")
    dev.lnl(table, cache, o, precision="fp64")
    out[name + "fp64"] = o.cpu().numpy()
    for prec in ("mixed", "mixed_accurate"):
        o = torch.empty((1, S), dtype=torch.float64, device="cuda")
        e = torch.empty((1, S), dtype=torch.float32, device="cuda")
        bk = dev.MaxKeys(2)
        dev.lnl(table, cache, o, precision=prec, err=e, bound_keys=bk)
        out[name + prec] = o.cpu().numpy(); out[name + prec + "_err"] = e.cpu().numpy()
np.savez(sys.argv[1], **out)
"""


def _run(tmp_path, paired):
    env = dict(os.environ, JOKER_MIXED_PAIRED="1" if paired else "0")
    path = str(tmp_path / f"out_{int(paired)}.npz")
    code = CHILD.format(root=os.path.dirname(HERE), tests=HERE)
    subprocess.run([sys.executable, "-c", code, path], check=True, env=env, timeout=600)
    return np.load(path)


def test_paired_and_scalar_within_bounds(cuda, tmp_path):
    a, b = _run(tmp_path, True), _run(tmp_path, False)
    for name in ("ref2", "jit2", "jit3", "ref3", "jitmu", "ref4"):
        f64 = a[name + "fp64"]
        np.testing.assert_array_equal(f64, b[name + "fp64"])
        for prec in ("mixed", "mixed_accurate"):
            for r in (a, b):
                d = np.abs(r[name + prec] - f64)
                assert np.all(d <= r[name + prec + "_err"]), (name, prec)
            gap = np.abs(a[name + prec] - b[name + prec])
            assert np.all(gap <= a[name + prec + "_err"] + b[name + prec + "_err"]), (name, prec)
