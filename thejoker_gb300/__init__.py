"""thejoker_gb300: The Joker's rejection-sampling hot path on GB300 (sm_103a).

The marginal likelihood over prior samples and the acceptance test run as
hand-written CUDA kernels in ``_lib/libjoker_gb300.so`` (C ABI:
include/joker_gb300.h).  The Python layer mirrors the reference's public API:
TheJoker, JokerPrior, JokerSamples, RVData and the CJokerHelper drop-in
GPUJokerHelper.
"""
from .data import RVData, validate_prepare_data  # noqa: F401
from .prior import JokerPrior  # noqa: F401
from .samples import JokerSamples  # noqa: F401

__version__ = "0.1.0"


def __getattr__(name):
    # GPU-facing classes import torch lazily
    if name == "TheJoker":
        from .sampler import TheJoker
        return TheJoker
    if name == "GPUJokerHelper":
        from .helper import GPUJokerHelper
        return GPUJokerHelper
    raise AttributeError(name)
