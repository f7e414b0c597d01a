"""GB300-native SG-MCMC sampler for the assortative mixed-membership
stochastic blockmodel (a-MMSB).

The hot path -- minibatch and neighbour sampling, update_phi, pi
normalisation, update_beta/theta and held-out perplexity -- runs as
hand-written sm_103a CUDA kernels behind the C ABI of libammsb_gpu.so
(include/ammsb_gpu.h).  This package is the thin host binding.
"""
from . import _native
from .network import Network
from .options import Options
from .sampler import ChainBatch, MCMCSamplerStochastic

__all__ = ["Network", "Options", "MCMCSamplerStochastic", "ChainBatch", "lib"]


def lib():
    return _native.lib()
