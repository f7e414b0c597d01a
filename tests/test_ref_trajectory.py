"""The GPU sampler's held-out perplexity trajectory against the reference's
own run() (mcmc_sampler_stochastic.cc:93-183), recorded by
tests/golden/make_ref_trajectory.py from the reference compiled from its
sources: the small workload (N=5,000, K=32, num-node-sample 32, minibatch
500, a=0.01, b=1024, c=0.55), 2,000 iterations, perplexity every 100.

Both sides use the same graph, the held-out and test sets the reference
drew, and the same initial state (phi, theta ~ Gamma(1, 1) from the Philox
stream of the seed, which the fixture's reference runs were given with
set_state).  They differ in the random streams of the draws: the reference
runs six xorshift128+ streams, the GPU six Philox streams (chain ids 0-5),
so single trajectories differ by the draws' own noise (~0.5% per point).
The check, at every perplexity point of both initial seeds: the mean over
the GPU's six trajectories is within 1% of the mean over the reference's
six.  (Measured with the oracle sampler in place of the GPU: at most 0.74%,
at step 101, and 0.05% at step 1,901.)
"""
import importlib.util
import os

import numpy as np
import pytest

from mcmc_for_ammsb_gb300 import MCMCSamplerStochastic, Network, Options, workloads

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURE = os.path.join(GOLDEN, "trajectory_ref_small.npz")


def _initial_state(seed, N):
    """The initial state the fixture's reference runs started from."""
    spec = importlib.util.spec_from_file_location(
        "make_ref_trajectory", os.path.join(GOLDEN, "make_ref_trajectory.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.initial_state(seed, N)


def test_trajectory_against_reference_run(native_lib):
    d = np.load(FIXTURE)
    iters, interval, streams = int(d["iters"]), int(d["interval"]), int(d["streams"])
    net = Network.synthetic(**workloads.WORKLOADS["small"]["gen"])
    assert net.N == int(d["N"])
    for s in (int(x) for x in d["init_seeds"]):
        net.held_out = tuple(d["s%d_%s" % (s, k)] for k in ("ha", "hb", "hy"))
        net.test = tuple(d["s%d_%s" % (s, k)] for k in ("ta", "tb", "ty"))
        phi, theta = _initial_state(s, net.N)
        ref = d["s%d_ppx" % s]
        gpu = []
        for c in range(streams):
            o = Options(K=32, alpha=1.0 / 32, epsilon=1e-7, a=0.01, b=1024.0, c=0.55,
                        num_node_sample=32, held_out_ratio=0.02, random_seed=s, chain=c)
            sm = MCMCSamplerStochastic(o, net).create()
            sm.set_state(phi, theta)
            curve = []
            for it in range(0, iters, interval):  # perplexity before the update, as run() does
                curve.append(sm.cal_perplexity_held_out())
                sm.step(interval)
            sm.close()
            gpu.append(curve)
        gpu = np.array(gpu)
        assert gpu.shape == ref.shape
        rel = gpu.mean(0) / ref.mean(0) - 1.0
        print("\ninitial seed %d: mean GPU / mean reference - 1 per point:" % s, np.round(rel, 4))
        assert np.all(np.abs(rel) <= 0.01), rel
