"""The GPU sampler's held-out perplexity trajectory against the reference's
own run() (mcmc_sampler_stochastic.cc:93-183), recorded by
tests/golden/make_ref_trajectory.py from the reference compiled from its
sources: the small workload (N=5,000, K=32, num-node-sample 32, minibatch
500, a=0.01, b=1024, c=0.55), 2,000 iterations, perplexity every 100, six
seeds.  For each seed the GPU run uses the held-out and test sets the
reference drew for that seed and its own initial state and draws (Philox,
so the trajectories match in distribution, not draw for draw).

At every perplexity point t:
  * per seed, |gpu - ref| <= max(1% of ref, the reference's own spread
    across the seeds at t) -- the reference's seeds differ by 1-5% early in
    the run and by 0.85% at its end;
  * over the seeds, |mean gpu - mean ref| <= max(1% of mean ref, two
    standard errors of that difference).
"""
import os

import numpy as np
import pytest

from mcmc_for_ammsb_gb300 import MCMCSamplerStochastic, Network, Options, workloads

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                       "trajectory_ref_small.npz")


def test_trajectory_against_reference_run(native_lib):
    d = np.load(FIXTURE)
    seeds = [int(s) for s in d["seeds"]]
    iters, interval = int(d["iters"]), int(d["interval"])
    net = Network.synthetic(**workloads.WORKLOADS["small"]["gen"])
    assert net.N == int(d["N"])
    ref = np.array([d["s%d_ppx" % s] for s in seeds])
    gpu = []
    for s in seeds:
        net.held_out = (d["s%d_ha" % s], d["s%d_hb" % s], d["s%d_hy" % s])
        net.test = (d["s%d_ta" % s], d["s%d_tb" % s], d["s%d_ty" % s])
        o = Options(K=32, alpha=1.0 / 32, epsilon=1e-7, a=0.01, b=1024.0, c=0.55,
                    num_node_sample=32, held_out_ratio=0.02, random_seed=s)
        sm = MCMCSamplerStochastic(o, net).create()
        sm.init()
        curve = []
        for it in range(0, iters, interval):  # perplexity before the update, as run() does
            curve.append(sm.cal_perplexity_held_out())
            sm.step(interval)
        sm.close()
        gpu.append(curve)
    gpu = np.array(gpu)
    assert gpu.shape == ref.shape
    spread = ref.max(0) - ref.min(0)
    tol = np.maximum(0.01 * ref, spread[None, :])
    worst = np.abs(gpu - ref) / tol
    print("\nper-seed |gpu - ref| / tolerance, worst per point:", np.round(worst.max(0), 3))
    assert np.all(np.abs(gpu - ref) <= tol), worst.max(0)
    diff = gpu.mean(0) - ref.mean(0)
    se = np.sqrt(gpu.var(0, ddof=1) / len(seeds) + ref.var(0, ddof=1) / len(seeds))
    tol_mean = np.maximum(0.01 * ref.mean(0), 2 * se)
    print("mean gpu", np.round(gpu.mean(0), 4))
    print("mean ref", np.round(ref.mean(0), 4))
    assert np.all(np.abs(diff) <= tol_mean), (diff, tol_mean)
