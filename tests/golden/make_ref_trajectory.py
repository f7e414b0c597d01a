"""Generates tests/golden/trajectory_ref_small.npz: held-out perplexity
trajectories of the reference's own run() loop on the small workload, from
a known initial state.

The reference's sequential sampler is compiled from its sources
(oracle/ref/build_ref.py -> oracle/_ref/libammsb_ref.so).  For each initial
seed s it loads the small workload's graph (N=5,000, written as relativity
text and read by the reference's own reader, preprocess/relativity.cc
:20-200) and draws its held-out and test sets with its own RNG
(network.cc:503-614).  The state is then set to phi ~ Gamma(1, 1), theta ~
Gamma(1, 1) from the Philox stream of seed s -- the state the GPU sampler's
init() draws for that seed, so both sides start from the same bits -- and
run() (mcmc_sampler_stochastic.cc:93-183) takes 2,000 iterations with K=32,
alpha=1/32, eta=(1, 1), epsilon=1e-7, a=0.01, b=1024, c=0.55,
num-node-sample 32, minibatch N/10, held-out ratio 0.02, printing the
held-out perplexity every 100 steps.  This is repeated with STREAMS fresh
random streams for the draws (the reference's xorshift128+ reseeded after
the held-out sets are drawn), so the fixture records, per initial seed,
the held-out and test sets and STREAMS perplexity curves at steps 1, 101,
..., 1901.

Run:  python tests/golden/make_ref_trajectory.py
"""
import os
import re
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

INIT_SEEDS = (11, 12)
STREAMS = 6
ITERS, INTERVAL = 2000, 100
K = 32
ARGS = ["--mcmc.K", str(K), "--mcmc.alpha", "0.03125", "--mcmc.epsilon", "1e-7", "--mcmc.a",
        "0.01", "--mcmc.b", "1024", "--mcmc.c", "0.55", "-n", "32", "--mcmc.held-out-ratio", "0.02",
        "-i", str(INTERVAL)]
LINE = re.compile(r"average_count is: (\d+) step count: (\d+) time: \S+ "
                  r"perplexity for hold out set: (\S+)")


def initial_state(seed, N):
    """phi (N x K) and theta (K x 2), Gamma(1, 1), from the Philox stream of
    `seed`: the state the GPU sampler's init() draws (chain 0)."""
    import oracle
    L = oracle.lib()
    phi = np.array([[L.oracle_gamma(seed, 0, oracle.P_PHI_INIT, v, k, 1.0, 1.0) for k in range(K)]
                    for v in range(N)], np.float32)
    theta = np.array([[L.oracle_gamma(seed, 0, oracle.P_THETA_INIT, 0, 2 * k + c, 1.0, 1.0)
                       for c in range(2)] for k in range(K)])
    return phi, theta


def run_curve(r):
    """run() for ITERS iterations; returns (steps, perplexities) it printed."""
    sys.stdout.flush()
    saved = os.dup(1)
    with tempfile.TemporaryFile(mode="w+") as f:
        os.dup2(f.fileno(), 1)
        try:
            r.run(ITERS, INTERVAL)
        finally:
            sys.stdout.flush()
            os.dup2(saved, 1)
            os.close(saved)
        f.seek(0)
        text = f.read()
    steps, ppx = [], []
    for line in text.splitlines():
        m = LINE.search(line)
        if m:
            steps.append(int(m.group(2)))
            ppx.append(float(m.group(3)))
    return steps, np.array(ppx)


def make():
    import refbuild
    from ref import build_ref
    from mcmc_for_ammsb_gb300 import Network, workloads

    build_ref.build()
    net = Network.synthetic(**workloads.WORKLOADS["small"]["gen"])
    und = net.undirected_edges()
    out = dict(init_seeds=np.array(INIT_SEEDS), streams=STREAMS, iters=ITERS, interval=INTERVAL,
               N=net.N)
    for s in INIT_SEEDS:
        phi, theta = initial_state(s, net.N)
        curves, sets = [], None
        for t in range(STREAMS):
            r = refbuild.RefSampler(und, ARGS + ["--mcmc.seed", str(s)])
            here = r.held_out() + r.test_set()
            if sets is None:
                sets = here
            assert all(np.array_equal(a, b) for a, b in zip(sets, here))
            r.set_state(phi, theta.astype(np.float32))
            r.reseed(1000 + 17 * t)
            steps, ppx = run_curve(r)
            r.close()
            assert steps == list(range(1, ITERS, INTERVAL)), steps
            curves.append(ppx)
        for k, v in zip(("ha", "hb", "hy", "ta", "tb", "ty"), sets):
            out["s%d_%s" % (s, k)] = v
        out["s%d_ppx" % s] = np.array(curves)
        print("seed", s, "mean curve", np.round(np.mean(curves, 0)[[0, 1, 5, -1]], 4))
    path = os.path.join(HERE, "trajectory_ref_small.npz")
    np.savez_compressed(path, **out)
    return path


if __name__ == "__main__":
    print(make())
