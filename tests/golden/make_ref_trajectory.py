"""Generates tests/golden/trajectory_ref_small.npz: held-out perplexity
trajectories of the reference's own run() loop on the small workload.

The reference's sequential sampler is compiled from its sources
(oracle/ref/build_ref.py -> oracle/_ref/libammsb_ref.so).  For each seed it
loads the small workload's graph (N=5,000, written as relativity text and
read by the reference's own reader, preprocess/relativity.cc:20-200), draws
its held-out and test sets with its own RNG (network.cc:503-614),
initialises phi and theta (mcmc_sampler_stochastic.cc:29-79) and runs
run() (cc:93-183) for 2,000 iterations with K=32, alpha=1/32, eta=(1, 1),
epsilon=1e-7, a=0.01, b=1024, c=0.55, num-node-sample 32, minibatch
N/10 and held-out ratio 0.02, printing the held-out perplexity every 100
steps.  The fixture records, per seed, the held-out and test sets the
reference drew and the perplexity it printed at steps 1, 101, ..., 1901.

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

SEEDS = (11, 12, 13, 14, 15, 16)
ITERS, INTERVAL = 2000, 100
LINE = re.compile(r"average_count is: (\d+) step count: (\d+) time: \S+ "
                  r"perplexity for hold out set: (\S+)")


def run_seed(und, seed):
    import refbuild
    r = refbuild.RefSampler(und, ["--mcmc.K", "32", "--mcmc.alpha", "0.03125",
                                  "--mcmc.epsilon", "1e-7", "--mcmc.a", "0.01", "--mcmc.b", "1024",
                                  "--mcmc.c", "0.55", "-n", "32", "--mcmc.held-out-ratio", "0.02",
                                  "--mcmc.seed", str(seed), "-i", str(INTERVAL)])
    ha, hb, hy = r.held_out()
    ta, tb, ty = r.test_set()
    # run() prints to the process's stdout: collect it from the file
    # descriptor
    sys.stdout.flush()
    saved = os.dup(1)
    with tempfile.TemporaryFile(mode="w+") as f:
        os.dup2(f.fileno(), 1)
        try:
            r.run(ITERS, INTERVAL)
        finally:
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
    r.close()
    return dict(ha=ha, hb=hb, hy=hy, ta=ta, tb=tb, ty=ty, steps=np.array(steps),
                ppx=np.array(ppx))


def make():
    from ref import build_ref
    from mcmc_for_ammsb_gb300 import workloads, Network

    build_ref.build()
    gen = workloads.WORKLOADS["small"]["gen"]
    net = Network.synthetic(**gen)
    und = net.undirected_edges()
    out = dict(seeds=np.array(SEEDS), iters=ITERS, interval=INTERVAL, N=net.N)
    for s in SEEDS:
        d = run_seed(und, s)
        assert list(d["steps"]) == list(range(1, ITERS, INTERVAL)), d["steps"]
        for k, v in d.items():
            out["s%d_%s" % (s, k)] = v
        print("seed", s, "perplexity", d["ppx"][[0, 1, 5, -1]])
    path = os.path.join(HERE, "trajectory_ref_small.npz")
    np.savez_compressed(path, **out)
    return path


if __name__ == "__main__":
    print(make())
