"""The synthetic workloads the sampler is specified and measured on.

Each workload names the planted-community generator parameters and the
sampler options (reference flag names).  No public dataset is involved:
graphs are generated from a seed with the shapes given below.

  small   N=5,000 (K_true 50, sizes Zipf(1.5) in [10, 500], intra degree 4,
          +10% background, ~14.5k edges), K=32, num-node-sample 32,
          minibatch N/10, held-out 1% of edges + equal non-edges, 2,000
          iterations with perplexity every 100, FP32.
  diff    N=2,000 (K_true 20, ~6k edges), K=16: the differentiation check.
  mid     N=100,000 (K_true 2,000, sizes [10, 5,000], intra degree 8),
          K=256, num-node-sample 64, minibatch 512.
  chains  64 graphs, N log-uniform in [1,000, 50,000], intra degree 6,
          K in {16, 32, 64, 128}, minibatch 32..1024, num-node-sample 32.
  large   N=4,000,000 (K_true 200,000, sizes [10, 20,000], intra degree
          16, ~35M edges), K=1024, num-node-sample 128, minibatch 4,096,
          held-out 0.1% of edges + equal non-edges, BF16 pi.
"""
import math

from .network import Network
from .options import Options

WORKLOADS = {
    "small": dict(
        gen=dict(n=5000, k_true=50, size_min=10, size_max=500, intra_degree=4.0, seed=0),
        opts=dict(K=32, alpha=1.0 / 32, eta0=1.0, eta1=1.0, epsilon=1e-7, a=0.01, b=1024.0,
                  c=0.55, num_node_sample=32, held_out_ratio=0.02, max_iteration=2001,
                  interval=100)),
    "diff": dict(
        gen=dict(n=2000, k_true=20, size_min=10, size_max=500, intra_degree=4.0, seed=0),
        opts=dict(K=16, num_node_sample=32, held_out_ratio=0.02)),
    "mid": dict(
        gen=dict(n=100000, k_true=2000, size_min=10, size_max=5000, intra_degree=8.0, seed=0),
        opts=dict(K=256, num_node_sample=64, mini_batch_size=512, held_out_ratio=0.02,
                  max_iteration=10001, interval=500, a=0.01, b=1024.0, c=0.55)),
    "large": dict(
        gen=dict(n=4000000, k_true=200000, size_min=10, size_max=20000, intra_degree=16.0,
                 seed=0),
        opts=dict(K=1024, num_node_sample=128, mini_batch_size=4096, held_out_ratio=0.002,
                  a=0.01, b=1024.0, c=0.55, interval=100)),
    # the large workload's kernel shapes on a 10x smaller graph (profiling)
    "large_s": dict(
        gen=dict(n=400000, k_true=20000, size_min=10, size_max=20000, intra_degree=16.0, seed=0),
        opts=dict(K=1024, num_node_sample=128, mini_batch_size=4096, held_out_ratio=0.002,
                  a=0.01, b=1024.0, c=0.55, interval=100)),
}


def chain_workload(i):
    """Chain i of the batching workload: its own graph from seed i."""
    import numpy as np
    rng = np.random.default_rng(1000 + i)
    n = int(round(math.exp(rng.uniform(math.log(1000), math.log(50000)))))
    K = int(rng.choice([16, 32, 64, 128]))
    m = int(round(math.exp(rng.uniform(math.log(32), math.log(1024)))))
    k_true = max(2, n // 100)
    return dict(gen=dict(n=n, k_true=k_true, size_min=10, size_max=500, intra_degree=6.0, seed=i),
                opts=dict(K=K, mini_batch_size=min(m, n // 2), num_node_sample=32,
                          held_out_ratio=0.02, pi_dtype=1, chain=i))


def build(name, seed=None, **opt_overrides):
    """(Network with held-out/test, Options) of a named workload."""
    w = WORKLOADS[name]
    gen = dict(w["gen"])
    if seed is not None:
        gen["seed"] = seed
    net = Network.synthetic(**gen)
    opts = dict(w["opts"])
    opts.update(opt_overrides)
    o = Options(**opts)
    net.make_held_out(o.held_out_ratio, seed=gen["seed"])
    return net, o
