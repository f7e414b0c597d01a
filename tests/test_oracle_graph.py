"""The oracle's own workload inputs (oracle/ammsb_oracle_graph.c) against
the product's: the CPU legs of the benchmark build their graphs and
held-out sets there, so they must be the same graphs and splits, element
for element.  Also: the threaded oracle iteration equals the sequential one
bit for bit.  CPU only (the product's generator is host code)."""
import numpy as np
import pytest

import oracle
from mcmc_for_ammsb_gb300 import Network, workloads


@pytest.mark.parametrize("gen", [
    workloads.WORKLOADS["small"]["gen"],
    workloads.WORKLOADS["diff"]["gen"],
    workloads.WORKLOADS["mid"]["gen"],
    dict(n=3000, k_true=30, intra_degree=6.0, seed=4),
    dict(n=800, k_true=400, size_min=2, size_max=3, intra_degree=1.0, seed=9,
         background_frac=0.5),
    dict(n=500, k_true=3, size_min=100, size_max=400, p1=0.2, p2=0.3, zipf_s=2.5, seed=1),
])
def test_generator_and_split_match_the_product(native_lib, gen):
    a = Network.synthetic(**gen)
    b = oracle.SyntheticNetwork.synthetic(**gen)
    assert np.array_equal(a.row_ptr, b.row_ptr)
    assert np.array_equal(a.col, b.col)
    for ratio, seed in ((0.02, gen.get("seed", 0)), (0.1, 77)):
        a.make_held_out(ratio, seed=seed)
        b.make_held_out(ratio, seed=seed)
        for x, y in zip(a.held_out + a.test, b.held_out + b.test):
            assert x.dtype == y.dtype and np.array_equal(x, y)


def test_generator_rejects_bad_parameters():
    with pytest.raises(RuntimeError):
        oracle.SyntheticNetwork.synthetic(n=1, k_true=1)
    with pytest.raises(RuntimeError):
        oracle.SyntheticNetwork.synthetic(n=100, k_true=5, zipf_s=1.0)


@pytest.mark.parametrize("strategy", [0, 1, 2])
def test_threaded_iteration_equals_sequential(strategy):
    net = oracle.SyntheticNetwork.synthetic(**workloads.WORKLOADS["small"]["gen"])
    net.make_held_out(0.02, seed=0)
    K = 32
    rng = np.random.default_rng(strategy)
    phi = rng.gamma(1.0, 1.0, (net.N, K)).astype(np.float32)
    theta = rng.gamma(1.0, 1.0, (K, 2)).astype(np.float32)
    seq = oracle.OracleSampler(net, K, strategy=strategy, a=0.01, b=1024.0, c=0.55)
    par = oracle.OracleSampler(net, K, strategy=strategy, a=0.01, b=1024.0, c=0.55)
    seq.set_state(phi, theta)
    par.set_state(phi, theta)
    for _ in range(12):
        i1 = seq.step()
        i2 = par.step_threads(4)
        assert (i1.flag, i1.n_nodes, i1.n_edges, i1.scale) == (i2.flag, i2.n_nodes, i2.n_edges,
                                                                i2.scale)
    for x, y in ((seq.phi, par.phi), (seq.pi, par.pi), (seq.theta, par.theta),
                 (seq.beta, par.beta)):
        assert np.array_equal(x, y)
