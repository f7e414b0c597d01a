"""Generates tests/golden/ref_*.npz from the reference's own sampler code.

Builds oracle/_ref/libammsb_ref.so from the reference sources (where
oracle/ref/build_ref.py finds them) and records, for small
fixed workloads, what the reference's functions return:

  * the graph, held-out and test sets as the reference loaded/drew them;
  * a state (phi, theta) and the pi/beta the reference derives from it;
  * update_phi (mcmc_sampler_stochastic.cc:269-313) on several nodes: the
    neighbour set in its iteration order, the noise drawn, the new phi row;
  * update_beta (cc:200-267) on a minibatch: edge order, noise, theta, beta;
  * cal_perplexity (learner.cc:138-183) on two consecutive calls;
  * minibatches and neighbour sets drawn by the reference's samplers
    (network.cc:156-421, mcmc_sampler_stochastic.h:87-108) for invariants.

Run:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

CASES = {
    # name: (graph n, k_true, seed, K, num_node_sample, mini_batch_size)
    "ref_k16": (600, 8, 3, 16, 10, 30),
    "ref_k40": (500, 6, 5, 40, 24, 40),
}


def make(name, n, k_true, seed, K, nns, mbs):
    from ref import build_ref
    import refbuild
    from mcmc_for_ammsb_gb300 import Network

    build_ref.build()
    net = Network.synthetic(n=n, k_true=k_true, size_min=10, size_max=200, intra_degree=4.0,
                            seed=seed)
    und = net.undirected_edges()
    r = refbuild.RefSampler(und, ["--mcmc.K", str(K), "-n", str(nns), "-m", str(mbs),
                                  "--mcmc.held-out-ratio", "0.05", "--mcmc.seed", "7",
                                  "--mcmc.a", "0.01", "--mcmc.c", "0.55"])
    rng = np.random.default_rng(seed)
    ea, eb = r.edges()
    ha, hb, hy = r.held_out()
    ta, tb, ty = r.test_set()
    out = dict(N=r.N, K=K, nns=r.nns, mbs=r.mbs, E=r.E, edge_a=ea, edge_b=eb, ho_a=ha, ho_b=hb,
               ho_y=hy, te_a=ta, te_b=tb, te_y=ty, alpha=1.0 / K, epsilon=1e-7, a=0.01, b=1024.0,
               c=0.55)
    phi = rng.gamma(1.0, 1.0, (r.N, K)).astype(np.float32) + np.float32(1e-3)
    theta = (rng.gamma(1.0, 1.0, (K, 2)) + 0.05).astype(np.float32)
    r.set_state(phi, theta)
    _, pi, th, bt = r.state()
    out.update(phi=phi, theta=theta, pi=pi, beta=bt)
    step = 37
    r.set_step(step)
    eps = r.eps_t()
    out.update(step=step, eps=eps)
    # update_phi on distinct nodes, neighbour sets drawn by the reference
    excl = set(zip(ha.tolist(), hb.tolist())) | set(zip(ta.tolist(), tb.tolist()))
    nodes = rng.choice(r.N, 6, replace=False).astype(np.int32)
    orders, noises, phis = [], [], []
    for v in nodes:
        nb = r.sample_neighbors(int(v))
        assert v not in nb and len(set(nb.tolist())) == nns + 1
        assert all((min(v, j), max(v, j)) not in excl for j in nb)
        order, noise, newphi = r.update_phi(int(v), nb, eps)
        orders.append(order)
        noises.append(noise)
        phis.append(newphi)
    out.update(phi_nodes=nodes, phi_order=np.array(orders), phi_noise=np.array(noises),
               phi_out=np.array(phis))
    # update_beta on a minibatch drawn by the reference (pi unchanged: the
    # harness does not renormalise between the calls)
    mea, meb, scale = r.sample_minibatch(mbs + 1000)
    oa, ob, bnoise, th2, bt2 = r.update_beta(mea, meb, scale)
    out.update(beta_edge_a=oa, beta_edge_b=ob, beta_scale=scale, beta_noise=bnoise,
               theta_out=th2, beta_out=bt2)
    # perplexity: two consecutive calls on the same state
    p1, ppx1 = r.perplexity()
    p2, ppx2 = r.perplexity()
    out.update(ppx1=p1, ppx_edges1=ppx1, ppx2=p2, ppx_edges2=ppx2)
    # minibatch and neighbour draws for invariants
    mb_sizes, mb_scales, mb_flags = [], [], []
    mb_pairs = []
    for _ in range(40):
        a_, b_, s_ = r.sample_minibatch(mbs + 1000)
        mb_sizes.append(len(a_))
        mb_scales.append(s_)
        mb_pairs.append(np.stack([a_, b_], 1))
    out.update(mb_sizes=np.array(mb_sizes), mb_scales=np.array(mb_scales, np.float32),
               mb_pairs=np.concatenate(mb_pairs), )
    r.close()
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    return path


if __name__ == "__main__":
    for name, args in CASES.items():
        print(make(name, *args))
