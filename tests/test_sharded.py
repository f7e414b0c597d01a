"""The sharded iteration (mcmc_for_ammsb_gb300/sharded.py, the distributed
sampler's split of an iteration over ranks, mcmc_sampler_stochastic_distr.cc
:630-708, 1430-1442, 1626-1632).

CPU: each rank's phases run on the oracle (float arithmetic in the
reference's order, the Philox draws of the spec).  One rank reproduces the
oracle's whole iteration bit for bit; two ranks over torch.distributed
(gloo, two processes) update the phi rows they own (phi is sharded, pi
replicated), which after the first iteration equal the oracle's bit for
bit (every node's update reads the same state); the replicated pi, theta
and beta agree exactly between the ranks; against the FP64 oracle (same
draws) the sharded chain is at most twice as far off as the single-rank
float chain (the beta-gradient sums are added per rank, which reorders
their float rounding).

GPU: the C ABI's shard phases on one handle that owns everything equal
ammsb_step bit for bit; two handles on one GPU, exchanging rows and sums
through the host in lockstep (no kernel waits on another), equal one
handle's chain within the same bounds.
"""
import os
import socket

import numpy as np
import pytest

import oracle
from mcmc_for_ammsb_gb300 import workloads
from mcmc_for_ammsb_gb300.sharded import ShardedChain, TorchComm, owner

K = 32


class OracleRank:
    """One rank's shard phases on the oracle (test infrastructure)."""

    def __init__(self, net, phi, theta, seed=42):
        self.o = oracle.OracleSampler(net, K, a=0.01, b=1024.0, c=0.55, seed=seed)
        self.o.set_state(phi, theta)
        self.K = K
        self.me = max(self.o.p.mini_batch_size, net.max_degree())

    def _eps(self):
        return oracle.eps_t(self.o.p.a, self.o.p.b, self.o.p.c, self.o.step_count)

    def shard_draw(self):
        p = self.o.p
        self.mb = oracle.sample_minibatch(self.o.og, p.strategy, p.mini_batch_size,
                                          p.num_total_edges, p.seed, p.chain, self.o.step_count,
                                          self.me)
        return self.mb

    def shard_update(self, slots):
        p, o = self.o.p, self.o
        rows = np.zeros((len(slots), K), np.float32)
        for q, s in enumerate(slots):
            i = int(self.mb["nodes"][s])
            nb, y = oracle.sample_neighbors(o.og, i, p.num_node_sample + 1, p.seed, p.chain,
                                            o.step_count)
            noise = oracle.normals(p.seed, p.chain, oracle.P_PHI_NOISE, i, o.step_count, K)
            o.phi[i] = oracle.update_phi(K, o.pi, o.phi[i], i, nb, y, o.beta, p.alpha, p.epsilon,
                                         self._eps(), o.N, p.num_node_sample, noise)
            rows[q] = oracle.normalize(o.phi[i][None, :])[0]
        return rows

    def shard_commit(self, rows_all, edge_idx):
        o, p = self.o, self.o.p
        nodes = self.mb["nodes"]
        o.pi[nodes] = rows_all
        ea = nodes[self.mb["edge_a"][edge_idx]].astype(np.int32)
        eb = nodes[self.mb["edge_b"][edge_idx]].astype(np.int32)
        ey = np.ascontiguousarray(self.mb["edge_y"][edge_idx], np.uint8)
        grads = np.zeros((K, 2), np.float32)
        oracle.lib().oracle_beta_grads_f32(
            K, oracle._p(o.pi), oracle._p(ea), oracle._p(eb), oracle._p(ey), len(ea),
            oracle._p(o.theta), oracle._p(o.beta), oracle.ctypes.c_float(p.epsilon),
            oracle._p(grads))
        return grads

    def shard_theta(self, total):
        o, p = self.o, self.o.p
        total = np.ascontiguousarray(total, np.float32)
        noise = oracle.normals(p.seed, p.chain, oracle.P_THETA_NOISE, 0, o.step_count, 2 * K)
        eta = np.array([p.eta0, p.eta1], np.float32)
        oracle.lib().oracle_theta_step_f32(
            K, oracle._p(o.theta), oracle._p(o.beta), oracle._p(eta),
            oracle.ctypes.c_float(self._eps()), oracle.ctypes.c_float(self.mb["scale"]),
            oracle._p(noise), oracle._p(total))
        o.step_count += 1


def _case():
    net = oracle.SyntheticNetwork.synthetic(**workloads.WORKLOADS["small"]["gen"])
    net.make_held_out(0.02, seed=0)
    rng = np.random.default_rng(3)
    phi = rng.gamma(1.0, 1.0, (net.N, K)).astype(np.float32)
    theta = rng.gamma(1.0, 1.0, (K, 2)).astype(np.float32)
    return net, phi, theta


class _Solo:
    def allgather(self, obj):
        return [obj]


def test_one_rank_is_the_oracle_iteration():
    net, phi, theta = _case()
    ref = oracle.OracleSampler(net, K, a=0.01, b=1024.0, c=0.55)
    ref.set_state(phi, theta)
    r = OracleRank(net, phi, theta)
    chain = ShardedChain(r, 0, 1)
    for _ in range(6):
        ref.step()
        chain.step(_Solo())
    for a, b in ((ref.phi, r.o.phi), (ref.pi, r.o.pi), (ref.theta, r.o.theta),
                 (ref.beta, r.o.beta)):
        assert np.array_equal(a, b)


def test_protocol_rejects_inconsistent_payloads():
    net, phi, theta = _case()
    c = ShardedChain(OracleRank(net, phi, theta), 0, 2)
    slots, rows = c.draw_and_update()
    with pytest.raises(ValueError):
        c.commit([(slots, rows)])  # a payload missing
    with pytest.raises(ValueError):
        c.commit([(slots, rows), (slots, rows)])  # rank 1 sending rank 0's nodes
    with pytest.raises(ValueError):
        ShardedChain(None, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir, iters):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        net, phi, theta = _case()
        r = OracleRank(net, phi, theta)
        chain = ShardedChain(r, rank, world)
        comm = TorchComm()
        for it in range(iters):
            chain.step(comm)
            if it == 0:
                np.save(os.path.join(out_dir, "phi1_%d.npy" % rank), r.o.phi)
        np.savez(os.path.join(out_dir, "rank%d.npz" % rank), phi=r.o.phi, pi=r.o.pi,
                 theta=r.o.theta, beta=r.o.beta)
    finally:
        dist.destroy_process_group()


def test_two_ranks_over_gloo(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    iters = 5
    mp.spawn(_rank_main, args=(2, _free_port(), str(tmp_path), iters), nprocs=2, join=True)
    net, phi, theta = _case()
    ref = oracle.OracleSampler(net, K, a=0.01, b=1024.0, c=0.55)
    ref.set_state(phi, theta)
    own = owner(np.arange(net.N), 2)
    ref.step()
    # first iteration: each rank's own phi rows are the oracle's, bit for bit
    for r in range(2):
        p1 = np.load(str(tmp_path / ("phi1_%d.npy" % r)))
        assert np.array_equal(p1[own == r], ref.phi[own == r])
    for _ in range(iters - 1):
        ref.step()
    got = [dict(np.load(str(tmp_path / ("rank%d.npz" % r)))) for r in range(2)]
    for k in ("pi", "theta", "beta"):  # the replicated state agrees exactly
        assert np.array_equal(got[0][k], got[1][k]), k
    phi = np.where((own == 0)[:, None], got[0]["phi"], got[1]["phi"])  # phi from its owners
    # against exact arithmetic (the FP64 oracle, same draws) the sharded
    # float chain is as close as the single-rank float chain: splitting the
    # float beta-gradient sums only reorders their rounding
    exact = oracle.OracleSampler64(net, K, a=0.01, b=1024.0, c=0.55)
    exact.set_state(phi=_case()[1], theta=_case()[2])
    for _ in range(iters):
        exact.step()

    def rel(x, want):
        return float(np.max(np.abs(np.asarray(x, np.float64) - want) / np.abs(want)))

    for k, x in (("phi", phi), ("pi", got[0]["pi"]), ("theta", got[0]["theta"]),
                 ("beta", got[0]["beta"])):
        want, single = getattr(exact, k), getattr(ref, k)
        assert rel(x, want) <= 2 * rel(single, want) + 1e-6, (k, rel(x, want), rel(single, want))
    # both ranks own part of the minibatch
    mb = oracle.sample_minibatch(oracle.OracleGraph(net), 0, net.N // 10, net.num_total_edges,
                                 42, 0, 1, max(net.N // 10, net.max_degree()))
    assert set(owner(mb["nodes"], 2).tolist()) == {0, 1}


# ---------------------------------------------------------------------------
# the C ABI's shard phases on the GPU
# ---------------------------------------------------------------------------
def _gpu_samplers(n, Kg, dtype):
    from mcmc_for_ammsb_gb300 import MCMCSamplerStochastic, Options
    net, _ = workloads.build("small")
    rng = np.random.default_rng(9)
    phi = rng.gamma(1.0, 1.0, (net.N, Kg)).astype(np.float32)
    theta = rng.gamma(1.0, 1.0, (Kg, 2)) + 0.05
    out = []
    for _ in range(n):
        s = MCMCSamplerStochastic(Options(K=Kg, num_node_sample=32, a=0.01, c=0.55, pi_dtype=dtype),
                                  net).create()
        s.set_state(phi, theta)
        out.append(s)
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("Kg,dtype", [(32, 0), (1024, 1)], ids=["k32-f32", "k1024-bf16"])
def test_gpu_one_rank_equals_step(native_lib, Kg, dtype):
    ref, sh = _gpu_samplers(2, Kg, dtype)
    chain = ShardedChain(sh, 0, 1)
    for _ in range(5):
        ref.step(1)
        chain.step(_Solo())
    for k in ("phi", "pi", "theta", "beta"):
        assert np.array_equal(getattr(ref, k), getattr(sh, k)), k
    assert ref.step_count == sh.step_count
    ref.close()
    sh.close()


@pytest.mark.gpu
def test_gpu_two_ranks_in_lockstep(native_lib):
    """Two handles on one GPU as two ranks; the host moves the rows and the
    sums between them between phases (no kernel waits on another)."""
    ref, a, b = _gpu_samplers(3, 32, 0)
    chains = [ShardedChain(a, 0, 2), ShardedChain(b, 1, 2)]
    for it in range(5):
        ref.step(1)
        payloads = [c.draw_and_update() for c in chains]
        sums = [c.commit(payloads) for c in chains]
        for c in chains:
            c.finish(sums)
        if it == 0:  # each rank's own phi rows, bit for bit
            for r, s in ((0, a), (1, b)):
                rows = owner(np.arange(ref.N), 2) == r
                assert np.array_equal(s.phi[rows], ref.phi[rows])
    own = owner(np.arange(ref.N), 2)
    for k in ("pi", "theta", "beta"):  # the replicated state agrees exactly
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    phi = np.where((own == 0)[:, None], a.phi, b.phi)
    for k, x, want in (("phi", phi, ref.phi), ("pi", a.pi, ref.pi), ("theta", a.theta, ref.theta),
                       ("beta", a.beta, ref.beta)):
        rel = np.max(np.abs(x.astype(np.float64) - want) / np.maximum(np.abs(want), 1e-30))
        assert rel < 1e-5, (k, rel)
    for s in (ref, a, b):
        s.close()
