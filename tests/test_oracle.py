"""CPU tests of the oracle: Philox known answers, the sampling spec's
invariants, and the literal hot-path restatements against independent
numpy formulations."""
import numpy as np
import pytest

import oracle


def test_philox_known_answers():
    # Random123 kat_vectors for philox4x32-10
    assert oracle.philox([0, 0, 0, 0], [0, 0]) == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    assert oracle.philox([0xffffffff] * 4, [0xffffffff] * 2) == [
        0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert oracle.philox([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344],
                         [0xa4093822, 0x299f31d0]) == [0xd16cfe09, 0x94fdcceb, 0x5001e420,
                                                       0x24126ea1]


def test_draw_layout():
    L = oracle.lib()
    blk = oracle.philox([3, 7, 11, oracle.P_NBR], [42, 5])
    assert L.oracle_draw_u64(42, 5, oracle.P_NBR, 7, 11, 6) == blk[0] | (blk[1] << 32)
    assert L.oracle_draw_u64(42, 5, oracle.P_NBR, 7, 11, 7) == blk[2] | (blk[3] << 32)


def test_normals_are_standard():
    z = oracle.normals(1, 0, oracle.P_PHI_NOISE, 3, 9, 20000)
    assert abs(z.mean()) < 0.03 and abs(z.std() - 1) < 0.03
    assert np.all(np.isfinite(z))


def test_gamma_moments():
    L = oracle.lib()
    g = np.array([L.oracle_gamma(5, 0, oracle.P_PHI_INIT, 0, k, 1.0, 1.0) for k in range(20000)])
    assert abs(g.mean() - 1) < 0.03 and abs(g.var() - 1) < 0.08
    g = np.array([L.oracle_gamma(5, 0, oracle.P_PHI_INIT, 1, k, 100.0, 0.01) for k in range(5000)])
    assert abs(g.mean() - 1) < 0.01 and abs(g.var() - 0.01) < 0.002
    g = np.array([L.oracle_gamma(5, 0, oracle.P_PHI_INIT, 2, k, 0.3, 2.0) for k in range(20000)])
    assert abs(g.mean() - 0.6) < 0.03


def test_eps_schedule():
    # mcmc_sampler_stochastic.h:112-115 with a = b^-c (options.h:257-259)
    a = 1024.0 ** -0.5
    assert oracle.eps_t(a, 1024.0, 0.5, 1) == pytest.approx(a * (1 + 1 / 1024.0) ** -0.5, rel=1e-7)


def test_nonlink_scale():
    # network.cc:341-342
    N, m, E = 5000, 500, 14668
    want = np.float32(np.float32(N) * np.float32(N) / np.float32(m))
    want = np.float32(float(want) * (E / (N * (N - 1.0) / 2.0 - E)))
    assert oracle.nonlink_scale(N, m, E) == want


class _Net:
    def __init__(self, n, edges, held, test):
        adj = [[] for _ in range(n)]
        for a, b in edges:
            adj[a].append(b)
            adj[b].append(a)
        self.row_ptr = np.zeros(n + 1, np.int64)
        for v in range(n):
            self.row_ptr[v + 1] = self.row_ptr[v] + len(set(adj[v]))
        self.col = np.concatenate([np.array(sorted(set(r)), np.int32) for r in adj]) \
            if edges else np.zeros(0, np.int32)
        self.N = n
        self.num_total_edges = int(self.row_ptr[-1] // 2)
        self.held_out = tuple(np.array(x, t) for x, t in zip(held, (np.int32, np.int32, np.uint8)))
        self.test = tuple(np.array(x, t) for x, t in zip(test, (np.int32, np.int32, np.uint8)))


@pytest.fixture(scope="module")
def toy():
    rng = np.random.default_rng(0)
    edges = set()
    while len(edges) < 600:
        a, b = rng.integers(0, 200, 2)
        if a != b:
            edges.add((min(a, b), max(a, b)))
    edges = sorted(edges)
    held = ([e[0] for e in edges[:10]] + [1, 2], [e[1] for e in edges[:10]] + [150, 160],
            [1] * 10 + [0, 0])
    test = ([e[0] for e in edges[10:20]], [e[1] for e in edges[10:20]], [1] * 10)
    return _Net(200, edges, held, test), edges


def test_minibatch_nonlink_invariants(toy):
    net, edges = toy
    og = oracle.OracleGraph(net)
    eset = set(edges)
    excl = {(min(a, b), max(a, b)) for a, b in zip(*net.held_out[:2])} | \
           {(min(a, b), max(a, b)) for a, b in zip(*net.test[:2])}
    for step in range(1, 30):
        mb = oracle.sample_minibatch(og, 2, 50, net.num_total_edges, 3, 0, step, 64)
        assert mb["flag"] == 0 and len(mb["edge_a"]) == 50
        v = mb["nodes"][0]
        us = mb["nodes"][1:]
        assert len(set(us.tolist())) == 50 and v not in us
        for u in us:
            p = (min(v, u), max(v, u))
            assert p not in eset and p not in excl
        assert np.all(mb["edge_a"] == 0) and np.array_equal(mb["edge_b"], np.arange(1, 51))
        assert mb["scale"] == oracle.nonlink_scale(200, 50, net.num_total_edges)


def test_minibatch_link_invariants(toy):
    net, edges = toy
    og = oracle.OracleGraph(net)
    for step in range(1, 30):
        mb = oracle.sample_minibatch(og, 1, 50, net.num_total_edges, 3, 0, step, 64)
        v = mb["nodes"][0]
        row = net.col[net.row_ptr[v]:net.row_ptr[v + 1]]
        keep = [u for u in row if not og.is_excluded(v, u)]
        assert np.array_equal(mb["nodes"][1:], keep)
        assert np.all(mb["edge_y"] == 1) and mb["scale"] == 200.0


def test_minibatch_is_deterministic_and_step_dependent(toy):
    net, _ = toy
    og = oracle.OracleGraph(net)
    a = oracle.sample_minibatch(og, 0, 40, net.num_total_edges, 9, 0, 5, 64)
    b = oracle.sample_minibatch(og, 0, 40, net.num_total_edges, 9, 0, 5, 64)
    c = oracle.sample_minibatch(og, 0, 40, net.num_total_edges, 9, 0, 6, 64)
    assert np.array_equal(a["nodes"], b["nodes"])
    assert not np.array_equal(a["nodes"], c["nodes"]) or a["flag"] != c["flag"]


def test_neighbors_invariants(toy):
    net, edges = toy
    og = oracle.OracleGraph(net)
    eset = set(edges)
    for node in (0, 1, 2, 50, 199):
        nb, y = oracle.sample_neighbors(og, node, 33, 4, 0, 12)
        assert len(set(nb.tolist())) == 33 and node not in nb
        for j, yy in zip(nb, y):
            assert not og.is_excluded(node, j)
            assert bool(yy) == ((min(node, j), max(node, j)) in eset)


def _np_update_phi(K, pi, phi_i, i, nbrs, y, beta, alpha, eps_, eps_t, N, n, noise):
    """Independent float64 numpy formulation of update_phi."""
    S = phi_i.sum()
    grads = np.zeros(K)
    for j, yy in zip(nbrs, y):
        f = (beta - eps_) if yy else (eps_ - beta)
        e = eps_ if yy else 1 - eps_
        probs = pi[i] * (pi[j] * f + e)
        grads += probs / probs.sum() / phi_i - 1.0 / S
    v = np.abs(phi_i + eps_t / 2 * (alpha - phi_i + N / n * grads) + np.sqrt(eps_t * phi_i) * noise)
    return np.maximum(v, 1e-24)


def test_update_phi_restatement():
    rng = np.random.default_rng(1)
    N, K = 50, 12
    phi = rng.gamma(1, 1, (N, K))
    pi = phi / phi.sum(1, keepdims=True)
    beta = rng.uniform(0.1, 0.9, K)
    nbrs = rng.choice(np.arange(1, N), 9, replace=False).astype(np.int32)
    y = (rng.uniform(size=9) < 0.3).astype(np.uint8)
    noise = rng.standard_normal(K)
    got64 = oracle.update_phi(K, pi, phi[0], 0, nbrs, y, beta, 0.1, 1e-7, 0.01, N, 8, noise,
                              np.float64)
    want = _np_update_phi(K, pi, phi[0], 0, nbrs, y, beta, 0.1, 1e-7, 0.01, N, 8, noise)
    assert np.allclose(got64, want, rtol=1e-12)
    got32 = oracle.update_phi(K, pi, phi[0], 0, nbrs, y, beta, 0.1, 1e-7, 0.01, N, 8, noise)
    assert np.allclose(got32, want, rtol=1e-5)
    g = oracle.phi_grad(K, pi, phi[0], 0, nbrs, y, beta, 1e-7)
    assert np.allclose(got64, np.maximum(np.abs(phi[0] + 0.005 * (0.1 - phi[0] + N / 8 * g)
                                                + np.sqrt(0.01 * phi[0]) * noise), 1e-24))


def test_update_beta_restatement():
    rng = np.random.default_rng(2)
    N, K = 40, 10
    pi = rng.dirichlet(np.ones(K), N)
    theta = rng.gamma(1, 1, (K, 2)) + 0.1
    beta = theta[:, 1] / theta.sum(1)
    ea = rng.integers(0, N, 15).astype(np.int32)
    eb = (ea + 1 + rng.integers(0, N - 1, 15)).astype(np.int32) % N
    ey = (rng.uniform(size=15) < 0.5).astype(np.uint8)
    noise = rng.standard_normal((K, 2))
    th, bt, grads = oracle.update_beta(K, pi, ea, eb, ey, theta, beta, np.array([1.0, 1.0]),
                                       1e-7, 0.01, 123.0, noise, np.float64)
    G = np.zeros((K, 2))
    ts = theta.sum(1)
    for a, b, y in zip(ea, eb, ey):
        f = pi[a] * pi[b]
        probs = (beta if y else 1 - beta) * f
        p0 = (1e-7 if y else 1 - 1e-7) * (1 - f.sum())
        P = probs.sum() + p0
        G[:, 0] += probs / P * ((1 - y) / theta[:, 0] - 1 / ts)
        G[:, 1] += probs / P * (y / theta[:, 1] - 1 / ts)
    assert np.allclose(grads, G, rtol=1e-12)
    want = np.maximum(np.abs(theta + 0.005 * (1.0 - theta + 123.0 * G) + np.sqrt(0.01 * theta) * noise),
                      1e-24)
    assert np.allclose(th, want, rtol=1e-12)
    assert np.allclose(bt, want[:, 1] / want.sum(1), rtol=1e-12)


def test_perplexity_restatement():
    rng = np.random.default_rng(3)
    N, K, H = 30, 8, 20
    pi = rng.dirichlet(np.ones(K), N)
    beta = rng.uniform(0.2, 0.8, K)
    ha = rng.integers(0, N, H).astype(np.int32)
    hb = ((ha + 1 + rng.integers(0, N - 1, H)) % N).astype(np.int32)
    hy = (np.arange(H) < H // 2).astype(np.uint8)
    ppx = np.zeros(H)
    got1 = oracle.perplexity(K, pi, (ha, hb, hy), beta, 1e-7, ppx, 1, "f64")
    f = pi[ha] * pi[hb]
    p = np.where(hy == 1, (f * beta).sum(1), (f * (1 - beta)).sum(1) + (1 - f.sum(1)) * (1 - 1e-7))
    assert got1 == pytest.approx(-np.mean(np.log(p)), rel=1e-12)
    got2 = oracle.perplexity(K, pi * 0.999 + 0.001 / K, (ha, hb, hy), beta, 1e-7, ppx, 2, "f64")
    pi2 = pi * 0.999 + 0.001 / K
    f2 = pi2[ha] * pi2[hb]
    p2 = np.where(hy == 1, (f2 * beta).sum(1), (f2 * (1 - beta)).sum(1) + (1 - f2.sum(1)) * (1 - 1e-7))
    assert got2 == pytest.approx(-np.mean(np.log((p + p2) / 2)), rel=1e-12)
