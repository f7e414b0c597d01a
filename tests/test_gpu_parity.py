"""GPU parity tests: the CUDA path through the C ABI against the CPU oracle.

Tolerances (written here, used below):
  * sampling (flag, scale, minibatch edges, nodes, neighbour ids, y): exact;
  * one fed phi/theta step, FP32 pi: phi and pi within 1e-5 relative of
    the oracle's literal float restatement of update_phi; theta/beta (FP64
    on the device) within 1e-6 of the FP64 oracle's update_beta applied to
    the device's own new pi, and end to end within 1e-4 of the FP64 chain
    and within the float restatement's own rounding (2x its distance to
    FP64) of the float chain;
  * the same step against the FP64 oracle: 1e-4 relative (stated error of
    the float paths; the reference itself is float);
  * perplexity: 1e-5 relative (device uses a compensated FP64 log-sum);
  * trajectories: held-out perplexity within 1% at every checkpoint.
"""
import numpy as np
import pytest

import oracle
from mcmc_for_ammsb_gb300 import MCMCSamplerStochastic, Network, Options, _native, workloads

pytestmark = pytest.mark.gpu

RTOL_STEP = 1e-5
RTOL_F64 = 1e-4
RTOL_PPX = 1e-5


def rel_err(a, b, floor=1e-30):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor))) if a.size else 0.0


def plain_rel_stats(got, want):
    """Plain elementwise relative error |got - want| / |want|: the largest,
    the 99.9th percentile and the fraction of elements above 1e-5."""
    r = np.abs(got.astype(np.float64) - want) / np.maximum(np.abs(want), 1e-30)
    return {"max": float(r.max()), "p999": float(np.quantile(r, 0.999)),
            "frac_above_1e-5": float(np.mean(r > 1e-5))}


def check_phi(got, f32, f64, M, tol=RTOL_STEP):
    """New phi rows against the oracle: element by element within tol of
    the update's term magnitude plus twice the float restatement's own
    rounding (its distance to FP64), and row-wise (L2) within tol of the
    float restatement.  Returns the plain elementwise relative errors
    against the FP64 and the float restatements, which are reported beside
    the term-magnitude check: where the update's terms cancel, a new phi
    element is far smaller than the terms that made it, so its relative
    error measures the cancellation, not the kernel."""
    got = got.astype(np.float64)
    e_ref = np.abs(f32.astype(np.float64) - f64)
    assert np.all(np.abs(got - f64) <= tol * M + 2 * e_ref + 1e-30), \
        float(np.max((np.abs(got - f64) - 2 * e_ref) / M))
    row = np.linalg.norm(got - f32, axis=1) / np.linalg.norm(f32, axis=1)
    assert np.all(row < tol), float(row.max())
    return {"vs_f64": plain_rel_stats(got, f64),
            "vs_f32_restatement": plain_rel_stats(got, f32.astype(np.float64)),
            "f32_restatement_vs_f64": plain_rel_stats(f32, f64),
            "row_l2_vs_f32_restatement": float(row.max())}


def random_state(N, K, seed=0, shape=1.0):
    rng = np.random.default_rng(seed)
    phi = rng.gamma(shape, 1.0 / shape if shape > 1 else 1.0, (N, K)).astype(np.float32)
    phi = np.maximum(phi, np.float32(1e-6))
    theta = rng.gamma(1.0, 1.0, (K, 2)).astype(np.float64) + 0.05
    return phi, theta


def make_sampler(net, dtype=_native.PI_F32, **kw):
    o = dict(K=32, num_node_sample=32, a=0.01, b=1024.0, c=0.55, random_seed=42)
    o.update(kw)
    opts = Options(pi_dtype=dtype, **o)
    return MCMCSamplerStochastic(opts, net).create(), opts


@pytest.fixture(scope="module")
def small(native_lib):
    return workloads.build("small")


@pytest.fixture(scope="module")
def sparse_net(native_lib):
    """A graph with many isolated vertices: the link stratum must redraw."""
    rng = np.random.default_rng(5)
    a = rng.integers(0, 300, 400)
    b = rng.integers(0, 300, 400)
    net = Network.from_edges(1200, a, b)
    net.make_held_out(0.05, seed=1)
    return net


# ---------------------------------------------------------------------------
# sampling: bit-exact against the oracle's Philox specification
# ---------------------------------------------------------------------------
def check_sampling(s, net, opts, steps):
    og = oracle.OracleGraph(net)
    m = s.resolved.mini_batch_size
    n_out = s.num_node_sample + 1
    for _ in range(steps):
        step = s.step_count
        s.step(1)
        got = s.last_minibatch()
        want = oracle.sample_minibatch(og, opts.strategy, m, net.num_total_edges,
                                       opts.random_seed, opts.chain, step, s.max_edges,
                                       max_source=opts.sampler_max_source)
        assert got["flag"] == want["flag"]
        assert got["scale"] == pytest.approx(want["scale"], rel=0, abs=0)
        for k in ("edge_a", "edge_b", "edge_y", "nodes"):
            assert np.array_equal(got[k], want[k]), k
        for r, node in enumerate(want["nodes"]):
            nb, y = oracle.sample_neighbors(og, int(node), n_out, opts.random_seed, opts.chain,
                                            step)
            assert np.array_equal(got["nbrs"][r], nb), (step, r)
            assert np.array_equal(got["nbr_y"][r], y), (step, r)


@pytest.mark.parametrize("dtype", [_native.PI_F32, _native.PI_BF16])
@pytest.mark.parametrize("strategy", [0, 1, 2])
def test_sampling_bit_exact(small, dtype, strategy):
    net, _ = small
    s, opts = make_sampler(net, dtype, strategy=strategy)
    phi, theta = random_state(net.N, 32)
    s.set_state(phi, theta)
    check_sampling(s, net, opts, steps=6)
    s.close()


def test_sampling_link_stratum_redraws_empty(sparse_net):
    s, opts = make_sampler(sparse_net, strategy=1, K=16, num_node_sample=8, mini_batch_size=50)
    s.set_state(*random_state(sparse_net.N, 16))
    check_sampling(s, sparse_net, opts, steps=10)
    s.close()


@pytest.mark.parametrize("m", [300, 1000])
def test_sampling_random_edge(small, m):
    """random-edge (network.cc:237-268): m distinct training edges drawn from
    the symmetric CSR, nodes numbered by first appearance."""
    net, _ = small
    s, opts = make_sampler(net, strategy=3, mini_batch_size=m)
    s.set_state(*random_state(net.N, 32))
    check_sampling(s, net, opts, steps=4)
    s.close()


def test_sampling_random_edge_full_training_set(native_lib):
    """m at least the training edges: the whole training set is the
    minibatch (network.cc:215-234, 238-241)."""
    net = Network.synthetic(n=300, k_true=6, size_min=10, size_max=60, intra_degree=3.0, seed=7)
    net.make_held_out(0.1, seed=7)
    s, opts = make_sampler(net, K=8, num_node_sample=8, strategy=3,
                           mini_batch_size=net.num_total_edges)
    s.set_state(*random_state(net.N, 8))
    check_sampling(s, net, opts, steps=2)
    mb = s.last_minibatch()
    train = net.num_total_edges - int(net.held_out[2].sum()) - int(net.test[2].sum())
    assert len(mb["edge_a"]) == train
    s.close()


@pytest.mark.parametrize("strategy", [0, 1])
def test_sampling_several_link_sources(small, strategy):
    """sampler.max-source > 1 (network.cc:355-407): several sources per
    link-stratum attempt, shared edges kept once."""
    net, _ = small
    s, opts = make_sampler(net, strategy=strategy, sampler_max_source=5, mini_batch_size=60)
    s.set_state(*random_state(net.N, 32))
    check_sampling(s, net, opts, steps=8)
    s.close()


def test_step_random_edge_and_several_sources_against_oracle(small):
    """A fed update over the general minibatches: random-edge and
    several link sources (edges between arbitrary node slots)."""
    net, _ = small
    for kw in (dict(strategy=3, mini_batch_size=200), dict(strategy=1, sampler_max_source=4,
                                                           mini_batch_size=60)):
        run_fed_case(net, 32, 11, _native.PI_F32, **kw)


@pytest.mark.parametrize("m", [30, 60])
def test_sampling_small_population_collisions(native_lib, m):
    """N small relative to the draws: many duplicate candidates.  With m = 60
    of the ~70 valid partners the non-link rounds run until the population
    is nearly exhausted, each sized from the acceptance rate of the rounds
    before it."""
    rng = np.random.default_rng(9)
    net = Network.from_edges(80, rng.integers(0, 80, 200), rng.integers(0, 80, 200))
    net.make_held_out(0.1, seed=2)
    s, opts = make_sampler(net, K=8, num_node_sample=40, mini_batch_size=m, strategy=0)
    s.set_state(*random_state(net.N, 8))
    check_sampling(s, net, opts, steps=8)
    s.close()


# ---------------------------------------------------------------------------
# one fed step: update_phi + pi + update_beta against the literal oracle
# ---------------------------------------------------------------------------
def oracle_fed_step(net, opts, resolved, phi, theta, mb, nbrs, nby, pn, tn, step, dtype,
                    pi_nbr=None):
    """The fed step through the literal oracle.  Neighbour rows of pi are
    `pi_nbr` (the device's stored pi, e.g. BF16 values) when given; a node's
    own pi row is phi_i / sum(phi_i), as the kernel computes it."""
    K = phi.shape[1]
    phi = phi.astype(dtype)
    pi = oracle.normalize(phi, dtype) if pi_nbr is None else pi_nbr.astype(dtype).copy()
    own = oracle.normalize(phi[mb["nodes"]], dtype)
    th = theta.astype(dtype)
    beta = (th[:, 1] / (th[:, 0] + th[:, 1])).astype(np.float32).astype(dtype)
    eps = oracle.eps_t(resolved.a, resolved.b, resolved.c, step)
    new_phi = phi.copy()
    for r, node in enumerate(mb["nodes"]):
        keep = pi[node].copy()
        pi[node] = own[r]
        new_phi[node] = oracle.update_phi(K, pi, phi[node], int(node), nbrs[r], nby[r], beta,
                                          resolved.alpha, resolved.epsilon, eps, net.N,
                                          resolved.num_node_sample, pn[r], dtype)
        pi[node] = keep
    new_pi = pi.copy()
    idx = mb["nodes"]
    new_pi[idx] = oracle.normalize(new_phi[idx], dtype)
    ea = mb["nodes"][mb["edge_a"]]
    eb = mb["nodes"][mb["edge_b"]]
    eta = np.array([resolved.eta0, resolved.eta1])
    th2, bt2, grads = oracle.update_beta(K, new_pi, ea, eb, mb["edge_y"], th, beta, eta,
                                         resolved.epsilon, eps, mb["scale"], tn, dtype)
    return new_phi, new_pi, th2, bt2


def phi_terms(net, resolved, phi, theta, mb, nbrs, nby, pn, step, pi_nbr=None):
    """FP64 magnitude of the terms that make up each new phi element,
    |phi| + eps/2 (|alpha| + |phi| + Nn G) + |sqrt(eps phi) noise|, with
    G = sum_j (|probs_jk / (P_j phi_k)| + 1/S) the sum of the absolute
    values of the gradient's terms (the condition of that cancelling sum):
    the scale against which floating-point rounding is measured."""
    K = phi.shape[1]
    phi64 = phi.astype(np.float64)
    pi64 = oracle.normalize(phi64, np.float64) if pi_nbr is None else pi_nbr.astype(np.float64)
    own = oracle.normalize(phi64[mb["nodes"]], np.float64)
    th = theta.astype(np.float64)
    beta = th[:, 1] / th.sum(1)
    eps = float(oracle.eps_t(resolved.a, resolved.b, resolved.c, step))
    Nn = net.N / resolved.num_node_sample
    M = np.zeros((len(mb["nodes"]), K))
    for r, node in enumerate(mb["nodes"]):
        keep = pi64[node].copy()
        pi64[node] = own[r]
        p = phi64[node]
        S = p.sum()
        yv = nby[r].astype(bool)[:, None]
        f = np.where(yv, beta[None, :] - resolved.epsilon, resolved.epsilon - beta[None, :])
        e = np.where(yv, resolved.epsilon, 1.0 - resolved.epsilon)
        probs = pi64[node][None, :] * (pi64[nbrs[r]] * f + e)
        G = (np.abs(probs / probs.sum(1, keepdims=True) / p[None, :]) + 1.0 / S).sum(0)
        pi64[node] = keep
        M[r] = np.abs(p) + eps / 2 * (abs(resolved.alpha) + np.abs(p) + Nn * G) + \
            np.abs(np.sqrt(eps * p) * pn[r])
    return M


def check_theta(s, K, theta, mb, tn, step, want_th, want_bt, f_th, f_bt):
    """theta/beta are FP64 on the device.  Isolated: update_beta on the
    device's own new pi (its phi rows normalised) in FP64 must match to 1e-6
    of the update's term magnitude |theta| + eps/2 |eta - theta + scale G| +
    |sqrt(eps theta) noise|; end to end within 1e-4 of that magnitude from
    the FP64 chain plus twice the float restatement's own rounding."""
    new_pi = oracle.normalize(s.phi.astype(np.float64), np.float64)
    th64 = theta.astype(np.float64)
    bt_dev = (th64[:, 1] / th64.sum(1)).astype(np.float32).astype(np.float64)
    eps = float(oracle.eps_t(s.resolved.a, s.resolved.b, s.resolved.c, step))
    eta = np.array([s.resolved.eta0, s.resolved.eta1])
    iso_th, _, G = oracle.update_beta(
        K, new_pi, mb["nodes"][mb["edge_a"]], mb["nodes"][mb["edge_b"]], mb["edge_y"], th64,
        bt_dev, eta, s.resolved.epsilon, eps, mb["scale"], tn, np.float64)
    M = np.abs(th64) + eps / 2 * np.abs(eta[None, :] - th64 + mb["scale"] * G) + \
        np.abs(np.sqrt(eps * th64) * tn.astype(np.float64))
    gth = s.theta
    assert np.all(np.abs(gth - iso_th) <= 1e-6 * M), float(np.max(np.abs(gth - iso_th) / M))
    e_ref = np.abs(want_th.astype(np.float64) - f_th)
    assert np.all(np.abs(gth - f_th) <= RTOL_F64 * M + 2 * e_ref)
    gbt = s.beta.astype(np.float64)
    bt_from_th = gth[:, 1] / gth.sum(1)
    assert np.allclose(gbt, bt_from_th, rtol=1e-6)


def run_fed_case(net, K, step, dtype, strategy=0, mini_batch_size=None, num_node_sample=32,
                 sampler_max_source=1, stats=None):
    kw = dict(K=K, num_node_sample=num_node_sample, strategy=strategy,
              sampler_max_source=sampler_max_source)
    if mini_batch_size:
        kw["mini_batch_size"] = mini_batch_size
    s, opts = make_sampler(net, dtype, **kw)
    phi, theta = random_state(net.N, K, seed=step)
    s.set_state(phi, theta)
    pi_dev = s.pi  # the stored pi the kernel gathers neighbour rows from
    og = oracle.OracleGraph(net)
    mb = oracle.sample_minibatch(og, strategy, s.resolved.mini_batch_size, net.num_total_edges,
                                 opts.random_seed, 0, step, s.max_edges,
                                 max_source=sampler_max_source)
    n_out = s.num_node_sample + 1
    nbrs = np.zeros((len(mb["nodes"]), n_out), np.int32)
    nby = np.zeros_like(nbrs, dtype=np.uint8)
    for r, node in enumerate(mb["nodes"]):
        nbrs[r], nby[r] = oracle.sample_neighbors(og, int(node), n_out, opts.random_seed, 0, step)
    rng = np.random.default_rng(step)
    pn = rng.standard_normal((len(mb["nodes"]), K)).astype(np.float32)
    tn = rng.standard_normal((K, 2)).astype(np.float32)
    s.step_fed(step, np.stack([mb["edge_a"], mb["edge_b"]], 1), mb["edge_y"], mb["scale"],
               mb["nodes"], nbrs, nby, pn, tn)
    want = oracle_fed_step(net, opts, s.resolved, phi, theta, mb, nbrs, nby, pn, tn, step,
                           np.float32, pi_dev)
    f64 = oracle_fed_step(net, opts, s.resolved, phi, theta, mb, nbrs, nby, pn, tn, step,
                          np.float64, pi_dev)
    M = phi_terms(net, s.resolved, phi, theta, mb, nbrs, nby, pn, step, pi_dev)
    idx = mb["nodes"]
    gphi = s.phi
    st = check_phi(gphi[idx], want[0][idx], f64[0][idx], M)
    if stats is not None:
        stats.update(st, nodes=len(idx), n_out=n_out, flag=int(mb["flag"]))
    untouched = np.setdiff1d(np.arange(net.N), idx)
    assert np.array_equal(gphi[untouched], phi[untouched])
    gpi = s.pi
    if dtype == _native.PI_F32:
        assert np.all(np.linalg.norm(gpi[idx] - want[1][idx], axis=1) /
                      np.linalg.norm(want[1][idx], axis=1) < RTOL_STEP)
    else:  # committed rows: the BF16 rounding of the device's own new FP32 row
        own = gphi[idx].astype(np.float64)
        own /= own.sum(1, keepdims=True)
        assert np.all(np.abs(gpi[idx] - own) <= (2.0 ** -8 + 1e-6) * np.abs(own) + 1e-30)
    assert np.array_equal(gpi[untouched], pi_dev[untouched])
    check_theta(s, K, theta, mb, tn, step, want[2], want[3], f64[2], f64[3])
    s.close()
    return mb


@pytest.mark.parametrize("dtype", [_native.PI_F32, _native.PI_BF16])
@pytest.mark.parametrize("K", [32, 20])
@pytest.mark.parametrize("step", [1, 37])
def test_fed_step_matches_oracle(small, K, step, dtype):
    net, _ = small
    run_fed_case(net, K, step, dtype)


@pytest.mark.parametrize("dtype", [_native.PI_F32, _native.PI_BF16])
@pytest.mark.parametrize("K,nns", [(8, 13), (12, 3), (16, 31)])
def test_fed_step_narrow_rows_split(small, K, nns, dtype):
    """Rows narrower than a warp: 1-4 lanes per node and the node's
    neighbours split over 8 sub-groups (shapes 1x8, 2x8, 4x8), with rows per
    sub-group uneven (14 and 32 neighbour rows) or fewer rows than
    sub-groups (4 rows: half the sub-groups have none)."""
    net, _ = small
    run_fed_case(net, K, 11, dtype, num_node_sample=nns)


@pytest.mark.parametrize("dtype", [_native.PI_F32, _native.PI_BF16])
def test_fed_step_link_stratum(small, dtype):
    """A link-stratum (y = 1) minibatch through the fed path."""
    net, _ = small
    mb = run_fed_case(net, 32, 5, dtype, strategy=1)
    assert mb["flag"] == 1 and mb["edge_y"].all()


@pytest.fixture(scope="module")
def wide_net(native_lib):
    net = Network.synthetic(n=3000, k_true=30, intra_degree=6.0, seed=4)
    net.make_held_out(0.02, seed=4)
    return net


@pytest.mark.parametrize("dtype", [_native.PI_F32, _native.PI_BF16])
@pytest.mark.parametrize("K", [1024, 256, 200, 64])
def test_fed_step_wide_rows(wide_net, K, dtype):
    """Wide-row kernels: the shared-memory ring (rows of >= 32 vectors; BF16
    K = 200 has padded rows, partly empty lane vectors) and the sub-warp
    register path (K = 64)."""
    run_fed_case(wide_net, K, 3, dtype, mini_batch_size=64, num_node_sample=40)


@pytest.mark.parametrize("stages", ["3", "6"])
def test_fed_step_ring_depths(wide_net, stages, monkeypatch):
    """The ring kernel at other ring depths (rows per warp not a
    multiple of the depth: 41 neighbours over 4 warps)."""
    monkeypatch.setenv("AMMSB_PHI_RING", stages)
    run_fed_case(wide_net, 1024, 9, _native.PI_BF16, mini_batch_size=64, num_node_sample=40)


@pytest.mark.parametrize("dtype", [_native.PI_F32, _native.PI_BF16])
@pytest.mark.parametrize("K", [1024, 256])
def test_fed_step_link_stratum_wide_rows(wide_net, K, dtype):
    """Few nodes (the link stratum) on the ring update."""
    run_fed_case(wide_net, K, 13, dtype, strategy=1, mini_batch_size=64, num_node_sample=40)


@pytest.mark.parametrize("dtype", [_native.PI_F32, _native.PI_BF16])
@pytest.mark.parametrize("strategy", [0, 1, 2])
def test_fed_step_ring_fewer_rows_than_depth(wide_net, dtype, strategy):
    """Three neighbour rows per node on the ring kernel: warps with fewer rows
    than the ring depth (empty commit groups) and warps with none."""
    run_fed_case(wide_net, 1024, 17, dtype, strategy=strategy, mini_batch_size=64, num_node_sample=2)


def test_fed_step_many_nodes_per_cta(wide_net):
    """More minibatch nodes than CTAs of one wave, on the ring kernel:
    every CTA restarts its warps' rings at each node."""
    run_fed_case(wide_net, 256, 7, _native.PI_BF16, strategy=2, mini_batch_size=1400,
                 num_node_sample=20)


# ---------------------------------------------------------------------------
# perplexity
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("dtype", [_native.PI_F32, _native.PI_BF16])
@pytest.mark.parametrize("K", [32, 24, 1024])
def test_perplexity_matches_oracle(small, K, dtype):
    net, _ = small
    s, opts = make_sampler(net, dtype, K=K)
    phi, theta = random_state(net.N, K, seed=11)
    s.set_state(phi, theta)
    pi = s.pi
    beta = s.beta
    ppx = np.zeros(len(net.held_out[0]), np.float32)
    for c in (1, 2, 3):
        got = s.cal_perplexity_held_out()
        want = oracle.perplexity(K, pi, net.held_out, beta, s.resolved.epsilon, ppx, c, "f64acc")
        assert got == pytest.approx(want, rel=RTOL_PPX)
        assert rel_err(s.ppx_per_heldout_edge, ppx) < 1e-5
    ref = oracle.perplexity(K, pi, net.held_out, beta, s.resolved.epsilon,
                            np.zeros_like(ppx), 1, "f32")
    assert np.isfinite(ref)
    s.close()


# ---------------------------------------------------------------------------
# trajectories
# ---------------------------------------------------------------------------
def run_trajectory(s, iters, interval):
    out = []
    for it in range(iters):
        if it % interval == 0:
            out.append(s.cal_perplexity_held_out())
        s.step(1)
    return np.array(out)


def test_trajectory_small_vs_oracle(small):
    """The small workload (2,000 iterations, perplexity every 100): GPU FP32
    against the oracle sampler with the same Philox draws."""
    net, opts = small
    s = MCMCSamplerStochastic(opts, net).create()
    phi, theta = random_state(net.N, 32, seed=21)
    s.set_state(phi, theta)
    r = s.resolved
    orc = oracle.OracleSampler(net, 32, mini_batch_size=r.mini_batch_size,
                               num_node_sample=r.num_node_sample, alpha=r.alpha,
                               epsilon=r.epsilon, a=r.a, b=r.b, c=r.c, seed=r.random_seed)
    orc.set_state(phi, theta)
    got, want = [], []
    for it in range(2000):
        if it % 100 == 0:
            got.append(s.cal_perplexity_held_out())
            want.append(orc.perplexity())
        s.step(1)
        orc.step()
    got, want = np.array(got), np.array(want)
    assert np.all(np.abs(got - want) <= 0.01 * np.abs(want)), (got, want)
    s.close()


def test_trajectory_bf16_within_1pct_of_f32(small):
    net, opts = small
    traj = {}
    for dtype in (_native.PI_F32, _native.PI_BF16):
        o = Options(**{k: getattr(opts, k) for k in ("K", "alpha", "a", "b", "c", "num_node_sample",
                                                     "held_out_ratio")}, pi_dtype=dtype)
        s = MCMCSamplerStochastic(o, net).create()
        s.set_state(*random_state(net.N, 32, seed=21))
        traj[dtype] = run_trajectory(s, 2000, 100)
        s.close()
    f32, bf16 = traj[_native.PI_F32], traj[_native.PI_BF16]
    assert np.all(np.abs(bf16 - f32) <= 0.01 * np.abs(f32)), (f32, bf16)


# ---------------------------------------------------------------------------
# init, driver loop, errors
# ---------------------------------------------------------------------------
def test_init_state(small):
    net, _ = small
    s, opts = make_sampler(net)
    s.init()
    phi = s.phi
    assert abs(phi.mean() - 1.0) < 0.02 and abs(phi.var() - 1.0) < 0.05
    assert np.allclose(s.pi.sum(1), 1.0, atol=1e-5)
    # theta follows the host gamma stream; the oracle computes the same draws
    want = np.array([[oracle.lib().oracle_gamma(42, 0, oracle.P_THETA_INIT, 0, 2 * k + c,
                                                1.0, 1.0) for c in range(2)] for k in range(32)])
    assert rel_err(s.theta, want) < 1e-12
    # phi on the device: the same Marsaglia-Tsang stream in device FP64
    sub = np.array([[oracle.lib().oracle_gamma(42, 0, oracle.P_PHI_INIT, v, k, 1.0, 1.0)
                     for k in range(32)] for v in range(50)], np.float32)
    assert rel_err(phi[:50], sub) < 1e-6
    s.close()


def test_run_prints_reference_lines(small, capfd):
    net, opts = small
    o = Options(K=32, num_node_sample=32, max_iteration=201, interval=100, held_out_ratio=0.02)
    s = MCMCSamplerStochastic(o, net).create()
    s.init()
    last = s.run()
    out = capfd.readouterr().out.strip().splitlines()
    lines = [l for l in out if l.startswith("average_count is:")]
    # the loop runs while step_count < max_iteration (cc:110): perplexity at
    # steps 1 and 101, the last update is step 200; average_count is printed
    # after cal_perplexity advanced it (cc:112-118, learner.cc:180)
    assert len(lines) == 2
    assert lines[0].startswith("average_count is: 2 step count: 1 time: ")
    assert lines[1].startswith("average_count is: 3 step count: 101 time: ")
    assert float(lines[1].split()[-1]) == pytest.approx(last, rel=1e-12)
    assert s.step_count == 201
    s.close()


def test_errors(small):
    net, _ = small
    with pytest.raises(_native.AmmsbError) as e:
        MCMCSamplerStochastic(Options(K=0), net).create()
    assert e.value.code == -1
    for bad in (dict(strategy=4), dict(sampler_max_source=0), dict(sampler_max_source=5000)):
        with pytest.raises(_native.AmmsbError) as e:
            MCMCSamplerStochastic(Options(K=16, **bad), net).create()
        assert e.value.code == -1
    s, _ = make_sampler(net)
    with pytest.raises(_native.AmmsbError) as e:
        s.step(1)
    assert e.value.code == -5
    s.close()


# ---------------------------------------------------------------------------
# the CUDA path against the reference's own outputs (tests/golden/ref_*.npz)
# ---------------------------------------------------------------------------
import glob as _glob
import os as _os

_FIXTURES = sorted(_glob.glob(_os.path.join(_os.path.dirname(_os.path.abspath(__file__)),
                                            "golden", "ref_*.npz")))


@pytest.mark.parametrize("path", _FIXTURES, ids=[_os.path.basename(p) for p in _FIXTURES])
def test_gpu_against_reference_fixture(native_lib, path):
    d = dict(np.load(path))
    N, K, nns = int(d["N"]), int(d["K"]), int(d["nns"])
    net = Network.from_edges(N, d["edge_a"], d["edge_b"])
    net.held_out = (d["ho_a"], d["ho_b"], d["ho_y"])
    net.test = (d["te_a"], d["te_b"], d["te_y"])
    E = set(zip(d["edge_a"].tolist(), d["edge_b"].tolist()))
    opts = Options(K=K, num_node_sample=nns, mini_batch_size=int(d["mbs"]), a=float(d["a"]),
                   b=float(d["b"]), c=float(d["c"]), alpha=float(np.float32(d["alpha"])),
                   epsilon=float(d["epsilon"]))
    s = MCMCSamplerStochastic(opts, net).create()
    # update_phi of the reference's nodes, neighbour sets and noise
    s.set_state(d["phi"], d["theta"].astype(np.float64))
    nodes = d["phi_nodes"]
    nbrs = d["phi_order"]
    nby = np.array([[(min(v, j), max(v, j)) in E for j in row] for v, row in zip(nodes, nbrs)],
                   np.uint8)
    s.step_fed(int(d["step"]), np.zeros((0, 2), np.int32), np.zeros(0, np.uint8), 1.0, nodes,
               nbrs, nby, d["phi_noise"], np.zeros((K, 2), np.float32))
    mb = dict(nodes=nodes)
    f64 = np.zeros((len(nodes), K))
    pi64 = d["pi"].astype(np.float64)
    for r, v in enumerate(nodes):
        f64[r] = oracle.update_phi(K, pi64, d["phi"][v], int(v), nbrs[r], nby[r],
                                   d["beta"].astype(np.float64), float(d["alpha"]),
                                   float(d["epsilon"]), float(d["eps"]), N, nns,
                                   d["phi_noise"][r], np.float64)
    M = phi_terms(net, s.resolved, d["phi"], d["theta"], mb, nbrs, nby, d["phi_noise"],
                  int(d["step"]), d["pi"])
    check_phi(s.phi[nodes], d["phi_out"], f64, M)
    # perplexity on the reference's state after update_beta (beta_out)
    s.set_state(d["phi"], d["theta_out"].astype(np.float64))
    p1 = s.cal_perplexity_held_out()
    p2 = s.cal_perplexity_held_out()
    assert p1 == pytest.approx(float(d["ppx1"]), rel=RTOL_PPX)
    assert p2 == pytest.approx(float(d["ppx2"]), rel=RTOL_PPX)
    assert rel_err(s.ppx_per_heldout_edge, d["ppx_edges2"]) < RTOL_PPX
    s.close()
