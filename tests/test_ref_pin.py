"""The oracle pinned to the reference's own code.

tests/golden/ref_*.npz hold what the reference's update_phi, update_beta,
cal_perplexity and samplers returned (built from the reference sources by
tests/golden/make_golden.py).  The oracle's float restatements must
reproduce them bit for bit; the live tests (only where the reference-built
library exists) repeat the comparison on fresh random cases."""
import glob
import os

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "ref_*.npz")))


def load(path):
    return dict(np.load(path))


def edge_set(d):
    return set(zip(d["edge_a"].tolist(), d["edge_b"].tolist()))


def y_of(edges, v, js):
    return np.array([(min(v, j), max(v, j)) in edges for j in js], np.uint8)


@pytest.fixture(params=FIXTURES, ids=[os.path.basename(f) for f in FIXTURES])
def golden(request):
    return load(request.param)


def test_fixtures_present():
    assert len(FIXTURES) >= 2


def test_pi_beta_from_state(golden):
    d = golden
    assert np.array_equal(oracle.normalize(d["phi"]), d["pi"])
    th = d["theta"]
    assert np.array_equal((th[:, 1] / (th[:, 0] + th[:, 1])).astype(np.float32), d["beta"])


def test_eps_t(golden):
    d = golden
    args = (float(d["a"]), float(d["b"]), float(d["c"]), int(d["step"]))
    # the reference's float evaluation, bit for bit
    assert oracle.eps_t_ref(*args) == d["eps"]
    # the device evaluates in double and rounds: within one float ulp
    assert abs(oracle.eps_t(*args) - d["eps"]) <= np.spacing(np.float32(d["eps"]))


def test_update_phi_bit_exact(golden):
    d = golden
    E = edge_set(d)
    K = int(d["K"])
    for r, v in enumerate(d["phi_nodes"]):
        order = d["phi_order"][r]
        got = oracle.update_phi(K, d["pi"], d["phi"][v], int(v), order, y_of(E, int(v), order),
                                d["beta"], float(np.float32(d["alpha"])), float(d["epsilon"]),
                                float(d["eps"]), int(d["N"]), int(d["nns"]), d["phi_noise"][r])
        assert np.array_equal(got, d["phi_out"][r]), (r, np.max(np.abs(got - d["phi_out"][r])))


def test_update_beta_bit_exact(golden):
    d = golden
    E = edge_set(d)
    K = int(d["K"])
    ea, eb = d["beta_edge_a"], d["beta_edge_b"]
    ey = np.array([(a, b) in E for a, b in zip(ea.tolist(), eb.tolist())], np.uint8)
    th, bt, _ = oracle.update_beta(K, d["pi"], ea, eb, ey, d["theta"], d["beta"],
                                   np.array([1.0, 1.0], np.float32), float(d["epsilon"]),
                                   float(d["eps"]), float(d["beta_scale"]), d["beta_noise"])
    assert np.array_equal(th, d["theta_out"])
    assert np.array_equal(bt, d["beta_out"])


def test_perplexity_bit_exact(golden):
    d = golden
    K = int(d["K"])
    ho = (d["ho_a"], d["ho_b"], d["ho_y"])
    # recorded after update_beta: beta is beta_out; pi is unchanged (the
    # harness does not renormalise pi after update_phi)
    beta = d["beta_out"]
    ppx = np.zeros(len(d["ho_a"]), np.float32)
    p1 = oracle.perplexity(K, d["pi"], ho, beta, float(d["epsilon"]), ppx, 1, "f32")
    assert np.float32(p1) == d["ppx1"] and np.array_equal(ppx, d["ppx_edges1"])
    p2 = oracle.perplexity(K, d["pi"], ho, beta, float(d["epsilon"]), ppx, 2, "f32")
    assert np.float32(p2) == d["ppx2"] and np.array_equal(ppx, d["ppx_edges2"])
    # the device semantics (FP64 log-sum) agree to 1e-6
    ppx = np.zeros(len(d["ho_a"]), np.float32)
    p64 = oracle.perplexity(K, d["pi"], ho, beta, float(d["epsilon"]), ppx, 1, "f64acc")
    assert p64 == pytest.approx(float(d["ppx1"]), rel=1e-6)


def test_reference_minibatches_follow_the_spec_semantics(golden):
    """Minibatches the reference drew obey what the sampling spec encodes:
    a non-link stratum is mini_batch_size distinct non-edges around one
    source with scale N^2/m * E/(N(N-1)/2 - E); a link stratum is the training
    edges of one node with scale N."""
    d = golden
    E = edge_set(d)
    N, m = int(d["N"]), int(d["mbs"])
    excl = set(zip(d["ho_a"].tolist(), d["ho_b"].tolist())) | \
        set(zip(d["te_a"].tolist(), d["te_b"].tolist()))
    nonlink_scale = oracle.nonlink_scale(N, m, int(d["E"]))
    off = 0
    flags = []
    for size, scale in zip(d["mb_sizes"], d["mb_scales"]):
        pairs = [tuple(p) for p in d["mb_pairs"][off:off + size].tolist()]
        off += size
        linked = [p in E for p in pairs]
        assert all(p not in excl for p in pairs)
        nodes = [x for p in pairs for x in p]
        src = max(set(nodes), key=nodes.count)
        assert all(src in p for p in pairs)  # star around one source
        if all(linked):
            assert scale == np.float32(N)
            flags.append(1)
        else:
            assert not any(linked) and size == m and scale == nonlink_scale
            flags.append(0)
    assert 0 < sum(flags) < len(flags)


# ---------------------------------------------------------------------------
# live comparison with the reference-built library (this container only)
# ---------------------------------------------------------------------------
refbuild = pytest.importorskip("refbuild")
needs_ref = pytest.mark.skipif(not refbuild.available(),
                               reason="reference-built library not present")


@needs_ref
@pytest.mark.parametrize("seed,K,nns", [(11, 8, 6), (12, 33, 20), (13, 64, 40)])
def test_live_reference_matches_oracle(seed, K, nns):
    from mcmc_for_ammsb_gb300 import Network
    net = Network.synthetic(n=400, k_true=5, size_min=10, size_max=150, intra_degree=5.0,
                            seed=seed)
    r = refbuild.RefSampler(net.undirected_edges(),
                            ["--mcmc.K", str(K), "-n", str(nns), "-m", "25",
                             "--mcmc.held-out-ratio", "0.05", "--mcmc.seed", str(seed)])
    try:
        rng = np.random.default_rng(seed)
        phi = (rng.gamma(0.5, 2.0, (r.N, K)) + 1e-4).astype(np.float32)
        theta = (rng.gamma(2.0, 1.0, (K, 2)) + 0.01).astype(np.float32)
        r.set_state(phi, theta)
        _, pi, th, bt = r.state()
        r.set_step(int(rng.integers(1, 5000)))
        eps = r.eps_t()
        a, b = r.edges()
        E = set(zip(a.tolist(), b.tolist()))
        alpha = np.float32(1.0 / K)
        for v in rng.choice(r.N, 5, replace=False):
            nb = r.sample_neighbors(int(v))
            order, noise, out = r.update_phi(int(v), nb, eps)
            got = oracle.update_phi(K, pi, phi[v], int(v), order, y_of(E, int(v), order), bt,
                                    float(alpha), 1e-7, eps, r.N, nns, noise)
            assert np.array_equal(got, out)
        ea, eb, scale = r.sample_minibatch(2000)
        oa, ob, bn, th2, bt2 = r.update_beta(ea, eb, scale)
        ey = np.array([(x, y) in E for x, y in zip(oa.tolist(), ob.tolist())], np.uint8)
        # update_beta reads the reference's pi, which update_phi did not touch
        th3, bt3, _ = oracle.update_beta(K, pi, oa, ob, ey, th, bt, np.array([1, 1], np.float32),
                                         1e-7, eps, scale, bn)
        assert np.array_equal(th3, th2) and np.array_equal(bt3, bt2)
        ho = r.held_out()
        p, ppx = r.perplexity()
        mine = np.zeros(len(ho[0]), np.float32)
        assert np.float32(oracle.perplexity(K, pi, ho, bt2, 1e-7, mine, 1, "f32")) == np.float32(p)
        assert np.array_equal(mine, ppx)
    finally:
        r.close()
