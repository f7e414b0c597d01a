"""The minibatch edge log-likelihood and its hand-written adjoint kernels.

Differentiation case: the planted-community graph with N=2,000, K_true=20
(~6k edges), model K=16; phi and theta iid Gamma(100, 0.01) in FP64; one
fixed minibatch of 50 nodes x 32 sampled neighbours.  The adjoint is checked
  * against central finite differences (h = 1e-6) of the FP64 forward with
    torch.autograd.gradcheck (atol 1e-6, rtol 1e-5: the loss is ~-70, so
    its FP64 rounding over 2h is ~1e-8);
  * against the reference's hand-derived gradients, as restated by the
    oracle: update_phi's grads (mcmc_sampler_stochastic.cc:274-296) and
    update_beta's grads (cc:212-240), to 1e-9 relative;
  * against a plain torch FP64 expression of the same forward and its
    autograd gradient, at K = 40 and K = 1024 (row widths of 2 and 32
    values per lane);
and FP32 against FP64 to 1e-4 of the gradient magnitude.
"""
import numpy as np
import pytest

import oracle
from mcmc_for_ammsb_gb300 import workloads

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

H = 1e-6
EPS = 1e-7


def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")


def c2_case(K=16, n_nodes=50, n_out=32, seed=11):
    net, _ = workloads.build("diff")
    rng = np.random.default_rng(seed)
    phi = rng.gamma(100.0, 0.01, (net.N, K))
    theta = rng.gamma(100.0, 0.01, (K, 2))
    og = oracle.OracleGraph(net)
    nodes = rng.choice(net.N, n_nodes, replace=False).astype(np.int32)
    nb, ys = [], []
    for v in nodes:
        o, y = oracle.sample_neighbors(og, int(v), n_out, 42, 0, 1)
        nb.append(o)
        ys.append(y)
    return net, phi, theta, nodes, np.stack(nb), np.stack(ys)


def torch_inputs(phi, theta, nodes, nbrs, ys, dtype=torch.float64):
    pi = phi / phi.sum(1, keepdims=True)
    uniq, inv = np.unique(nbrs.ravel(), return_inverse=True)
    dev = "cuda"
    phi_src = torch.tensor(phi[nodes], dtype=dtype, device=dev, requires_grad=True)
    pi_nbr = torch.tensor(pi[uniq], dtype=dtype, device=dev, requires_grad=True)
    th = torch.tensor(theta, dtype=dtype, device=dev, requires_grad=True)
    src = torch.arange(len(nodes), device=dev).repeat_interleave(nbrs.shape[1])
    nbr = torch.tensor(inv.reshape(-1), device=dev)
    y = torch.tensor(ys.ravel(), dtype=torch.uint8, device=dev)
    return phi_src, pi_nbr, th, src, nbr, y, uniq


def torch_reference(phi_src, pi_nbr, theta, src, nbr, y, eps):
    """The same forward as a plain torch expression (autograd reference)."""
    pa = phi_src / phi_src.sum(1, keepdim=True)
    beta = theta[:, 1] / theta.sum(1)
    yf = y.to(pa.dtype)
    sig = 2.0 * yf - 1.0
    e = yf * eps + (1.0 - yf) * (1.0 - eps)
    D = (pa[src] * pi_nbr[nbr] * (beta - eps)[None, :]).sum(1)
    return torch.log(sig * D + e).sum()


def test_gradcheck_central_differences(native_lib):
    _need_gpu()
    from mcmc_for_ammsb_gb300.autograd import edge_log_likelihood
    net, phi, theta, nodes, nbrs, ys = c2_case()
    phi_src, pi_nbr, th, src, nbr, y, _ = torch_inputs(phi, theta, nodes, nbrs, ys)

    def f(a, b, c):
        return edge_log_likelihood(a, b, c, src, nbr, y, EPS)

    assert torch.autograd.gradcheck(f, (phi_src, pi_nbr, th), eps=H, atol=1e-6, rtol=1e-5)


def test_adjoint_equals_reference_hand_derived_gradients(native_lib):
    _need_gpu()
    from mcmc_for_ammsb_gb300.autograd import edge_log_likelihood
    K = 16
    net, phi, theta, nodes, nbrs, ys = c2_case(K=K)
    phi_src, pi_nbr, th, src, nbr, y, _ = torch_inputs(phi, theta, nodes, nbrs, ys)
    L = edge_log_likelihood(phi_src, pi_nbr, th, src, nbr, y, EPS)
    gphi, gth = torch.autograd.grad(L, (phi_src, th))
    gphi = gphi.cpu().numpy()
    gth = gth.cpu().numpy()

    pi = phi / phi.sum(1, keepdims=True)
    beta = theta[:, 1] / theta.sum(1)
    for r, v in enumerate(nodes):
        want = oracle.phi_grad(K, pi, phi[v], int(v), nbrs[r], ys[r], beta, EPS)
        np.testing.assert_allclose(gphi[r], want, rtol=1e-9, atol=1e-11)
    ea = np.repeat(nodes, nbrs.shape[1]).astype(np.int32)
    eb = nbrs.ravel().astype(np.int32)
    _, _, want_th = oracle.update_beta(K, pi, ea, eb, ys.ravel(), theta, beta,
                                       np.array([1.0, 1.0]), EPS, 0.01, 1.0,
                                       np.zeros((K, 2)), dtype=np.float64)
    np.testing.assert_allclose(gth, want_th, rtol=1e-9, atol=1e-11)

    # the forward is the log of update_beta's prob_sum (cc:212-240) summed
    # over the pairs; cal_edge_likelihood (learner.h:100-139) differs from it
    # only by leaving out the eps * (1 - sum pi_a pi_b) term of a link
    pa = pi[np.repeat(nodes, nbrs.shape[1])]
    pb = pi[nbrs.ravel()]
    yv = ys.ravel().astype(bool)
    f = np.where(yv[:, None], beta[None, :], 1.0 - beta[None, :])
    e = np.where(yv, EPS, 1.0 - EPS)
    s_ab = (pa * pb).sum(1)
    want_L = np.log((pa * pb * f).sum(1) + e * (1.0 - s_ab)).sum()
    assert float(L.detach()) == pytest.approx(want_L, rel=1e-12)
    ce = np.array([oracle.edge_likelihood(K, pi[v], pi[j], yy, beta, EPS)
                   for r, v in enumerate(nodes) for j, yy in zip(nbrs[r], ys[r])])
    np.testing.assert_allclose(ce, np.where(yv, (pa * pb * f).sum(1),
                                            (pa * pb * f).sum(1) + e * (1.0 - s_ab)),
                               rtol=1e-13)


@pytest.mark.parametrize("K", [40, 1024])
def test_adjoint_matches_torch_autograd(native_lib, K):
    _need_gpu()
    from mcmc_for_ammsb_gb300.autograd import edge_log_likelihood
    net, phi, theta, nodes, nbrs, ys = c2_case(K=K, n_nodes=20, n_out=16)
    phi_src, pi_nbr, th, src, nbr, y, _ = torch_inputs(phi, theta, nodes, nbrs, ys)
    L = edge_log_likelihood(phi_src, pi_nbr, th, src, nbr, y, EPS)
    g = torch.autograd.grad(L, (phi_src, pi_nbr, th))
    a, b, c = (t.detach().clone().requires_grad_(True) for t in (phi_src, pi_nbr, th))
    Lr = torch_reference(a, b, c, src, nbr, y, EPS)
    gr = torch.autograd.grad(Lr, (a, b, c))
    assert float(L.detach()) == pytest.approx(float(Lr.detach()), rel=1e-12)
    for mine, ref in zip(g, gr):
        scale = float(ref.abs().max())
        assert float((mine - ref).abs().max()) <= 1e-11 * scale


def test_fp32_against_fp64(native_lib):
    _need_gpu()
    from mcmc_for_ammsb_gb300.autograd import edge_log_likelihood
    net, phi, theta, nodes, nbrs, ys = c2_case()
    out = {}
    for dt in (torch.float64, torch.float32):
        phi_src, pi_nbr, th, src, nbr, y, _ = torch_inputs(phi, theta, nodes, nbrs, ys, dtype=dt)
        L = edge_log_likelihood(phi_src, pi_nbr, th, src, nbr, y, EPS)
        out[dt] = [float(L.detach())] + [t.double().cpu() for t in torch.autograd.grad(
            L, (phi_src, pi_nbr, th))]
    assert out[torch.float32][0] == pytest.approx(out[torch.float64][0], rel=1e-5)
    for a, b in zip(out[torch.float32][1:], out[torch.float64][1:]):
        assert float((a - b).abs().max()) <= 1e-4 * float(b.abs().max())


def test_backward_is_deterministic_and_handles_edge_cases(native_lib):
    _need_gpu()
    from mcmc_for_ammsb_gb300.autograd import edge_log_likelihood
    net, phi, theta, nodes, nbrs, ys = c2_case()
    phi_src, pi_nbr, th, src, nbr, y, _ = torch_inputs(phi, theta, nodes, nbrs, ys)
    runs = []
    for _ in range(2):
        L = edge_log_likelihood(phi_src, pi_nbr, th, src, nbr, y, EPS)
        runs.append(torch.autograd.grad(L, (phi_src, pi_nbr, th)))
    for a, b in zip(*runs):
        assert torch.equal(a, b)

    # no pairs: zero loss, zero gradients
    e = torch.empty(0, dtype=torch.int64, device="cuda")
    L = edge_log_likelihood(phi_src, pi_nbr, th, e, e, e.to(torch.uint8), EPS)
    g = torch.autograd.grad(L, (phi_src, pi_nbr, th))
    assert float(L.detach()) == 0.0 and all(float(t.abs().max()) == 0.0 for t in g)

    # neighbour rows without pairs get zero gradient; pi_nbr without grad
    extra = torch.rand(3, phi_src.shape[1], dtype=torch.float64, device="cuda")
    pin2 = torch.cat([pi_nbr.detach(), extra]).requires_grad_(True)
    L = edge_log_likelihood(phi_src, pin2, th, src, nbr, y, EPS)
    gp = torch.autograd.grad(L, pin2)[0]
    assert float(gp[-3:].abs().max()) == 0.0
    L = edge_log_likelihood(phi_src, pi_nbr.detach(), th, src, nbr, y, EPS)
    assert torch.autograd.grad(L, th)[0].shape == th.shape


def test_out_of_range_pairs_are_rejected(native_lib):
    _need_gpu()
    from mcmc_for_ammsb_gb300.autograd import EdgeLogLikelihood, edge_log_likelihood, group_pairs
    net, phi, theta, nodes, nbrs, ys = c2_case()
    phi_src, pi_nbr, th, src, nbr, y, _ = torch_inputs(phi, theta, nodes, nbrs, ys)
    bad = nbr.clone()
    bad[5] = pi_nbr.shape[0]
    with pytest.raises(IndexError):
        edge_log_likelihood(phi_src, pi_nbr, th, src, bad, y, EPS)
    # past the host check, the kernels' own bounds checks skip and flag it
    groups = list(group_pairs(src, nbr, y, phi_src.shape[0], pi_nbr.shape[0]))
    groups[1] = groups[1].clone()
    groups[1][7] = pi_nbr.shape[0]
    with pytest.raises(IndexError):
        EdgeLogLikelihood.apply(phi_src, pi_nbr, th, *groups, EPS)
