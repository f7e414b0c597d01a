"""Batches of independent chains (ammsb_batch_*) and the update_phi autotuner.

A chain advanced inside a batch runs the same kernel bodies on the same
draws as the chain stepped on its own, so its state must match bit for bit:
the batching workload's chains (own graph from seed i, N log-uniform in
[1,000, 50,000], intra degree 6, K in {16, 32, 64, 128}, uneven minibatch
sizes, 32 neighbours) in FP32 and BF16 pi, stepped as one batch and one by
one.  The autotuner must pick one of the kernel shapes it timed and leave
the chain's state and draws untouched.
"""
import numpy as np
import pytest

from mcmc_for_ammsb_gb300 import ChainBatch, MCMCSamplerStochastic, Network, Options, _native
from mcmc_for_ammsb_gb300 import workloads

pytestmark = pytest.mark.gpu


def _need_gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")


def _chain(i, dtype):
    w = workloads.chain_workload(i)
    net = Network.synthetic(**w["gen"])
    net.make_held_out(w["opts"]["held_out_ratio"], seed=w["gen"]["seed"])
    opts = dict(w["opts"], pi_dtype=dtype)
    return net, opts


def _pair(i, dtype):
    net, opts = _chain(i, dtype)
    a = MCMCSamplerStochastic(Options(**opts), net).init()
    b = MCMCSamplerStochastic(Options(**opts), net).init()
    return a, b


def _same(a, b):
    for name in ("phi", "pi", "theta", "beta"):
        assert np.array_equal(getattr(a, name), getattr(b, name)), name
    assert a.step_count == b.step_count


CHAINS = [(0, _native.PI_BF16), (1, _native.PI_F32), (2, _native.PI_BF16), (3, _native.PI_BF16),
          (4, _native.PI_F32), (5, _native.PI_BF16)]


def test_batch_matches_chains_stepped_alone(native_lib):
    _need_gpu()
    pairs = [_pair(i, dt) for i, dt in CHAINS]
    Ks = {p[0].K for p in pairs}
    assert len(Ks) >= 3  # several row widths in one batch
    batch = ChainBatch([a for a, _ in pairs])
    assert 1 <= batch.groups() <= len(pairs)
    batch.step(30)
    for _, b in pairs:
        b.step(30)
    for a, b in pairs:
        _same(a, b)
    # a chain stepped on its own between batch steps, then the batch again
    pairs[0][0].step(7)
    pairs[0][1].step(7)
    batch.step(11)
    for _, b in pairs:
        b.step(11)
    for a, b in pairs:
        _same(a, b)
    # the perplexity of a batched chain is the chain's own
    for a, b in pairs[:2]:
        assert a.cal_perplexity_held_out() == b.cal_perplexity_held_out()
    batch.close()
    for a, b in pairs:
        a.close()
        b.close()


def test_autotune_picks_a_timed_shape_and_keeps_the_chain(native_lib):
    _need_gpu()
    for i, dt in [(2, _native.PI_BF16), (1, _native.PI_F32)]:
        a, b = _pair(i, dt)
        before = a.phi
        cfg = a.autotune(reps=2, fresh=True)
        assert cfg["lanes"] in (1, 2, 4, 8, 16, 32) and cfg["split"] in (1, 2, 4)
        ev = 8 if dt == _native.PI_BF16 else 4
        nvec = -(-a.K // ev)
        assert cfg["lanes"] * cfg["vectors"] >= nvec
        assert np.array_equal(a.phi, before)  # tuned against a scratch copy
        # the tuned chain draws the same minibatches as the untuned one
        a.step(3)
        b.step(3)
        ma, mb = a.last_minibatch(), b.last_minibatch()
        for k in ("nodes", "nbrs", "edge_a", "edge_b"):
            assert np.array_equal(ma[k], mb[k]), k
        # and stays within the update's tolerance of it (the kernels differ
        # only in the order of their sums)
        assert np.allclose(a.phi, b.phi, rtol=1e-4, atol=1e-6)
        # a second handle of the same shape takes the cached choice
        c = MCMCSamplerStochastic(Options(**_chain(i, dt)[1]), a.network).init()
        assert c.autotune(reps=2) == cfg
        for s in (a, b, c):
            s.close()


def test_batch_of_tuned_chains(native_lib):
    _need_gpu()
    pairs = [_pair(i, dt) for i, dt in CHAINS[:4]]
    for a, b in pairs:
        a.autotune(reps=2)
        b.autotune(reps=2)
    batch = ChainBatch([a for a, _ in pairs])
    batch.step(12)
    for _, b in pairs:
        b.step(12)
    for a, b in pairs:
        _same(a, b)
    batch.close()


def test_batch_rejects_bad_input(native_lib):
    _need_gpu()
    a, _ = _pair(0, _native.PI_BF16)
    with pytest.raises(_native.AmmsbError):
        ChainBatch([a, a])
    with pytest.raises(ValueError):
        ChainBatch([])
