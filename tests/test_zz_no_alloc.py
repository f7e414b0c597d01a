"""ammsb_perplexity_noalloc: the held-out perplexity for callers that cannot
allocate GPU memory, checked against the handle's ammsb_perplexity.

The caller here owns its device buffers (torch tensors stand in for memory a
host framework hands out) and calls the entry point through the C ABI; the
result and the updated running averages must agree with the handle path
within the perplexity tolerance of the other GPU tests, on two consecutive
calls (the second also exercises reuse of the shared static scratch), also
when the caller's rows are wider than K and their padding holds non-zero
values.  Pairs outside the caller's pi are rejected without a row being
read.  This
file is collected last, and passes alone in a fresh process as well as
after the other tests.
"""
import ctypes

import numpy as np
import pytest

from mcmc_for_ammsb_gb300 import MCMCSamplerStochastic, Options, _native, workloads

pytestmark = pytest.mark.gpu

RTOL_PPX = 1e-5  # the perplexity tolerance of tests/test_gpu_parity.py


def _call(L, pi_dev, dtype, K, stride, n_rows, beta_dev, epsilon, ha, hb, hy, H, ppx_dev, count,
          stream):
    out = ctypes.c_double()
    rc = L.ammsb_perplexity_noalloc(
        ctypes.c_void_p(pi_dev.data_ptr()), dtype, K, stride, n_rows,
        ctypes.c_void_p(beta_dev.data_ptr()), epsilon, ctypes.c_void_p(ha.data_ptr()),
        ctypes.c_void_p(hb.data_ptr()), ctypes.c_void_p(hy.data_ptr()), H,
        ctypes.c_void_p(ppx_dev.data_ptr()), count, ctypes.c_void_p(stream.cuda_stream),
        ctypes.byref(out))
    return rc, out.value


# (K, extra stride elements, padding value): rows exactly as wide as K; K = 20
# (not a multiple of the 16-byte vector) in a wider row whose padding holds
# non-zero values, which must not enter the sums; a row stride above 1,024
# elements (pi as a column slice of a wider matrix)
ROWS = [(32, 0, 0.0), (1024, 0, 0.0), (20, 16, 7.0), (32, 2016, 3.0)]


@pytest.mark.parametrize("dtype", [_native.PI_F32, _native.PI_BF16])
@pytest.mark.parametrize("K,extra,pad", ROWS)
def test_noalloc_perplexity_matches_handle(native_lib, dtype, K, extra, pad):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    net, _ = workloads.build("small")
    s = MCMCSamplerStochastic(Options(K=K, num_node_sample=32, pi_dtype=dtype), net).create()
    rng = np.random.default_rng(3)
    phi = rng.gamma(1.0, 1.0, (net.N, K)).astype(np.float32) + np.float32(1e-4)
    theta = rng.gamma(1.0, 1.0, (K, 2)) + 0.05
    s.set_state(phi, theta)
    pi = s.pi          # the stored pi, exactly (BF16 values are exact in float)
    beta = s.beta

    # the caller's own device buffers: pi rows padded to a 16-byte stride,
    # the padding filled with `pad`
    ev = 8 if dtype == _native.PI_BF16 else 4
    Kp = (K + ev - 1) // ev * ev + extra
    assert Kp % ev == 0
    tdt = torch.bfloat16 if dtype == _native.PI_BF16 else torch.float32
    pi_dev = torch.full((net.N, Kp), pad, dtype=tdt, device="cuda")
    pi_dev[:, :K] = torch.from_numpy(pi).to(device="cuda", dtype=tdt)
    beta_dev = torch.from_numpy(beta).cuda()
    ha = torch.from_numpy(net.held_out[0]).cuda()
    hb = torch.from_numpy(net.held_out[1]).cuda()
    hy = torch.from_numpy(net.held_out[2]).cuda()
    H = int(net.held_out[0].shape[0])
    ppx_dev = torch.zeros(H, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()

    L = native_lib
    for count in (1, 2):
        rc, got = _call(L, pi_dev, dtype, K, Kp, net.N, beta_dev, s.resolved.epsilon, ha, hb, hy,
                        H, ppx_dev, count, stream)
        assert rc == 0
        want = s.cal_perplexity_held_out()  # the existing entry point, same count
        assert got == pytest.approx(want, rel=RTOL_PPX)
        got_ppx = ppx_dev.cpu().numpy()
        want_ppx = s.ppx_per_heldout_edge
        assert np.max(np.abs(got_ppx - want_ppx) / np.abs(want_ppx)) < RTOL_PPX
    s.close()


def test_noalloc_rejects_pairs_outside_pi(native_lib):
    """A held-out pair that names a row past n_rows is skipped on the device
    before any row is read, and the call reports it; the call after it,
    with valid pairs, succeeds (the flag is cleared per call)."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    K, H, n_rows = 32, 600, 500
    rng = np.random.default_rng(4)
    pi = rng.gamma(1.0, 1.0, (n_rows, K)).astype(np.float32)
    pi /= pi.sum(1, keepdims=True)
    pi_dev = torch.from_numpy(pi).cuda()
    beta_dev = torch.full((K,), 0.3, dtype=torch.float32, device="cuda")
    a = rng.integers(0, n_rows, H).astype(np.int32)
    b = rng.integers(0, n_rows, H).astype(np.int32)
    y = (rng.random(H) < 0.5).astype(np.uint8)
    ha, hb, hy = (torch.from_numpy(x).cuda() for x in (a, b, y))
    ppx_dev = torch.zeros(H, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    bad = hb.clone()
    bad[17] = n_rows       # one past the last row
    bad[301] = -5          # negative
    torch.cuda.synchronize()
    rc, _ = _call(native_lib, pi_dev, _native.PI_F32, K, K, n_rows, beta_dev, 1e-7, ha, bad, hy,
                  H, ppx_dev, 1, stream)
    assert rc == -1
    ppx = ppx_dev.cpu().numpy()
    assert ppx[17] == 0.0 and ppx[301] == 0.0 and np.all(np.delete(ppx, [17, 301]) > 0)
    ppx_dev.zero_()
    rc, got = _call(native_lib, pi_dev, _native.PI_F32, K, K, n_rows, beta_dev, 1e-7, ha, hb, hy,
                    H, ppx_dev, 1, stream)
    assert rc == 0 and np.isfinite(got) and got > 0


def test_noalloc_rejects_sizes_beyond_its_scratch(native_lib):
    out = ctypes.c_double()
    # 4,194,305 held-out edges is one more than the static scratch covers;
    # rejected before any device pointer is touched
    rc = native_lib.ammsb_perplexity_noalloc(
        ctypes.c_void_p(16), _native.PI_F32, 32, 32, 100, ctypes.c_void_p(16), 1e-7,
        ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16), 4194305,
        ctypes.c_void_p(16), 1, None, ctypes.byref(out))
    assert rc == -4
    # a row count below 1 is an argument error, also before any device access
    rc = native_lib.ammsb_perplexity_noalloc(
        ctypes.c_void_p(16), _native.PI_F32, 32, 32, 0, ctypes.c_void_p(16), 1e-7,
        ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16), 10,
        ctypes.c_void_p(16), 1, None, ctypes.byref(out))
    assert rc == -1
