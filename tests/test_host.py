"""CPU tests of the native library's host side: it loads, exports every
entry point of include/ammsb_gpu.h, builds graphs and held-out sets, reads
and writes relativity text; and of the Python option surface."""
import ctypes
import os
import re

import numpy as np
import pytest

from mcmc_for_ammsb_gb300 import Network, Options, _native, workloads
from mcmc_for_ammsb_gb300.options import NumberFormatError, parse_size_t

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "ammsb_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(ammsb_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(native_lib):
    syms = declared_symbols()
    assert len(syms) >= 30
    for s in syms:
        assert hasattr(native_lib, s), s
    # and the ctypes table covers them all
    assert {n for n, _, _ in _native.SIGNATURES} == set(syms)


def test_options_default_matches_reference(native_lib):
    o = _native.AmmsbOptions()
    native_lib.ammsb_options_default(ctypes.byref(o))
    # options.h:144-185
    assert (o.alpha, o.eta0, o.eta1, o.epsilon, o.a, o.b, o.c) == (0.0, 1.0, 1.0, 1e-7, 0.0, 1024, 0.5)
    assert (o.K, o.mini_batch_size, o.num_node_sample, o.strategy, o.sampler_max_source) == (300, 0, 0, 0, 1)
    assert (o.max_iteration, o.interval, o.stats_print_interval, o.num_updates) == (10000000, 0, 0, 1000)
    assert (o.held_out_ratio, o.random_seed, o.convergence_threshold) == (0.0, 42, 1e-12)


def test_python_options_parse_like_reference():
    o = Options(["--mcmc.K", "32", "-m", "1k", "-n", "0x20", "--mcmc.alpha=0.5", "-x", "2001",
                 "--mcmc.strategy", "stratified-random-node-links", "--unknown", "v",
                 "--mcmc.input.contiguous"])
    assert o.K == 32 and o.mini_batch_size == 1024 and o.num_node_sample == 32
    assert o.alpha == 0.5 and o.max_iteration == 2001 and o.strategy == 1
    assert o.input_contiguous_ is True
    assert o.remains == ["--unknown", "v"]
    # derived defaults (options.h:257-262)
    d = Options(["-K", "64"])
    assert d.a == pytest.approx(1024 ** -0.5) and d.alpha == pytest.approx(1 / 64)
    assert parse_size_t("010") == 8 and parse_size_t("2g") == 2 << 30
    with pytest.raises(NumberFormatError):
        parse_size_t("12q")
    with pytest.raises(ValueError):
        Options(["--mcmc.strategy", "bogus"])
    with pytest.raises(ValueError):
        Options(["-K", "3", "-K", "4"])


def test_options_config_file(tmp_path):
    p = tmp_path / "c.ini"
    p.write_text("[mcmc]\nK = 48\nepsilon = 1e-6\n")
    o = Options(["--config", str(p), "--mcmc.K", "16"])
    assert o.K == 16 and o.epsilon == 1e-6  # command line wins


def test_generator_small_workload(native_lib):
    net, opts = workloads.build("small")
    assert net.N == 5000
    assert 13000 < net.num_total_edges < 16000  # ~14.5k edges
    rp, col = net.row_ptr, net.col
    src = np.repeat(np.arange(net.N), np.diff(rp))
    assert np.all(col != src)
    for v in range(0, net.N, 97):
        row = col[rp[v]:rp[v + 1]]
        assert np.all(np.diff(row) > 0)
    # symmetric
    fw = set(zip(src.tolist(), col.tolist()))
    assert all((b, a) in fw for a, b in list(fw)[:5000])
    # deterministic
    net2 = Network.synthetic(n=5000, k_true=50, size_min=10, size_max=500, intra_degree=4.0, seed=0)
    assert np.array_equal(net2.col, net.col)


def test_held_out_split(native_lib):
    net, opts = workloads.build("small")
    E = net.num_total_edges
    p = int(0.02 * E) // 2
    ha, hb, hy = net.held_out
    ta, tb, ty = net.test
    assert len(ha) == 2 * p and len(ta) == 2 * p and hy.sum() == p and ty.sum() == p
    und = {tuple(e) for e in net.undirected_edges().tolist()}
    hk = set(zip(ha.tolist(), hb.tolist()))
    tk = set(zip(ta.tolist(), tb.tolist()))
    assert not (hk & tk)
    assert np.all(ha < hb) and np.all(ta < tb)
    for a, b, y in zip(ha, hb, hy):
        assert ((a, b) in und) == bool(y)
    for a, b, y in zip(ta, tb, ty):
        assert ((a, b) in und) == bool(y)


def test_relativity_round_trip(tmp_path, native_lib):
    net = Network.synthetic(n=300, k_true=5, intra_degree=4.0, seed=1)
    f = tmp_path / "g.txt"
    net.write_relativity(str(f))
    lines = f.read_text().splitlines()
    assert all(l.startswith("#") for l in lines[:4]) and len(lines) == 4 + net.num_total_edges
    back = Network.from_relativity(str(f), contiguous=True)
    n_used = int(net.undirected_edges().max()) + 1
    assert back.N == n_used
    assert np.array_equal(back.row_ptr[:n_used + 1], net.row_ptr[:n_used + 1])
    assert np.array_equal(back.col, net.col)
    # non-contiguous ids are renumbered in ascending order
    g = tmp_path / "h.txt"
    g.write_text("# a\n# b\n# c\n# d\n10\t30\n30\t20\n20\t20\n10\t30\n")
    h = Network.from_relativity(str(g))
    assert h.N == 3 and h.num_total_edges == 2


def test_graph_from_edges_rejects_bad_ids(native_lib):
    with pytest.raises(_native.AmmsbError):
        Network.from_edges(10, [1, 2], [3, 12])


def test_create_without_gpu_fails_cleanly(native_lib):
    """Without a CUDA device, create reports a CUDA error (no fallback)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    from mcmc_for_ammsb_gb300 import MCMCSamplerStochastic
    net = Network.synthetic(n=300, k_true=5, intra_degree=4.0, seed=1)
    net.make_held_out(0.05)
    with pytest.raises(_native.AmmsbError) as e:
        MCMCSamplerStochastic(Options(K=8, num_node_sample=8), net).create()
    assert e.value.code == -2


def test_edge_loglik_has_no_cpu_path(native_lib):
    """The differentiable edge log-likelihood runs on the GPU only: CPU
    tensors are refused before any kernel is queued, and the C ABI checks its
    arguments before touching a device pointer."""
    torch = pytest.importorskip("torch")
    from mcmc_for_ammsb_gb300.autograd import edge_log_likelihood
    x = torch.full((2, 4), 0.25, dtype=torch.float64)
    th = torch.ones(4, 2, dtype=torch.float64)
    idx = torch.zeros(3, dtype=torch.int64)
    with pytest.raises(RuntimeError):
        edge_log_likelihood(x, x, th, idx, idx, idx.to(torch.uint8), 1e-7)
    L = native_lib
    assert L.ammsb_edge_loglik_workspace_size(_native.REAL_F64, 16, 50, 1600) >= 8 * (
        2 * 50 + 1600 + 50 * 16)
    p = ctypes.c_void_p(256)
    # unknown dtype, K out of range, stride below K: rejected without a GPU
    for args in ((7, 16, 16), (_native.REAL_F64, 0, 16), (_native.REAL_F64, 2000, 2000),
                 (_native.REAL_F64, 16, 8)):
        dt, K, ld = args
        assert L.ammsb_edge_loglik_forward(dt, K, p, ld, p, ld, 1, p, 1e-7, p, 1, p, p, 1, p, p,
                                           None) == -1


def _cli(args, **kw):
    import subprocess
    from mcmc_for_ammsb_gb300 import build
    exe = build.CLI
    return subprocess.run([exe] + list(args), capture_output=True, text=True, timeout=120, **kw)


def test_cli_options_and_errors(native_lib, tmp_path):
    """The C++ driver mirrors apps/main/main.cc: command-line echo, --help,
    exit status 33 for option and IO errors (main.cc:79-86)."""
    r = _cli(["--help"])
    assert r.returncode == 0 and r.stdout.startswith("Command line: ")
    for name in ("--mcmc.K [-K]", "--mcmc.mini-batch-size [-m]", "--mcmc.held-out-ratio [-h]",
                 "--mcmc.strategy", "--mcmc.input.file [-f]", "--config"):
        assert name in r.stdout
    r = _cli(["--mcmc.strategy", "bogus"])
    assert r.returncode == 33 and "Option error: Unknown strategy" in r.stderr
    r = _cli(["-K", "12q"])
    assert r.returncode == 33 and "Unknown characters in number" in r.stderr
    r = _cli(["-K", "16", "--mcmc.K", "32"])
    assert r.returncode == 33 and "more than once" in r.stderr
    r = _cli(["-f", str(tmp_path / "missing.txt")])
    assert r.returncode == 33 and "IO error" in r.stderr
    cfg = tmp_path / "run.cfg"
    cfg.write_text("[mcmc]\nK = 0x10\nbogus = 1\n")
    r = _cli(["--config", str(cfg), "-c", "synthetic", "-f", "n=200,k_true=4"])
    assert r.returncode == 33 and "unrecognised option 'mcmc.bogus'" in r.stderr


def test_cli_reads_relativity_and_needs_a_gpu(native_lib, tmp_path):
    """Without a GPU the driver gets as far as ammsb_create and reports the
    CUDA error (no CPU fallback)."""
    pytest.importorskip("torch")
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    net = Network.synthetic(n=300, k_true=6, size_min=10, size_max=100, intra_degree=4.0, seed=1)
    path = tmp_path / "g.txt"
    net.write_relativity(str(path))
    r = _cli(["-f", str(path), "--mcmc.input.contiguous", "-K", "8", "-x", "11"])
    assert r.returncode == 1, r.stderr
    assert "Set held_out_ratio to default 0.1" in r.stderr
    assert "start MCMC stochastical" in r.stdout and "MCMC error" in r.stderr
