"""Checkpoint / resume and the command-line driver on the GPU.

Every draw is a function of (seed, chain, step), so a chain restored from a
checkpoint must continue bit for bit: after the same number of further
iterations, phi, the stored pi, theta, beta, the held-out running averages
and the perplexity equal those of the chain that never stopped.  The C++
driver (csrc/ammsb_main.cpp, the sequential branch of apps/main/main.cc)
must print the same perplexity lines as the Python front end on the same
graph, options and held-out set, and resume a saved chain the same way.
"""
import re
import subprocess

import numpy as np
import pytest

from mcmc_for_ammsb_gb300 import MCMCSamplerStochastic, Network, Options, _native, build, workloads

pytestmark = pytest.mark.gpu


def _need_gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")


def _state(s):
    return dict(phi=s.phi, pi=s.pi, theta=s.theta, beta=s.beta, ppx=s.ppx_per_heldout_edge)


@pytest.mark.parametrize("dtype", [_native.PI_F32, _native.PI_BF16])
def test_resume_continues_bit_for_bit(native_lib, tmp_path, dtype):
    _need_gpu()
    net, opts = workloads.build("small")
    o = dict(K=32, num_node_sample=32, pi_dtype=dtype, interval=50)
    a = MCMCSamplerStochastic(Options(**o), net).init()
    a.step(120)
    a.cal_perplexity_held_out()
    a.step(30)
    ck = tmp_path / "chain.ck"
    a.save_checkpoint(ck)
    a.step(100)
    want_ppx = a.cal_perplexity_held_out()
    want = _state(a)
    step_a = a.step_count

    b = MCMCSamplerStochastic(Options(**o), net).load_checkpoint(ck)
    b.step(100)
    got_ppx = b.cal_perplexity_held_out()
    got = _state(b)
    assert b.step_count == step_a
    assert got_ppx == want_ppx
    for k in want:
        assert np.array_equal(got[k], want[k]), k
    a.close()
    b.close()


def test_checkpoint_rejects_another_chain(native_lib, tmp_path):
    _need_gpu()
    net, opts = workloads.build("small")
    a = MCMCSamplerStochastic(Options(K=32, num_node_sample=32), net).init()
    a.step(5)
    ck = tmp_path / "c.ck"
    a.save_checkpoint(ck)
    for other in (dict(K=16, num_node_sample=32), dict(K=32, num_node_sample=32, chain=3),
                  dict(K=32, num_node_sample=32, pi_dtype=_native.PI_BF16)):
        b = MCMCSamplerStochastic(Options(**other), net)
        with pytest.raises(_native.AmmsbError) as e:
            b.load_checkpoint(ck)
        assert e.value.code == -1
        b.close()
    bad = tmp_path / "bad.ck"
    bad.write_bytes(b"not a checkpoint")
    b = MCMCSamplerStochastic(Options(K=32, num_node_sample=32), net)
    with pytest.raises(_native.AmmsbError):
        b.load_checkpoint(bad)
    trunc = tmp_path / "trunc.ck"
    trunc.write_bytes(ck.read_bytes()[:4096])
    with pytest.raises(_native.AmmsbError):
        b.load_checkpoint(trunc)
    b.close()
    a.close()


LINE = re.compile(r"average_count is: (\d+) step count: (\d+) time: [0-9.]+ perplexity for hold "
                  r"out set: ([0-9.]+)")


def _cli(args):
    r = subprocess.run([build.CLI] + args, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return [(int(a), int(s), float(p)) for a, s, p in LINE.findall(r.stdout)]


def test_cli_matches_python_front_end_and_resumes(native_lib, tmp_path, capfd):
    _need_gpu()
    gen = dict(n=5000, k_true=50, size_min=10, size_max=500, intra_degree=4.0, seed=0)
    spec = ",".join("%s=%s" % kv for kv in gen.items())
    base = ["-c", "synthetic", "-f", spec, "-K", "32", "-n", "32", "--mcmc.held-out-ratio",
            "0.02", "-i", "100", "--mcmc.a", "0.01", "--mcmc.b", "1024", "--mcmc.c", "0.55"]
    full = _cli(base + ["-x", "301"])
    assert [(a, s) for a, s, _ in full] == [(2, 1), (3, 101), (4, 201)]

    # the Python front end on the same graph, held-out set (seed 42) and options
    net = Network.synthetic(**gen)
    net.make_held_out(0.02, seed=42)
    py = MCMCSamplerStochastic(Options(["-K", "32", "-n", "32", "--mcmc.held-out-ratio", "0.02",
                                        "-i", "100", "--mcmc.a", "0.01", "--mcmc.b", "1024",
                                        "--mcmc.c", "0.55", "-x", "301"]), net)
    capfd.readouterr()
    py.run()
    lines = [(int(a), int(s), float(p)) for a, s, p in LINE.findall(capfd.readouterr().out)]
    assert lines == full
    py.close()

    ck = str(tmp_path / "cli.ck")
    first = _cli(base + ["-x", "101", "--gb300.save", ck])
    rest = _cli(base + ["-x", "301", "--gb300.resume", ck])
    assert first + rest == full
