"""Preprocessed networks (network.cc:88-145 save, :49-65 reload) and graphs
read from relativity text through the GPU path.

CPU: a saved network reads back equal (CSR, held-out and test sets, ratio);
damaged files are rejected.  GPU: the command-line driver saves a network
with --gb300.save-network and a second run with -c preprocessed -f DIR
prints the same perplexity lines; a graph read from relativity text
(preprocess/relativity.cc:20-200) samples bit for bit like the oracle and
takes a fed update within the parity tolerances.
"""
import os
import re
import subprocess

import numpy as np
import pytest

from mcmc_for_ammsb_gb300 import Network, _native, build


def _net(seed=2):
    net = Network.synthetic(n=700, k_true=10, size_min=10, size_max=150, intra_degree=5.0,
                            seed=seed)
    net.make_held_out(0.04, seed=seed)
    return net


def test_round_trip(native_lib, tmp_path):
    net = _net()
    d = tmp_path / "net"
    net.save_preprocessed(d)
    assert sorted(os.listdir(d)) == ["aux.bin", "graph.bin", "held-out.bin", "test.bin"]
    back = Network.load_preprocessed(d)
    assert back.N == net.N and back.held_out_ratio == 0.04
    assert np.array_equal(back.row_ptr, net.row_ptr) and np.array_equal(back.col, net.col)
    for x, y in zip(back.held_out + back.test, net.held_out + net.test):
        assert x.dtype == y.dtype and np.array_equal(x, y)
    # saving again into the same directory overwrites it
    net2 = _net(seed=3)
    net2.save_preprocessed(d)
    assert np.array_equal(Network.load_preprocessed(d).col, net2.col)


def _damage(path, fn):
    data = bytearray(open(path, "rb").read())
    open(path, "wb").write(bytes(fn(data)))


@pytest.mark.parametrize("what", ["truncated", "trailing", "tag", "asymmetric", "unsorted",
                                  "pair_range", "self_pair", "aux", "missing"])
def test_damaged_files_are_rejected(native_lib, tmp_path, what):
    net = _net()
    d = tmp_path / "net"
    net.save_preprocessed(d)
    g = str(d / "graph.bin")
    n = net.N
    col0 = 24 + 8 * (n + 1)  # byte offset of col[0]
    if what == "truncated":
        _damage(g, lambda b: b[:-3])
    elif what == "trailing":
        _damage(g, lambda b: b + b"\0")
    elif what == "tag":
        _damage(str(d / "test.bin"), lambda b: b"XXXXXXXX" + b[8:])
    elif what == "asymmetric":  # col[0] moved to another vertex: row 0 still sorted
        c = np.frombuffer(bytes(open(g, "rb").read()[col0:col0 + 8]), np.int32)
        new = int(c[0]) - 1 if int(c[0]) > 1 else None
        assert new is not None and new != 0 and (new < int(c[1]))
        _damage(g, lambda b: b[:col0] + np.int32(new).tobytes() + b[col0 + 4:])
    elif what == "unsorted":  # row 0's first two columns swapped
        _damage(g, lambda b: b[:col0] + b[col0 + 4:col0 + 8] + b[col0:col0 + 4] + b[col0 + 8:])
    elif what == "pair_range":  # held-out a[0] = N
        _damage(str(d / "held-out.bin"), lambda b: b[:24] + np.int32(n).tobytes() + b[28:])
    elif what == "self_pair":  # test b[0] = a[0]
        t = bytearray(open(str(d / "test.bin"), "rb").read())
        cnt = int(np.frombuffer(bytes(t[8:16]), np.int64)[0])
        a0 = bytes(t[16:20])
        _damage(str(d / "test.bin"), lambda b: b[:16 + 4 * cnt] + a0 + b[20 + 4 * cnt:])
    elif what == "aux":
        _damage(str(d / "aux.bin"), lambda b: b[:16] + np.int64(1).tobytes() + b[24:])
    elif what == "missing":
        os.remove(str(d / "aux.bin"))
    with pytest.raises(_native.AmmsbError) as e:
        Network.load_preprocessed(d)
    assert e.value.code == -1


LINE = re.compile(r"average_count is: (\d+) step count: (\d+) time: [0-9.]+ perplexity for hold "
                  r"out set: ([0-9.]+)")


def _need_gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")


@pytest.mark.gpu
def test_cli_saves_and_reruns_a_preprocessed_network(native_lib, tmp_path):
    _need_gpu()
    d = str(tmp_path / "pre")
    common = ["-K", "16", "-n", "16", "-i", "50", "-x", "151", "--mcmc.a", "0.01"]

    def run(args):
        r = subprocess.run([build.CLI] + args, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr
        return r, [(int(a), int(s), float(p)) for a, s, p in LINE.findall(r.stdout)]

    r1, first = run(["-c", "synthetic", "-f", "n=1500,k_true=20,seed=5", "--mcmc.held-out-ratio",
                     "0.05", "--gb300.save-network", d] + common)
    assert len(first) == 3
    r2, again = run(["-c", "preprocessed", "-f", d, "--mcmc.held-out-ratio", "0.05"] + common)
    assert again == first
    assert "WARNING" not in r2.stderr
    # the run() report closes both runs
    assert r1.stdout.count("  update_phi") == 1 and r2.stdout.count("  update_phi") == 1
    r = subprocess.run([build.CLI, "-c", "preprocessed", "-f", str(tmp_path / "none")] + common,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 33 and "IO error" in r.stderr


@pytest.mark.gpu
def test_relativity_graph_through_the_gpu_path(native_lib, tmp_path):
    """A graph written as relativity text with non-contiguous ids, read back
    (ids renumbered in ascending order), then sampled and updated on the GPU
    against the oracle."""
    _need_gpu()
    from test_gpu_parity import check_sampling, make_sampler, random_state, run_fed_case
    src = Network.synthetic(n=2000, k_true=25, intra_degree=5.0, seed=8)
    und = src.undirected_edges().astype(np.int64)
    ids = np.arange(src.N, dtype=np.int64) * 7 + 1000  # sparse, ascending external ids
    path = tmp_path / "g.txt"
    with open(path, "w") as f:
        f.write("# Undirected graph\n# test\n# Nodes Edges\n# FromNodeId\tToNodeId\n")
        for a, b in und:
            f.write("%d\t%d\n" % (ids[a], ids[b]))
    net = Network.from_relativity(str(path), contiguous=False)
    # text carries edges only: vertices without edges drop out, the rest
    # are numbered in ascending order of their ids
    used = np.unique(und)
    want = Network.from_edges(len(used), np.searchsorted(used, und[:, 0]),
                              np.searchsorted(used, und[:, 1]))
    assert net.N == len(used) <= src.N
    assert np.array_equal(net.row_ptr, want.row_ptr) and np.array_equal(net.col, want.col)
    net.make_held_out(0.02, seed=4)
    s, opts = make_sampler(net, _native.PI_F32, K=32)
    s.set_state(*random_state(net.N, 32))
    check_sampling(s, net, opts, steps=4)
    s.close()
    for dt in (_native.PI_F32, _native.PI_BF16):
        run_fed_case(net, 64, 9, dt)
