"""run()'s per-phase report and its convergence stop.

  * PrintStats (mcmc_sampler_stochastic.cc:185-198): every
    `mcmc.stats` iterations (cc:177-179) and once after the loop (cc:182),
    a table in the reference Timer's layout (timer.cc:18-53): outer,
    perplexity, sample_mini_batch, nodes_in_mini_batch (unused here: the
    minibatch kernel yields the nodes), sample_neighbor_nodes and
    update_phi (one tick per minibatch node, as the reference's per-node
    timers), update_pi (pi commit with the beta gradient, fused) and
    update_beta (the theta step); the device phases are CUDA-event times.
  * The convergence stop (learner.cc:130-136): run() ends once two
    consecutive held-out perplexities differ by at most
    mcmc.convergence relative.
"""
import re

import pytest

from mcmc_for_ammsb_gb300 import MCMCSamplerStochastic, Options

pytestmark = pytest.mark.gpu

NAMES = ["outer", "perplexity", "sample_mini_batch", "nodes_in_mini_batch",
         "sample_neighbor_nodes", "update_phi", "update_pi", "update_beta"]
ROW = re.compile(r"^  (\S+) +(\d+\.\d{3}) +(\d+) +(\d+\.\d{3})$")


def parse_tables(out):
    """The stats tables printed to stdout: a list of {timer: (total_s,
    ticks, per_tick_us) or None for <unused>}."""
    lines = out.splitlines()
    tables = []
    for q, line in enumerate(lines):
        if line.startswith("timer"):
            assert line == "%-37s%13s%9s%15s" % ("timer", "total (s)", "ticks", "per tick (us)")
            t = {}
            for row in lines[q + 1:q + 1 + len(NAMES)]:
                if row.endswith("<unused>"):
                    assert row == "%-36s<unused>" % ("  " + row.split()[0])
                    t[row.split()[0]] = None
                    continue
                m = ROW.match(row)
                assert m, row
                assert len(row) == 36 + 1 + 12 + 1 + 8 + 1 + 14
                t[m.group(1)] = (float(m.group(2)), int(m.group(3)), float(m.group(4)))
            assert list(t) == NAMES
            tables.append(t)
    return tables


@pytest.mark.parametrize("pipeline", [1, 0])
def test_run_prints_stats_every_interval_and_at_the_end(small_net, capfd, pipeline):
    net, _ = small_net
    o = Options(K=32, num_node_sample=32, max_iteration=251, interval=100, stats_print_interval=100,
                held_out_ratio=0.02, pipeline=pipeline)
    s = MCMCSamplerStochastic(o, net).create()
    s.init()
    s.run()
    out = capfd.readouterr().out
    tables = parse_tables(out)
    # at step_count 100 and 200 (cc:177) and after the loop (cc:182)
    assert len(tables) == 3
    n_out = s.num_node_sample + 1
    evals = s.counters()[0]
    for t, iters, ppx_calls in zip(tables, (99, 199, 250), (1, 2, 3)):
        assert t["nodes_in_mini_batch"] is None
        assert t["outer"][1] == iters
        assert t["perplexity"][1] == ppx_calls
        for name in ("sample_mini_batch", "update_pi", "update_beta"):
            assert t[name][1] == iters, name
        assert t["sample_neighbor_nodes"][1] == t["update_phi"][1]
        for name in NAMES:
            if t[name] is not None:
                total, ticks, per = t[name]
                assert total >= 0 and per > 0
                assert per == pytest.approx(total * 1e6 / ticks, rel=0.01, abs=2e3 / ticks + 1e-3)
        # the device phases fit inside the wall time of the iterations
        dev = sum(t[k][0] for k in ("update_phi", "update_pi", "update_beta"))
        assert dev <= t["outer"][0] + 1e-3
    # node ticks: every minibatch node of every updated iteration
    assert tables[-1]["update_phi"][1] == evals // n_out
    assert s.step_count == 251
    s.close()


def test_convergence_stops_run(small_net, capfd):
    """A threshold every pair of perplexities meets: run() stops after the
    second perplexity point (steps 1 and 101), before the next update
    batch reaches the third."""
    net, _ = small_net
    o = Options(K=32, num_node_sample=32, max_iteration=2001, interval=100, held_out_ratio=0.02,
                convergence_threshold=10.0)
    s = MCMCSamplerStochastic(o, net).create()
    s.init()
    s.run()
    out = capfd.readouterr().out
    lines = [l for l in out.splitlines() if l.startswith("average_count is:")]
    assert len(lines) == 2
    assert " step count: 1 " in lines[0] and " step count: 101 " in lines[1]
    assert s.step_count == 201
    assert len(parse_tables(out)) == 1  # the closing report only
    s.close()

    # a threshold no pair meets: the loop runs to max_iteration
    o = Options(K=32, num_node_sample=32, max_iteration=501, interval=100, held_out_ratio=0.02,
                convergence_threshold=0.0)
    s = MCMCSamplerStochastic(o, net).create()
    s.init()
    s.run()
    out = capfd.readouterr().out
    assert len([l for l in out.splitlines() if l.startswith("average_count is:")]) == 5
    assert s.step_count == 501
    s.close()


@pytest.mark.parametrize("K,dtype", [(32, 0), (1024, 1)], ids=["k32-f32", "k1024-bf16"])
def test_launch_modes_give_the_same_chain(small_net, monkeypatch, K, dtype):
    """The draws depend only on (seed, chain, step), so the chain is the same
    bit for bit whether the iterations run as CUDA graphs or launched one by
    one, with the draws made ahead on a second stream or in the loop's order
    on one stream, and with or without the early (programmatic dependent)
    starts of update_phi, the commit and the theta step (AMMSB_PDL, read at
    create: 0 none, 7 all three; the default starts update_phi and theta
    early).  K = 1024 runs the ring kernels and their 16-warp variant."""
    import numpy as np
    net, _ = small_net
    out = {}
    for pdl in (None, "0", "7"):
        for graph in (1, 0):
            for pipeline in (1, 0):
                if pdl is None:
                    monkeypatch.delenv("AMMSB_PDL", raising=False)
                else:
                    monkeypatch.setenv("AMMSB_PDL", pdl)
                o = Options(K=K, num_node_sample=32, held_out_ratio=0.02, use_graph=graph,
                            pipeline=pipeline, pi_dtype=dtype)
                s = MCMCSamplerStochastic(o, net).create()
                s.init()
                s.step(37)
                p1 = s.cal_perplexity_held_out()
                s.step(20)
                out[pdl, graph, pipeline] = (s.phi, s.pi, s.theta, p1, s.step_count)
                s.close()
    ref = out[None, 1, 1]
    for key, got in out.items():
        for a, b in zip(got, ref):
            assert np.array_equal(a, b), key
