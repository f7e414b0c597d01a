"""Benchmark of the GB300 SG-MCMC sampler: sampled edge evaluations per
second of the a-MMSB stochastic-gradient iteration.

One "step" is one SG-MCMC iteration on the large synthetic workload
(N=4,000,000 nodes, ~43M edges, K=1024, num-node-sample 128, minibatch
4,096, BF16 pi with FP32 phi master): stratified minibatch + neighbour
sampling, update_phi, pi, update_beta/theta, all resident in HBM.

  python bench.py [--steps K] [--warmup W] [--workload large|mid|small]
                  [--pi-dtype bf16|f32] [--impl ours|reference]

Prints one JSON line.  `value` is device-timed (CUDA events on the
sampler's stream around K captured-graph iterations); `e2e` times the
public run() loop (perplexity every `interval` iterations, host reads)
with the host clock; `roofline` is the update_phi kernel's algorithmic
bytes over its per-launch CUDA-event duration; `cpu_baseline` is the
oracle's restatement of the reference sampler timed on a bounded sample of
the same workload on this host.  --impl reference times that CPU
implementation alone (all host threads) and prints the reference line.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SG-MCMC edge-evals/s & time-to-perplexity, BF16-pi vs FP32 plain, 1 GB300"
UNIT = "edge-evals/s"
PEAKS_FALLBACK = {"hbm_gbs": 6800.0}


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return PEAKS_FALLBACK, "fallback"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None
        self.skip = 0

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        # nvidia-smi takes a moment to start: wait (at most 10 s) for its
        # first sample so that the timed region is covered from its start
        t0 = time.time()
        while time.time() - t0 < 10.0 and self.proc.poll() is None:
            if self._lines():
                break
            time.sleep(0.02)
        self.skip = len(self._lines())

    def _lines(self):
        with open(self.path) as f:
            return [ln for ln in f.read().splitlines() if ln.count(",") >= 8]

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self._lines()
        if len(lines) > self.skip:  # samples taken after the timed region began
            lines = lines[self.skip:]
        for line in lines:
            parts = [x.strip() for x in line.split(",")]
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def reduce_over_ranks(secs, evals, world):
    """Whole-job timing over N replicas: the slowest rank's seconds (max) and
    the evaluations of all ranks (sum)."""
    if world <= 1:
        return secs, evals
    import torch
    import torch.distributed as dist
    t = torch.tensor([secs], dtype=torch.float64)
    e = torch.tensor([evals], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(e, op=dist.ReduceOp.SUM)
    return float(t[0]), float(e[0])


def phi_bytes_per_eval(K, pi_bytes, n_out):
    """Algorithmic bytes of update_phi per sampled edge evaluation: the
    neighbour pi row (K * s_pi) and id (4), plus the node's own traffic
    (pi_i read, pi_i write, phi read + write: K * (2 s_pi + 8)) shared by
    its n_out evaluations."""
    return K * pi_bytes + 4 + K * (2 * pi_bytes + 8) / n_out


# ---------------------------------------------------------------------------
# CPU side: the oracle's restatement of the reference sampler
# ---------------------------------------------------------------------------
def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    return oracle


def cpu_workload(name, strategy=0):
    """The workload's graph and held-out / test sets built by the oracle's own
    restatement of the generator and the split (equal to the product's,
    tests/test_oracle_graph.py), so that the CPU arm loads no product
    library; returns (network, Options)."""
    from mcmc_for_ammsb_gb300.options import Options
    from mcmc_for_ammsb_gb300.workloads import WORKLOADS
    w = WORKLOADS[name]
    net = _oracle().SyntheticNetwork.synthetic(**w["gen"])
    opts = Options(**dict(w["opts"], strategy=strategy))
    net.make_held_out(opts.held_out_ratio, seed=w["gen"]["seed"])
    return net, opts


def cpu_sampler(net, opts, fill_threads):
    """The oracle's whole-iteration sampler (float arithmetic in the
    reference's order) over the workload's full N x K state: phi ~ Gamma(1,
    1), pi its row normalisation, theta ~ Gamma(1, 1)."""
    oracle = _oracle()
    o = oracle.OracleSampler(net, opts.K, strategy=opts.strategy,
                             mini_batch_size=opts.mini_batch_size or None,
                             num_node_sample=opts.num_node_sample or None, alpha=opts.alpha,
                             epsilon=opts.epsilon, eta0=opts.eta0, eta1=opts.eta1, a=opts.a,
                             b=opts.b, c=opts.c, seed=42)
    o.init_state_threads(3, fill_threads)
    # minibatch edge capacity of the strategy (network.cc:188-201)
    me = max(o.p.mini_batch_size, net.max_degree())
    if o.p.max_source > 1:
        me = o.p.mini_batch_size + net.max_degree()
    if opts.strategy == 3:
        me = max(me, net.num_total_edges)
    o.max_edges = me
    return o


def cpu_time(o, threads, max_iters, seconds=None, warmup=0):
    """Times whole iterations -- minibatch (network.cc:274-421), neighbour
    sets (mcmc_sampler_stochastic.h:87-108), update_phi (cc:269-313), pi
    (cc:162-166), update_beta/theta (cc:200-267) -- of the oracle sampler
    on `threads` host threads, after `warmup` untimed ones; stops after
    max_iters iterations or, if given, once `seconds` have passed.  Returns
    (edge evaluations, seconds, iterations, nodes, non-link iterations)."""
    n_out = o.p.num_node_sample + 1
    for _ in range(warmup):
        o.step_threads(threads, o.max_edges)
    evals = nodes = iters = nonlink = 0
    t0 = time.perf_counter()
    while iters < max_iters:
        info = o.step_threads(threads, o.max_edges)
        evals += info.n_nodes * n_out
        nodes += info.n_nodes
        nonlink += info.flag == 0
        iters += 1
        if seconds is not None and time.perf_counter() - t0 >= seconds:
            break
    return evals, time.perf_counter() - t0, iters, nodes, nonlink


def reference_arm(args):
    """The reference's CPU sampler on this workload: the oracle's
    whole-iteration restatement (the compiled reference needs its sources,
    which only the build container holds) on all host threads, the
    per-node work spread as the reference's distributed sampler spreads it
    (distr.cc:1142).  At most 200 iterations are timed so that the run ends
    in minutes; a 1-thread figure (the reference's sequential build) is
    taken on the same state."""
    threads = os.cpu_count() or 1
    from mcmc_for_ammsb_gb300.options import STRATEGIES
    net, opts = cpu_workload(args.workload, STRATEGIES[args.strategy])
    o = cpu_sampler(net, opts, threads)
    timed = min(args.steps, 200)
    ev, secs, iters, nodes, nonlink = cpu_time(o, threads, timed, warmup=min(args.warmup, 5))
    value = ev / secs
    ev1, secs1, iters1, _, nl1 = cpu_time(o, 1, 1000, seconds=args.cpu_seconds)
    sample = ("oracle restatement of the reference's whole iteration (minibatch, neighbour sets, "
              "update_phi, pi, update_beta/theta; FP32, reference operation order) on the full "
              "%d x %d state of the %s workload: %d iterations timed (%d non-link), %d nodes, %d "
              "edge evaluations, %d host threads (update_phi over nodes); graph and held-out set "
              "from the oracle's generator" % (net.N, opts.K, args.workload, iters, nonlink, nodes,
                                               ev, threads))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * secs / max(iters, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (planted-community generator, seed 0)",
        "config": workload_config(args.workload, net.N, net.num_total_edges, opts,
                                  int(net.held_out[0].shape[0])),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "single_thread": {"value": ev1 / secs1, "unit": UNIT, "cores": 1, "iterations": iters1,
                          "nonlink_iterations": nl1, "seconds": secs1},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def workload_config(workload, N, E, opts, held_out):
    """The workload's identity, the same in both arms (the arithmetic type
    is the line's `dtype`)."""
    return {"workload": workload, "N": N, "E": E, "K": opts.K,
            "num_node_sample": opts.num_node_sample, "mini_batch_size": opts.mini_batch_size,
            "strategy": opts.strategy, "held_out": held_out,
            "l2": "inputs larger than L2 (pi %d x %d)" % (N, opts.K)}


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def ours_arm(args, net, opts, rank, world, local):
    import torch
    from mcmc_for_ammsb_gb300 import MCMCSamplerStochastic, _native

    torch.cuda.set_device(local)
    opts.device = local
    opts.chain = rank  # independent replicas (the path does not shard)
    opts.pi_dtype = _native.PI_BF16 if args.pi_dtype == "bf16" else _native.PI_F32
    s = MCMCSamplerStochastic(opts, net).create()
    s.init()
    stream = torch.cuda.ExternalStream(s.stream())
    K = s.K
    n_out = s.num_node_sample + 1
    pi_bytes = 2 if args.pi_dtype == "bf16" else 4

    s.step(args.warmup)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    # kernels per iteration: minibatch, neighbour sets, update_phi (the ring
    # kernel launches its many-node and few-node variants), commit/beta, theta
    launches_per_iter = 6 if s.kernel_config()["ring"] else 5
    e0, i0 = s.counters()
    clocks = ClockSampler(local)
    clocks.start()
    ev_start = torch.cuda.Event(enable_timing=True)
    ev_stop = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev_start.record(stream)
    s.step(args.steps)
    ev_stop.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = ev_start.elapsed_time(ev_stop)
    e1, i1 = s.counters()
    evals = e1 - e0
    secs, total_evals = reduce_over_ranks(ms / 1000.0, float(evals), world)
    value = total_evals / secs

    # per-phase CUDA-event durations of the same iteration (not captured),
    # for the roofline of the dominant kernel
    phase = {k: [] for k in ("sample_mini_batch", "sample_neighbor_nodes", "update_phi",
                             "update_pi+beta_grads", "update_theta")}
    phi_bytes, phi_ms = 0.0, 0.0
    nl_bytes, nl_ms, nl_n = 0.0, 0.0, 0
    m_nodes = (s.resolved.mini_batch_size + 1) * n_out
    for _ in range(args.profile_steps):
        ea, _ = s.counters()
        p = s.profile_step()
        eb, _ = s.counters()
        for k, v in p.items():
            phase[k].append(v)
        by = (eb - ea) * phi_bytes_per_eval(K, pi_bytes, n_out)
        phi_bytes += by
        phi_ms += p["update_phi"]
        if eb - ea == m_nodes:  # a non-link stratum launch (m + 1 nodes)
            nl_bytes += by
            nl_ms += p["update_phi"]
            nl_n += 1
    peaks, peak_src = load_peaks()
    achieved = phi_bytes / (phi_ms / 1000.0) / 1e9 if phi_ms > 0 else 0.0
    # DRAM bytes per launch: the ncu-measured bytes per edge evaluation of
    # the update_phi kernel (same K, n_out and pi type) times this run's
    # mean evaluations per launch
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "update_phi_traffic.json")
    if os.path.exists(tpath) and args.profile_steps > 0:
        with open(tpath) as f:
            tr = json.load(f)
        if (tr.get("K") == K and tr.get("n_out") == n_out and tr.get("pi_dtype") == args.pi_dtype
                and tr.get("bytes_per_eval")):
            traffic = tr["bytes_per_eval"] * (phi_bytes / phi_bytes_per_eval(K, pi_bytes, n_out)) \
                / args.profile_steps

    # e2e: the public run() loop (perplexity every interval, host reads)
    e2e = None
    if rank == 0 and not args.no_e2e:
        interval = opts.interval or 50
        n_e2e = max(args.steps, args.e2e_steps)
        s.step(1)  # resumes the draws ahead after the profiled iterations
        torch.cuda.synchronize()
        ea, _ = s.counters()
        t0 = time.perf_counter()
        n_ppx = 0
        done = 0
        while done < n_e2e:
            if done % interval == 0:
                s.cal_perplexity_held_out()  # D2H of the perplexity, synchronises
                n_ppx += 1
            n = min(interval - done % interval, n_e2e - done)
            s.step(n)
            done += n
        s.beta  # the iteration's global parameters read back (D2H, synchronises)
        t1 = time.perf_counter()
        eb, _ = s.counters()
        e2e = {"value": (eb - ea) / (t1 - t0), "unit": UNIT, "h2d_bytes_per_step": 0,
               "d2h_bytes_per_step": (8 * n_ppx + 4 * K) / n_e2e, "iterations": n_e2e,
               "note": "public API loop (what run() does): step() with held-out perplexity "
                       "every %d iterations (its D2H read), beta read back at the end, host "
                       "clock, %d iterations; minibatch and neighbour draws are generated on "
                       "the device, so an iteration has no host input to copy"
                       % (interval, n_e2e)}

    s.close()
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        o = cpu_sampler(net, opts, os.cpu_count() or 1)
        ev, secs_cpu, it_cpu, nodes_cpu, nl_cpu = cpu_time(o, 1, 1000, seconds=args.cpu_seconds,
                                                           warmup=1)
        del o
        cpu = {"value": ev / secs_cpu, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": "oracle restatement of the reference's whole iteration (minibatch, "
                         "neighbour sets, update_phi, pi, update_beta/theta; FP32, reference "
                         "operation order) on the full %d x %d state of this workload: %d "
                         "iterations (%d non-link), %d nodes, %.1f s on 1 host core"
                         % (net.N, K, it_cpu, nl_cpu, nodes_cpu, secs_cpu)}

    ttp = vs_fp64 = None
    if rank == 0 and world == 1 and args.ttp_iters_line > 0:
        ttp = ttp_summary(net, opts, args.ttp_iters_line, args.ttp_interval_line)
    if rank == 0 and world == 1 and not args.no_fp64:
        vs_fp64 = fp64_summary()

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * secs / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16-pi/f32" if args.pi_dtype == "bf16" else "f32",
            "data": "synthetic (planted-community generator, seed 0)",
            "config": workload_config(args.workload, net.N, net.num_total_edges, opts,
                                      int(net.held_out[0].shape[0])),
            "parallelism": "replicas" if world > 1 else "single",
            "iterations_per_s": (i1 - i0) / secs if world == 1 else None,
            "gpu_launches": launches_per_iter * args.steps,
            "roofline": {"bound": "hbm", "achieved": achieved,
                         "peak": peaks.get("hbm_gbs", PEAKS_FALLBACK["hbm_gbs"]),
                         "unit": "GB/s", "frac": achieved / peaks.get("hbm_gbs", 6800.0),
                         "traffic": traffic, "kernel": "k_update_phi",
                         "peak_source": peak_src,
                         "launches": args.profile_steps,
                         "nonlink_launches": nl_n,
                         "nonlink_achieved": (nl_bytes / (nl_ms / 1000.0) / 1e9) if nl_ms else None,
                         "nonlink_ms": (nl_ms / nl_n) if nl_n else None},
            "phase_ms_mean": {k: statistics.mean(v) for k, v in phase.items() if v},
            "clocks": clk,
            "e2e": e2e,
            "cpu_baseline": cpu,
            "ttp": ttp,
            "vs_fp64": vs_fp64,
        }
        print(json.dumps(line))


# ---------------------------------------------------------------------------
# time to perplexity
# ---------------------------------------------------------------------------
def _gpu_curve(net, opts_kw, pi_dtype, use_graph, iters, interval, pipeline=1):
    """Held-out perplexity every `interval` iterations (before the update,
    as run() does) against wall time from the start of the loop; state
    initialisation is outside the clock, as it is outside the reference's
    run() timer."""
    import torch
    from mcmc_for_ammsb_gb300 import MCMCSamplerStochastic, Options, _native
    o = Options(**dict(opts_kw, pi_dtype=pi_dtype, use_graph=use_graph, pipeline=pipeline))
    s = MCMCSamplerStochastic(o, net).init()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    curve = []
    done = 0
    while True:
        p = s.cal_perplexity_held_out()
        curve.append((done, time.perf_counter() - t0, p))
        if done >= iters:
            break
        n = min(interval, iters - done)
        s.step(n)
        done += n
    s.close()
    return curve


def _cpu_curve(net, opts_kw, iters, interval):
    """The oracle's whole-iteration restatement (FP32, reference operation
    order, one host core) on the same workload, same clock convention."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    K = opts_kw["K"]
    o = oracle.OracleSampler(net, K, strategy=opts_kw.get("strategy", 0),
                             mini_batch_size=opts_kw.get("mini_batch_size") or None,
                             num_node_sample=opts_kw.get("num_node_sample") or None,
                             alpha=opts_kw.get("alpha", 0.0), epsilon=opts_kw.get("epsilon", 1e-7),
                             a=opts_kw.get("a", 0.0), b=opts_kw.get("b", 1024.0),
                             c=opts_kw.get("c", 0.5))
    rng = np.random.default_rng(0)
    o.set_state(rng.gamma(1.0, 1.0, (net.N, K)).astype(np.float32),
                rng.gamma(1.0, 1.0, (K, 2)).astype(np.float32))
    t0 = time.perf_counter()
    curve = []
    done = 0
    while True:
        p = o.perplexity("f32")
        curve.append((done, time.perf_counter() - t0, p))
        if done >= iters:
            break
        for _ in range(min(interval, iters - done)):
            o.step()
        done += min(interval, iters - done)
    return curve


def _f64_compare(net, kw, iters, interval):
    """Perplexity of the FP32 and BF16 device paths against the oracle's FP64
    restatement of the same iterations (identical draws: the sampling is
    bit-exact and the noise is the same Philox normals), from one seeded
    state, every `interval` iterations up to `iters`.  Returns per path the
    largest relative perplexity error and the curves."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from mcmc_for_ammsb_gb300 import MCMCSamplerStochastic, Options, _native
    K = kw["K"]
    rng = np.random.default_rng(0)
    phi = rng.gamma(1.0, 1.0, (net.N, K)).astype(np.float32)
    theta = rng.gamma(1.0, 1.0, (K, 2))
    ref = oracle.OracleSampler64(net, K, strategy=kw.get("strategy", 0),
                                 mini_batch_size=kw.get("mini_batch_size") or None,
                                 num_node_sample=kw.get("num_node_sample") or None,
                                 alpha=kw.get("alpha", 0.0), epsilon=kw.get("epsilon", 1e-7),
                                 eta0=kw.get("eta0", 1.0), eta1=kw.get("eta1", 1.0),
                                 a=kw.get("a", 0.0), b=kw.get("b", 1024.0), c=kw.get("c", 0.5))
    ref.set_state(phi, theta)
    want = []
    for it in range(iters + 1):
        if it % interval == 0:
            want.append(ref.perplexity())
        if it < iters:
            ref.step()
    out = {}
    for name, dt in (("f32", _native.PI_F32), ("bf16", _native.PI_BF16)):
        s = MCMCSamplerStochastic(Options(**dict(kw, pi_dtype=dt)), net).set_state(phi, theta)
        got = []
        for it in range(0, iters + 1, interval):
            got.append(s.cal_perplexity_held_out())
            if it < iters:
                s.step(interval)
        s.close()
        rel = [abs(g - w) / abs(w) for g, w in zip(got, want)]
        out[name] = {"max_rel_err": max(rel), "final_rel_err": rel[-1], "perplexity": got}
    out["f64_oracle"] = {"perplexity": want}
    return out


def _grad_vs_fp64():
    """Error of the FP32 adjoint kernels against the FP64 oracle on the
    differentiation workload (N=2,000, K=16, phi and theta iid Gamma(100,
    0.01), 50 nodes x 32 sampled neighbours): the gradient in phi against the
    oracle's restatement of update_phi's hand-derived gradient
    (mcmc_sampler_stochastic.cc:274-296), in theta against update_beta's
    (cc:212-240); largest absolute error over the largest gradient."""
    import numpy as np
    import torch
    oracle = _oracle()
    from mcmc_for_ammsb_gb300 import workloads
    from mcmc_for_ammsb_gb300.autograd import edge_log_likelihood
    net, _ = workloads.build("diff")
    K, n_nodes, n_out, eps = 16, 50, 32, 1e-7
    rng = np.random.default_rng(11)
    phi = rng.gamma(100.0, 0.01, (net.N, K))
    theta = rng.gamma(100.0, 0.01, (K, 2))
    og = oracle.OracleGraph(net)
    nodes = rng.choice(net.N, n_nodes, replace=False).astype(np.int32)
    drawn = [oracle.sample_neighbors(og, int(v), n_out, 42, 0, 1) for v in nodes]
    nbrs = np.stack([d[0] for d in drawn])
    ys = np.stack([d[1] for d in drawn])
    pi = phi / phi.sum(1, keepdims=True)
    beta = theta[:, 1] / theta.sum(1)
    want_phi = np.stack([oracle.phi_grad(K, pi, phi[v], int(v), nbrs[r], ys[r], beta, eps)
                         for r, v in enumerate(nodes)])
    ea = np.repeat(nodes, n_out).astype(np.int32)
    _, _, want_th = oracle.update_beta(K, pi, ea, nbrs.ravel().astype(np.int32), ys.ravel(),
                                       theta, beta, np.array([1.0, 1.0]), eps, 0.01, 1.0,
                                       np.zeros((K, 2)), dtype=np.float64)
    uniq, inv = np.unique(nbrs.ravel(), return_inverse=True)
    dev = "cuda"
    ps = torch.tensor(phi[nodes], dtype=torch.float32, device=dev, requires_grad=True)
    pn = torch.tensor(pi[uniq], dtype=torch.float32, device=dev)
    th = torch.tensor(theta, dtype=torch.float32, device=dev, requires_grad=True)
    src = torch.arange(n_nodes, device=dev).repeat_interleave(n_out)
    L = edge_log_likelihood(ps, pn, th, src, torch.tensor(inv.reshape(-1), device=dev),
                            torch.tensor(ys.ravel(), dtype=torch.uint8, device=dev), eps)
    gphi, gth = (t.double().cpu().numpy() for t in torch.autograd.grad(L, (ps, th)))
    return {"workload": "diff (N=2,000, K=16, 50 nodes x 32 neighbours)", "dtype": "f32",
            "phi_grad_err": float(np.abs(gphi - want_phi).max() / np.abs(want_phi).max()),
            "theta_grad_err": float(np.abs(gth - want_th).max() / np.abs(want_th).max())}


def fp64_summary():
    """Errors against the FP64 oracle, stated with every run: held-out
    perplexity of the FP32 and BF16 device paths over 500 iterations of the
    small workload (same draws; oracle_step_f64), and the FP32 adjoint's
    gradient."""
    from mcmc_for_ammsb_gb300 import workloads
    net, opts = workloads.build("small")
    kw = dict(K=32, num_node_sample=32, a=0.01, b=1024.0, c=0.55)
    f = _f64_compare(net, kw, 500, 50)
    return {"perplexity": {"workload": "small (N=5,000, K=32), 500 iterations, every 50",
                           "f32_max_rel_err": f["f32"]["max_rel_err"],
                           "bf16_max_rel_err": f["bf16"]["max_rel_err"]},
            "gradient": _grad_vs_fp64()}


def ttp_summary(net, opts, iters, interval):
    """Time to held-out perplexity within 1% of the FP32 plain GPU path's
    final value (`iters` iterations, perplexity every `interval`), from the
    same initial state, for
      f32_plain   FP32 pi, the kernels launched one by one in run()'s loop
                  order on one stream (draws, then update);
      f32_graph   FP32 pi with the BF16 sampler's launch design: the
                  iteration captured in CUDA graphs, the next iterations'
                  draws on a second stream during the update;
      bf16_graph  the BF16-pi graph-captured sampler.
    `speedup` is f32_plain / bf16_graph; `speedup_vs_f32_graph` isolates the
    BF16 rows (same launch design on both sides)."""
    from mcmc_for_ammsb_gb300 import _native
    keys = ("K", "alpha", "eta0", "eta1", "epsilon", "a", "b", "c", "mini_batch_size",
            "num_node_sample", "strategy", "held_out_ratio")
    kw = {k: getattr(opts, k) for k in keys}
    runs = {"f32_plain": _gpu_curve(net, kw, _native.PI_F32, 0, iters, interval, pipeline=0),
            "f32_graph": _gpu_curve(net, kw, _native.PI_F32, 1, iters, interval),
            "bf16_graph": _gpu_curve(net, kw, _native.PI_BF16, 1, iters, interval)}
    target = 1.01 * runs["f32_plain"][-1][2]
    out = {"target": target, "iterations": iters, "interval": interval}
    for name, c in runs.items():
        t, it = _time_to(c, target)
        out[name] = {"time_to_target_s": t, "iterations_to_target": it,
                     "final_perplexity": c[-1][2], "wall_s": c[-1][1],
                     "ms_per_iteration": 1000.0 * c[-1][1] / iters}
    tb = out["bf16_graph"]["time_to_target_s"]
    for base, key in (("f32_plain", "speedup"), ("f32_graph", "speedup_vs_f32_graph")):
        tp = out[base]["time_to_target_s"]
        out[key] = tp / tb if tp and tb else None
    out["final_rel_diff"] = abs(runs["bf16_graph"][-1][2] / runs["f32_plain"][-1][2] - 1.0)
    return out


def _time_to(curve, target):
    for it, t, p in curve:
        if p <= target:
            return t, it
    return None, None


def ttp_arm(args):
    """Time to held-out perplexity within 1% of the FP32 plain GPU path's
    final value, with full curves (see ttp_summary for the three runs)."""
    from mcmc_for_ammsb_gb300 import _native, workloads
    net, opts = workloads.build(args.workload)
    keys = ("K", "alpha", "eta0", "eta1", "epsilon", "a", "b", "c", "mini_batch_size",
            "num_node_sample", "strategy", "held_out_ratio")
    kw = {k: getattr(opts, k) for k in keys}
    iters = args.ttp_iters
    interval = args.ttp_interval
    runs = {
        "f32_plain": _gpu_curve(net, kw, _native.PI_F32, 0, iters, interval, pipeline=0),
        "f32_graph": _gpu_curve(net, kw, _native.PI_F32, 1, iters, interval),
        "bf16_graph": _gpu_curve(net, kw, _native.PI_BF16, 1, iters, interval),
    }
    if args.ttp_cpu_iters:
        runs["cpu_oracle_f32"] = _cpu_curve(net, kw, args.ttp_cpu_iters, interval)
    f64 = _f64_compare(net, kw, args.ttp_f64_iters, args.ttp_f64_interval) \
        if args.ttp_f64_iters else None
    final = runs["f32_plain"][-1][2]
    target = 1.01 * final
    out = {}
    for name, c in runs.items():
        t, it = _time_to(c, target)
        out[name] = {"time_to_target_s": t, "iterations_to_target": it,
                     "final_perplexity": c[-1][2], "iterations": c[-1][0],
                     "wall_s": c[-1][1], "curve": [(i, round(tt, 4), p) for i, tt, p in c]}
    base = out["f32_plain"]["time_to_target_s"]
    line = {"metric": "time to held-out perplexity within 1% of the FP32 plain GPU path",
            "workload": args.workload, "N": net.N, "E": net.num_total_edges, "K": opts.K,
            "target": target, "f32_plain_final": final, "interval": interval,
            "speedup_bf16_graph_vs_f32_plain":
                (base / out["bf16_graph"]["time_to_target_s"])
                if base and out["bf16_graph"]["time_to_target_s"] else None,
            "runs": out, "vs_fp64": f64}
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# many chains: one launch per iteration for all of them
# ---------------------------------------------------------------------------
def chains_arm(args):
    """The batching workload: args.chains independent chains, each on its own
    synthetic graph from seed i (N log-uniform in [1,000, 50,000], intra
    degree 6, K in {16, 32, 64, 128}, minibatch 32..1024, 32 neighbours,
    BF16 pi), advanced as one batch (one CUDA graph launch per iteration for
    all chains), against the same chains stepped one after another with
    their own per-chain graphs."""
    import torch
    from mcmc_for_ammsb_gb300 import ChainBatch, MCMCSamplerStochastic, Network, Options, workloads
    samplers, configs = [], []
    for i in range(args.chains):
        w = workloads.chain_workload(i)
        net = Network.synthetic(**w["gen"])
        net.make_held_out(w["opts"]["held_out_ratio"], seed=w["gen"]["seed"])
        s = MCMCSamplerStochastic(Options(**w["opts"]), net).init()
        if not args.no_autotune:
            configs.append(s.autotune(reps=5))
        samplers.append(s)
    batch = ChainBatch(samplers)
    stream = torch.cuda.ExternalStream(batch.stream())

    def evals():
        return sum(s.counters()[0] for s in samplers)

    batch.step(args.warmup)
    torch.cuda.synchronize()
    e0 = evals()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    batch.step(args.steps)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    e1 = evals()
    # the same chains without the batch: every chain runs its own graph on
    # its own stream (all streams queued at once, so the GPU runs them side
    # by side), host clock around all of them
    for s in samplers:
        s.step(args.warmup)
    torch.cuda.synchronize()
    e2 = evals()
    t0 = time.perf_counter()
    for s in samplers:
        s.step(args.steps)
    torch.cuda.synchronize()
    seq_s = time.perf_counter() - t0
    e3 = evals()
    Ks = sorted({s.K for s in samplers})
    line = {"metric": "edge-evals/s, %d independent chains, one graph launch per iteration" % args.chains,
            "value": (e1 - e0) / (ms / 1000.0), "unit": UNIT,
            "ms_per_iteration_all_chains": ms / args.steps,
            "chain_iterations_per_s": args.chains * args.steps / (ms / 1000.0),
            "per_chain_streams_value": (e3 - e2) / seq_s,
            "per_chain_streams_ms_per_iteration_all_chains": 1000.0 * seq_s / args.steps,
            "update_phi_launches_per_iteration": batch.groups(),
            "chains": args.chains, "K_values": Ks, "steps": args.steps, "warmup": args.warmup,
            "autotuned": not args.no_autotune,
            "configs": sorted({json.dumps(c, sort_keys=True) for c in configs}),
            "N_range": [min(s.N for s in samplers), max(s.N for s in samplers)],
            "dtype": "bf16-pi/f32", "data": "synthetic (planted-community generator, seed i per chain)"}
    print(json.dumps(line))
    batch.close()
    for s in samplers:
        s.close()


def gather_roofline_arm():
    """Random whole-row gathers from an 8 GiB table into a shared-memory ring
    (mcmc_for_ammsb_gb300/csrc/gather_roofline.cu), 16 warps per SM as
    k_update_phi_ring: one JSON line per row size, then one with the 2 KiB
    rate as a fraction of the measured copy peak."""
    from mcmc_for_ammsb_gb300 import build as pkg_build
    r = subprocess.run([pkg_build.build_probe(), "8", "4"], capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stderr)
        raise SystemExit(r.returncode)
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    for x in lines:
        print(json.dumps(x))
    peaks, src = load_peaks()
    peak = float(peaks.get("hbm_gbs", 0.0))
    two = [x for x in lines if x["row_bytes"] == 2048]
    if two and peak:
        print(json.dumps({"gather_2KiB_GBps": two[0]["GBps"], "copy_peak_GBps": peak, "peak_source": src,
                          "frac": two[0]["GBps"] / peak}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=6000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="large", choices=["large", "large_s", "mid", "small"])
    ap.add_argument("--strategy", default="stratified-random-node",
                    choices=["stratified-random-node", "stratified-random-node-links",
                             "stratified-random-node-nonlinks"])
    ap.add_argument("--pi-dtype", default="bf16", choices=["bf16", "f32"])
    ap.add_argument("--profile-steps", type=int, default=40)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ttp-iters-line", type=int, default=100000,
                    help="iterations of the time-to-perplexity runs in the throughput line "
                         "(0: leave them out)")
    ap.add_argument("--ttp-interval-line", type=int, default=5000)
    ap.add_argument("--no-fp64", action="store_true",
                    help="leave out the errors against the FP64 oracle")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=2000,
                    help="iterations of the public-loop (e2e) measurement, at least --steps")
    ap.add_argument("--ttp", action="store_true",
                    help="time to perplexity (FP32 plain vs BF16 graph-captured) instead of "
                         "the throughput line")
    ap.add_argument("--ttp-iters", type=int, default=2000)
    ap.add_argument("--ttp-interval", type=int, default=100)
    ap.add_argument("--ttp-cpu-iters", type=int, default=0,
                    help="also run the oracle's CPU restatement for this many iterations")
    ap.add_argument("--ttp-f64-iters", type=int, default=0,
                    help="perplexity error of the FP32/BF16 paths against the FP64 oracle "
                         "over this many iterations")
    ap.add_argument("--ttp-f64-interval", type=int, default=50)
    ap.add_argument("--chains", type=int, default=0,
                    help="run the batching workload with this many chains instead")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--gather-roofline", action="store_true",
                    help="run the random-row gather probe (the ceiling of update_phi's access "
                         "pattern) instead of the throughput line")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.gather_roofline:
        gather_roofline_arm()
        return
    if args.ttp:
        ttp_arm(args)
        return
    if args.chains:
        chains_arm(args)
        return

    rank, world, local = dist_env()
    if args.impl == "reference" and rank != 0:
        return
    if world > 1 and args.impl == "ours":
        import torch.distributed as dist
        dist.init_process_group("gloo")

    from mcmc_for_ammsb_gb300 import workloads
    from mcmc_for_ammsb_gb300.options import STRATEGIES
    if args.impl == "reference":
        reference_arm(args)
    else:
        net, opts = workloads.build(args.workload, strategy=STRATEGIES[args.strategy])
        ours_arm(args, net, opts, rank, world, local)
    if world > 1 and args.impl == "ours":
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
