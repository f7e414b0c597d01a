"""The N-GPU bench path on CPU: ranks of independent replicas (one chain
per rank, Philox chain = rank) reduce their timings over a gloo process
group -- the slowest rank's seconds and the sum of the evaluations -- which
is how `python -m torch.distributed.run ... bench.py --gpus N` reports the
whole-job throughput.  World size 2, 127.0.0.1 rendezvous."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    secs, evals = bench.reduce_over_ranks(1.0 + rank, 10.0 * (rank + 1), world)
    out.put((rank, secs, evals))
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_reduce_over_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert got == [(0, 2.0, 30.0), (1, 2.0, 30.0)]


def test_single_rank_is_identity():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    assert bench.reduce_over_ranks(1.5, 7.0, 1) == (1.5, 7.0)
