"""One SG-MCMC iteration split over ranks: the distributed sampler's
partition (mcmc_sampler_stochastic_distr.cc) on GPUs that each hold all of
pi.

The reference's distributed sampler gives each rank the minibatch nodes it
owns, node % ranks (distr.cc:1626-1632); the ranks update those nodes'
phi, write the new pi rows to a distributed key-value store read by all
(distr.cc:630-708), and add their beta-gradient sums with MPI (distr.cc:
1430-1442) before the theta step.  Here pi is replicated on every GPU
(8 GB in BF16 at N = 4M, K = 1024), so neighbour rows are always read
locally, and only what changed moves:
  1. every rank draws the same minibatch and neighbour sets -- the draws are
     a function of (seed, chain, step), so no rank broadcasts them;
  2. each rank updates the phi rows of the nodes it owns and returns their
     new pi rows;
  3. the ranks exchange those rows (an all-gather of at most m + 1 rows);
  4. each rank commits every new row into its pi and sums the beta gradient
     over the edges it owns (an edge belongs to the owner of its second
     node, the partner of the star minibatch);
  5. the ranks exchange their K x 2 sums and add them in rank order, so
     every rank takes the same theta step.
A backend is one rank's sampler (MCMCSamplerStochastic: the shard_* calls
of the C ABI); `comm` moves Python objects between ranks (TorchComm over
torch.distributed, or any object with the same allgather).  With one rank
the iteration equals MCMCSamplerStochastic.step(1) bit for bit.
"""
import numpy as np


def owner(nodes, world):
    """The rank that owns each node (distr.cc:1626-1632)."""
    return np.asarray(nodes, np.int64) % world


class TorchComm:
    """allgather of picklable objects over a torch.distributed group."""

    def __init__(self, group=None):
        import torch.distributed as dist
        self.dist = dist
        self.group = group
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)

    def allgather(self, obj):
        out = [None] * self.world
        self.dist.all_gather_object(out, obj, group=self.group)
        return out


class ShardedChain:
    """One rank of a sharded chain.  step(comm) runs a whole iteration;
    draw_and_update / commit / finish are its three phases between the two
    exchanges, for drivers that move the data themselves."""

    def __init__(self, backend, rank, world):
        if not (0 <= rank < world):
            raise ValueError("rank %d outside a world of %d" % (rank, world))
        self.backend = backend
        self.rank = rank
        self.world = world
        self._mb = None

    def draw_and_update(self):
        """Phases 1-2: returns (owned slots, their new pi rows)."""
        mb = self.backend.shard_draw()
        self._mb = mb
        slots = np.nonzero(owner(mb["nodes"], self.world) == self.rank)[0].astype(np.int32)
        return slots, self.backend.shard_update(slots)

    def commit(self, payloads):
        """Phase 4: every rank's (slots, rows) in rank order; returns this
        rank's beta-gradient sums."""
        mb = self._mb
        if mb is None:
            raise RuntimeError("commit() follows draw_and_update()")
        if len(payloads) != self.world:
            raise ValueError("one payload per rank expected")
        n = len(mb["nodes"])
        rows_all = np.zeros((n, self.backend.K), np.float32)
        seen = np.zeros(n, np.int32)
        for r, (slots, rows) in enumerate(payloads):
            slots = np.asarray(slots, np.int64)
            if np.any(owner(mb["nodes"][slots], self.world) != r):
                raise ValueError("rank %d sent rows of nodes it does not own" % r)
            rows_all[slots] = rows
            seen[slots] += 1
        if not np.all(seen == 1):
            raise ValueError("every drawn node needs exactly one new row")
        partner = mb["nodes"][mb["edge_b"]]
        edges = np.nonzero(owner(partner, self.world) == self.rank)[0].astype(np.int32)
        return self.backend.shard_commit(rows_all, edges)

    def finish(self, sums):
        """Phase 5: the ranks' sums, added in rank order; the theta step."""
        if len(sums) != self.world:
            raise ValueError("one sum per rank expected")
        total = sums[0].copy()
        for x in sums[1:]:
            total = total + x
        self.backend.shard_theta(total)
        self._mb = None

    def step(self, comm):
        payload = self.draw_and_update()
        mine = self.commit(comm.allgather(payload))
        self.finish(comm.allgather(mine))
