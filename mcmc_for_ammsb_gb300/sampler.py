"""MCMCSamplerStochastic on the GPU: the reference's sampler object
(mcmc_sampler_stochastic.h:32-140, learner.h:24-172) as a thin Python handle
over libammsb_gpu.so.

Usage mirrors apps/main/main.cc:69-76::

    s = MCMCSamplerStochastic(Options(argv), network)
    s.init()
    s.run()

All state lives in GPU memory owned by the native handle; the methods below
call the C ABI and copy results back only when asked.
"""
import ctypes

import numpy as np

from . import _native
from .network import Network
from .options import Options


class MCMCSamplerStochastic:
    def __init__(self, args, network=None):
        if not isinstance(args, Options):
            args = Options(args)
        self.args = args
        self.network = network
        self._h = None

    # -- Learner::LoadNetwork + init ------------------------------------------
    def load_network(self):
        """Learner::LoadNetwork (learner.cc:86-97): graph from the input file
        when no Network was given, then the held-out and test sets."""
        if self.network is None:
            if not self.args.input_filename_:
                raise ValueError("no network given and --mcmc.input.file empty")
            self.network = Network.from_relativity(self.args.input_filename_,
                                                   self.args.input_contiguous_)
        if self.network.held_out[0].shape[0] == 0 and self.network.test[0].shape[0] == 0:
            ratio = self.args.held_out_ratio if self.args.held_out_ratio != 0.0 else 0.1
            self.network.make_held_out(ratio, seed=self.args.random_seed & 0xffffffff)
        return self.network

    def create(self):
        if self._h is not None:
            return self
        net = self.load_network()
        L = _native.lib()
        opt = self.args.to_native()
        g = net.native_graph()
        ho, self._ho_keep = Network.native_edge_set(net.held_out)
        te, self._te_keep = Network.native_edge_set(net.test)
        h = ctypes.c_void_p()
        _native.check(L.ammsb_create(ctypes.byref(opt), ctypes.byref(g), ctypes.byref(ho),
                                     ctypes.byref(te), ctypes.byref(h)))
        self._h = h
        N, K, me, mn, nns, H = (ctypes.c_int64() for _ in range(6))
        L.ammsb_get_sizes(h, *(ctypes.byref(x) for x in (N, K, me, mn, nns, H)))
        self.N, self.K = N.value, K.value
        self.max_edges, self.max_nodes = me.value, mn.value
        self.num_node_sample, self.held_out_count = nns.value, H.value
        o = _native.AmmsbOptions()
        L.ammsb_get_options(h, ctypes.byref(o))
        self.resolved = o
        return self

    def init(self):
        """MCMCSamplerStochastic::init (cc:29-79)."""
        self.create()
        self._check(_native.lib().ammsb_init_state(self._h))
        return self

    def set_state(self, phi, theta):
        self.create()
        phi = np.ascontiguousarray(phi, dtype=np.float32)
        theta = np.ascontiguousarray(theta, dtype=np.float64)
        assert phi.shape == (self.N, self.K) and theta.shape == (self.K, 2)
        self._check(_native.lib().ammsb_set_state(
            self._h, phi.ctypes.data_as(_native._F32P), theta.ctypes.data_as(_native._F64P)))
        return self

    def autotune(self, reps=5, fresh=False):
        """Times the built update_phi shapes for this chain (ammsb_autotune)
        and keeps the fastest; returns the configuration in use."""
        self._check(_native.lib().ammsb_autotune(self._h, int(reps),
                                                 _native.TUNE_FRESH if fresh else 0))
        return self.kernel_config()

    def kernel_config(self):
        """(ring kernel, lanes per node, vectors per lane, sub-groups
        per node, ring depth) of update_phi."""
        out = (ctypes.c_int32 * 5)()
        self._check(_native.lib().ammsb_get_kernel_config(self._h, out))
        return dict(zip(("ring", "lanes", "vectors", "split", "stages"), list(out)))

    def save_checkpoint(self, path):
        """Writes the whole chain (state, counters, running averages, Philox
        key) to `path`; see ammsb_save_checkpoint."""
        self._check(_native.lib().ammsb_save_checkpoint(self._h, str(path).encode()))

    def load_checkpoint(self, path):
        """Restores a chain saved by save_checkpoint; the trajectory then
        continues bit for bit."""
        self.create()
        self._check(_native.lib().ammsb_load_checkpoint(self._h, str(path).encode()))
        return self

    # -- iteration ------------------------------------------------------------
    def run(self):
        """MCMCSamplerStochastic::run (cc:93-183); returns the last perplexity.
        Initialises the state first (init()) when nothing set it."""
        self.create()
        out = ctypes.c_double()
        self._check(_native.lib().ammsb_run(self._h, ctypes.byref(out)))
        return out.value

    def step(self, n=1):
        self._check(_native.lib().ammsb_step(self._h, int(n)))

    def cal_perplexity_held_out(self):
        out = ctypes.c_double()
        self._check(_native.lib().ammsb_perplexity(self._h, ctypes.byref(out)))
        return out.value

    def step_fed(self, step, edge_slots, edge_y, scale, nodes, nbrs, nbr_y, phi_noise,
                 theta_noise):
        """One iteration with every draw given (parity hook)."""
        es = np.ascontiguousarray(edge_slots, dtype=np.int32).reshape(-1, 2)
        ea = np.ascontiguousarray(es[:, 0])
        eb = np.ascontiguousarray(es[:, 1])
        ey = np.ascontiguousarray(edge_y, dtype=np.uint8)
        nodes = np.ascontiguousarray(nodes, dtype=np.int32)
        nbrs = np.ascontiguousarray(nbrs, dtype=np.int32)
        nbr_y = np.ascontiguousarray(nbr_y, dtype=np.uint8)
        pn = np.ascontiguousarray(phi_noise, dtype=np.float32)
        tn = np.ascontiguousarray(theta_noise, dtype=np.float32)
        assert nbrs.shape == (nodes.shape[0], self.num_node_sample + 1)
        assert pn.shape == (nodes.shape[0], self.K) and tn.shape == (self.K, 2)
        self._check(_native.lib().ammsb_step_fed(
            self._h, int(step), ea.shape[0], ea.ctypes.data_as(_native._I32P),
            eb.ctypes.data_as(_native._I32P), ey.ctypes.data_as(_native._U8P), float(scale),
            nodes.shape[0], nodes.ctypes.data_as(_native._I32P),
            nbrs.ctypes.data_as(_native._I32P), nbr_y.ctypes.data_as(_native._U8P),
            pn.ctypes.data_as(_native._F32P), tn.ctypes.data_as(_native._F32P)))

    def profile_step(self):
        ms = (ctypes.c_double * 5)()
        self._check(_native.lib().ammsb_profile_step(self._h, ms))
        names = ["sample_mini_batch", "sample_neighbor_nodes", "update_phi",
                 "update_pi+beta_grads", "update_theta"]
        return dict(zip(names, list(ms)))

    # -- state ------------------------------------------------------------------
    def _get(self, fn, shape, dtype, ptype):
        out = np.empty(shape, dtype=dtype)
        self._check(fn(self._h, out.ctypes.data_as(ptype)))
        return out

    @property
    def pi(self):
        return self._get(_native.lib().ammsb_get_pi, (self.N, self.K), np.float32, _native._F32P)

    @property
    def phi(self):
        return self._get(_native.lib().ammsb_get_phi, (self.N, self.K), np.float32, _native._F32P)

    @property
    def theta(self):
        return self._get(_native.lib().ammsb_get_theta, (self.K, 2), np.float64, _native._F64P)

    @property
    def beta(self):
        return self._get(_native.lib().ammsb_get_beta, (self.K,), np.float32, _native._F32P)

    @property
    def ppx_per_heldout_edge(self):
        return self._get(_native.lib().ammsb_get_ppx, (self.held_out_count,), np.float32,
                         _native._F32P)

    @property
    def step_count(self):
        s, a = ctypes.c_uint64(), ctypes.c_uint64()
        _native.lib().ammsb_get_step(self._h, ctypes.byref(s), ctypes.byref(a))
        return s.value

    @property
    def average_count(self):
        s, a = ctypes.c_uint64(), ctypes.c_uint64()
        _native.lib().ammsb_get_step(self._h, ctypes.byref(s), ctypes.byref(a))
        return a.value

    def set_step(self, step_count):
        self._check(_native.lib().ammsb_set_step(self._h, int(step_count)))

    def last_minibatch(self):
        """Draws of the last iteration: dict of flag, scale, edges, nodes,
        neighbours (for sampling parity)."""
        L = _native.lib()
        me, mn, n_out = self.max_edges, self.max_nodes, self.num_node_sample + 1
        flag, ne, nn = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        scale = ctypes.c_float()
        ea = np.zeros(me, np.int32)
        eb = np.zeros(me, np.int32)
        ey = np.zeros(me, np.uint8)
        nodes = np.zeros(mn, np.int32)
        nbrs = np.zeros(mn * n_out, np.int32)
        nby = np.zeros(mn * n_out, np.uint8)
        self._check(L.ammsb_get_last_minibatch(
            self._h, ctypes.byref(flag), ctypes.byref(ne), ctypes.byref(nn), ctypes.byref(scale),
            ea.ctypes.data_as(_native._I32P), eb.ctypes.data_as(_native._I32P),
            ey.ctypes.data_as(_native._U8P), nodes.ctypes.data_as(_native._I32P),
            nbrs.ctypes.data_as(_native._I32P), nby.ctypes.data_as(_native._U8P)))
        e, n = ne.value, nn.value
        return dict(flag=flag.value, scale=scale.value, edge_a=ea[:e], edge_b=eb[:e],
                    edge_y=ey[:e], nodes=nodes[:n], nbrs=nbrs[:n * n_out].reshape(n, n_out),
                    nbr_y=nby[:n * n_out].reshape(n, n_out))

    # -- one rank's phases of a sharded iteration (sharded.ShardedChain) -----
    def shard_draw(self):
        """Draws iteration step_count's minibatch and neighbour sets on the
        device (ammsb_shard_draw); returns them as last_minibatch() does."""
        self._check(_native.lib().ammsb_shard_draw(self._h))
        return self.last_minibatch()

    def shard_update(self, slots):
        """update_phi of the drawn nodes at `slots` (ascending); returns
        their new pi rows (len(slots) x K, float32)."""
        slots = np.ascontiguousarray(slots, np.int32)
        rows = np.zeros((slots.shape[0], self.K), np.float32)
        self._check(_native.lib().ammsb_shard_update(
            self._h, slots.shape[0], slots.ctypes.data_as(_native._I32P),
            rows.ctypes.data_as(_native._F32P)))
        return rows

    def shard_commit(self, rows_all, edge_idx):
        """Commits every drawn node's new pi row (slot order) and returns
        the beta-gradient sums over the edges at `edge_idx` (K x 2)."""
        rows_all = np.ascontiguousarray(rows_all, np.float32)
        edge_idx = np.ascontiguousarray(edge_idx, np.int32)
        R = np.zeros((self.K, 2), np.float64)
        self._check(_native.lib().ammsb_shard_commit(
            self._h, rows_all.ctypes.data_as(_native._F32P), edge_idx.shape[0],
            edge_idx.ctypes.data_as(_native._I32P), R.ctypes.data_as(_native._F64P)))
        return R

    def shard_theta(self, R_total):
        """The theta step from the beta-gradient sums of all ranks."""
        R_total = np.ascontiguousarray(R_total, np.float64)
        self._check(_native.lib().ammsb_shard_theta(self._h, R_total.ctypes.data_as(_native._F64P)))

    def counters(self):
        """(edge evaluations, iterations) sampled on the device so far."""
        e, i = ctypes.c_uint64(), ctypes.c_uint64()
        self._check(_native.lib().ammsb_get_counters(self._h, ctypes.byref(e), ctypes.byref(i)))
        return e.value, i.value

    def stream(self):
        return _native.lib().ammsb_stream(self._h)

    def _check(self, code):
        return _native.check(code, self._h)

    def close(self):
        if self._h is not None:
            _native.lib().ammsb_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class ChainBatch:
    """Independent chains advanced together, one CUDA graph launch per
    iteration for all of them (ammsb_batch_*).  Every sampler keeps its own
    graph, state and step counter; step(n) advances all of them by n."""

    def __init__(self, samplers):
        self.samplers = list(samplers)
        if not self.samplers:
            raise ValueError("need at least one sampler")
        for s in self.samplers:
            s.create()
        arr = (ctypes.c_void_p * len(self.samplers))(*[s._h.value for s in self.samplers])
        out = ctypes.c_void_p()
        code = _native.lib().ammsb_batch_create(arr, len(self.samplers), ctypes.byref(out))
        if code != _native.AMMSB_OK:
            raise _native.AmmsbError(code, (_native.lib().ammsb_batch_create_error() or b"").decode())
        self._b = out

    def step(self, n=1):
        code = _native.lib().ammsb_batch_step(self._b, int(n))
        if code != _native.AMMSB_OK:
            raise _native.AmmsbError(code, (_native.lib().ammsb_batch_last_error(self._b) or b"").decode())

    def groups(self):
        """update_phi launches per iteration (distinct kernel shapes)."""
        return _native.lib().ammsb_batch_groups(self._b)

    def stream(self):
        return _native.lib().ammsb_batch_stream(self._b)

    def close(self):
        if getattr(self, "_b", None) is not None:
            _native.lib().ammsb_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
