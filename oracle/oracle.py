"""ctypes front end of the CPU oracle (ammsb_oracle.c).

TEST INFRASTRUCTURE ONLY.  Imported by tests/, __graft_entry__.smoke() and
bench.py's cpu_baseline / reference legs, as the checker.  The product
package never imports this module.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libammsb_oracle.so")
SRC = [os.path.join(HERE, f) for f in ("ammsb_oracle.c", "ammsb_oracle_graph.c",
                                       "ammsb_oracle_impl.h", "ammsb_oracle.h")]

# stream tags (ammsb_oracle.h)
P_MB_FLAG, P_MB_NODE, P_MB_CAND, P_NBR, P_PHI_NOISE, P_THETA_NOISE, P_PHI_INIT, P_THETA_INIT = range(1, 9)


def build(force=False):
    os.makedirs(BUILD, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and all(os.path.getmtime(s) <= os.path.getmtime(LIB) for s in SRC)):
        return LIB
    cmd = ["gcc", "-O2", "-std=c11", "-Wall", "-Wextra", "-ffp-contract=off", "-fPIC", "-shared",
           "-fopenmp", "-o", LIB + ".tmp", SRC[0], SRC[1], "-lm"]
    subprocess.run(cmd, check=True, cwd=HERE)
    os.replace(LIB + ".tmp", LIB)
    return LIB


class MbInfo(ctypes.Structure):
    _fields_ = [("flag", ctypes.c_int32), ("n_edges", ctypes.c_int32),
                ("n_nodes", ctypes.c_int32), ("scale", ctypes.c_float),
                ("rounds", ctypes.c_int32)]


class Graph(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("row_ptr", ctypes.c_void_p), ("col", ctypes.c_void_p),
                ("excl", ctypes.c_void_p), ("n_excl", ctypes.c_int64)]


class Params(ctypes.Structure):
    _fields_ = [("K", ctypes.c_int32), ("N", ctypes.c_int64), ("num_total_edges", ctypes.c_int64),
                ("strategy", ctypes.c_int32), ("mini_batch_size", ctypes.c_int64),
                ("num_node_sample", ctypes.c_int64), ("alpha", ctypes.c_float),
                ("epsilon", ctypes.c_float), ("eta0", ctypes.c_float), ("eta1", ctypes.c_float),
                ("a", ctypes.c_double), ("b", ctypes.c_double), ("c", ctypes.c_double),
                ("seed", ctypes.c_uint32), ("chain", ctypes.c_uint32),
                ("max_source", ctypes.c_int64)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.oracle_draw_u64.restype = ctypes.c_uint64
        L.oracle_draw_u64.argtypes = [ctypes.c_uint32] * 5 + [ctypes.c_uint64]
        L.oracle_normal.restype = ctypes.c_float
        L.oracle_normal.argtypes = [ctypes.c_uint32] * 5 + [ctypes.c_uint64]
        L.oracle_gamma.restype = ctypes.c_double
        L.oracle_gamma.argtypes = [ctypes.c_uint32] * 4 + [ctypes.c_uint64, ctypes.c_double,
                                                           ctypes.c_double]
        L.oracle_nonlink_scale.restype = ctypes.c_float
        L.oracle_nonlink_scale.argtypes = [ctypes.c_int64] * 3
        L.oracle_eps_t.restype = ctypes.c_float
        L.oracle_eps_t.argtypes = [ctypes.c_double] * 3 + [ctypes.c_uint64]
        L.oracle_eps_t_ref.restype = ctypes.c_float
        L.oracle_eps_t_ref.argtypes = [ctypes.c_float] * 3 + [ctypes.c_uint64]
        L.oracle_sample_minibatch.restype = ctypes.c_int
        L.oracle_sample_neighbors.restype = ctypes.c_int64
        L.oracle_edge_likelihood_f32.restype = ctypes.c_float
        L.oracle_edge_likelihood_f64.restype = ctypes.c_double
        L.oracle_perplexity_f32.restype = ctypes.c_float
        L.oracle_perplexity_f64.restype = ctypes.c_double
        L.oracle_perplexity_f64acc.restype = ctypes.c_double
        L.oracle_step_f32.restype = ctypes.c_int
        L.oracle_step_f64.restype = ctypes.c_int
        L.oracle_step_f32_threads.restype = ctypes.c_int
        L.oracle_generate_graph.restype = ctypes.c_int
        L.oracle_held_out_pairs.restype = ctypes.c_int64
        L.oracle_held_out_pairs.argtypes = [ctypes.c_int64, ctypes.c_double]
        L.oracle_make_held_out.restype = ctypes.c_int
        L.oracle_free.argtypes = [ctypes.c_void_p]
        _lib = L
    return _lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def philox(ctr, key):
    o = (ctypes.c_uint32 * 4)()
    lib().oracle_philox4x32_10((ctypes.c_uint32 * 4)(*ctr), (ctypes.c_uint32 * 2)(*key), o)
    return list(o)


class GenParams(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("k_true", ctypes.c_int64), ("zipf_s", ctypes.c_double),
                ("size_min", ctypes.c_int64), ("size_max", ctypes.c_int64),
                ("p1", ctypes.c_double), ("p2", ctypes.c_double),
                ("intra_degree", ctypes.c_double), ("background_frac", ctypes.c_double),
                ("seed", ctypes.c_uint32)]


class SyntheticNetwork:
    """A workload's graph and held-out / test sets built by the oracle's own
    restatement of the generator and the split (ammsb_oracle_graph.c), with
    the attributes OracleGraph and OracleSampler read.  The CPU legs of the
    benchmark use it so that they load no library of the product."""

    def __init__(self, row_ptr, col):
        self.row_ptr = row_ptr
        self.col = col
        self.N = int(row_ptr.shape[0] - 1)
        z = (np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros(0, np.uint8))
        self.held_out, self.test = z, z

    @staticmethod
    def synthetic(n, k_true, size_min=10, size_max=500, zipf_s=1.5, p1=0.7, p2=0.25,
                  intra_degree=4.0, background_frac=0.1, seed=0):
        prm = GenParams(n, k_true, zipf_s, size_min, size_max, p1, p2, intra_degree,
                        background_frac, seed & 0xffffffff)
        rp = ctypes.c_void_p()
        cl = ctypes.c_void_p()
        if lib().oracle_generate_graph(ctypes.byref(prm), ctypes.byref(rp), ctypes.byref(cl)):
            raise RuntimeError("oracle graph generation failed")
        try:
            row_ptr = np.ctypeslib.as_array(ctypes.cast(rp, ctypes.POINTER(ctypes.c_int64)),
                                            shape=(n + 1,)).copy()
            ne = int(row_ptr[-1])
            col = (np.ctypeslib.as_array(ctypes.cast(cl, ctypes.POINTER(ctypes.c_int32)),
                                         shape=(ne,)).copy() if ne else np.zeros(0, np.int32))
        finally:
            lib().oracle_free(rp)
            lib().oracle_free(cl)
        return SyntheticNetwork(row_ptr, col)

    def make_held_out(self, ratio, seed=0):
        p = lib().oracle_held_out_pairs(self.num_total_edges, ratio)
        arr = [np.zeros(2 * p, t) for t in (np.int32, np.int32, np.uint8) * 2]
        rc = lib().oracle_make_held_out(ctypes.c_int64(self.N), _p(self.row_ptr), _p(self.col),
                                        ctypes.c_double(ratio), ctypes.c_uint32(seed & 0xffffffff),
                                        *[_p(a) for a in arr])
        if rc:
            raise RuntimeError("oracle held-out construction failed")
        self.held_out = tuple(arr[:3])
        self.test = tuple(arr[3:])
        return self

    @property
    def num_total_edges(self):
        return int(self.row_ptr[-1]) // 2

    def max_degree(self):
        return int(np.max(np.diff(self.row_ptr))) if self.N else 0


class OracleGraph:
    """Graph + exclusion keys held for the C oracle."""

    def __init__(self, network):
        self.row_ptr = np.ascontiguousarray(network.row_ptr, np.int64)
        self.col = np.ascontiguousarray(network.col, np.int32)
        a = np.concatenate([network.held_out[0], network.test[0]]).astype(np.uint64)
        b = np.concatenate([network.held_out[1], network.test[1]]).astype(np.uint64)
        keys = (np.minimum(a, b) << np.uint64(32)) | np.maximum(a, b)
        self.excl = np.ascontiguousarray(np.unique(keys), np.uint64)
        self.N = int(self.row_ptr.shape[0] - 1)
        self.g = Graph(self.N, self.row_ptr.ctypes.data, self.col.ctypes.data,
                       self.excl.ctypes.data, self.excl.shape[0])

    def has_edge(self, a, b):
        return bool(lib().oracle_has_edge(ctypes.byref(self.g), int(a), int(b)))

    def is_excluded(self, a, b):
        return bool(lib().oracle_is_excluded(ctypes.byref(self.g), int(a), int(b)))


def sample_minibatch(og, strategy, m, num_total_edges, seed, chain, step, max_edges,
                     max_source=1):
    ea = np.zeros(max_edges, np.int32)
    eb = np.zeros(max_edges, np.int32)
    ey = np.zeros(max_edges, np.uint8)
    nodes = np.zeros(2 * max_edges + 1, np.int32)
    info = MbInfo()
    rc = lib().oracle_sample_minibatch_ex(
        ctypes.byref(og.g), ctypes.c_int(strategy), ctypes.c_int64(m), ctypes.c_int64(max_source),
        ctypes.c_int64(num_total_edges), ctypes.c_uint32(seed), ctypes.c_uint32(chain),
        ctypes.c_uint32(step), _p(ea), _p(eb), _p(ey), ctypes.c_int32(max_edges), _p(nodes),
        ctypes.c_int32(2 * max_edges + 1), ctypes.byref(info))
    if rc != 0:
        raise RuntimeError("oracle minibatch sampling failed: %d" % rc)
    e, n = info.n_edges, info.n_nodes
    return dict(flag=info.flag, scale=info.scale, edge_a=ea[:e], edge_b=eb[:e], edge_y=ey[:e],
                nodes=nodes[:n], rounds=info.rounds)


def sample_neighbors(og, node, n_out, seed, chain, step):
    out = np.zeros(n_out, np.int32)
    y = np.zeros(n_out, np.uint8)
    rc = lib().oracle_sample_neighbors(ctypes.byref(og.g), ctypes.c_int32(node),
                                       ctypes.c_int32(n_out), ctypes.c_uint32(seed),
                                       ctypes.c_uint32(chain), ctypes.c_uint32(step), _p(out),
                                       _p(y))
    if rc < 0:
        raise RuntimeError("oracle neighbour sampling failed")
    return out, y


def normals(seed, chain, tag, entity, step, count):
    L = lib()
    return np.array([L.oracle_normal(seed, chain, tag, entity, step, k) for k in range(count)],
                    np.float32)


def eps_t(a, b, c, step):
    return lib().oracle_eps_t(a, b, c, step)


def eps_t_ref(a, b, c, step):
    return lib().oracle_eps_t_ref(a, b, c, step)


def nonlink_scale(N, m, E):
    return lib().oracle_nonlink_scale(N, m, E)


def update_phi(K, pi, phi_i, i, nbrs, y, beta, alpha, epsilon, eps, N, num_node_sample, noise,
               dtype=np.float32):
    """Literal update_phi of one node; returns the new phi row."""
    f64 = dtype == np.float64
    pi = np.ascontiguousarray(pi, dtype)
    out = np.ascontiguousarray(phi_i, dtype).copy()
    nbrs = np.ascontiguousarray(nbrs, np.int32)
    y = np.ascontiguousarray(y, np.uint8)
    beta = np.ascontiguousarray(beta, dtype)
    noise = np.ascontiguousarray(noise, dtype)
    fn = lib().oracle_update_phi_f64 if f64 else lib().oracle_update_phi_f32
    real = ctypes.c_double if f64 else ctypes.c_float
    fn(ctypes.c_int32(K), _p(pi), _p(out), ctypes.c_int32(i), _p(nbrs), _p(y),
       ctypes.c_int32(nbrs.shape[0]), _p(beta), real(alpha), real(epsilon), real(eps),
       ctypes.c_int64(N), ctypes.c_int64(num_node_sample), _p(noise))
    return out


def phi_grad(K, pi, phi_i, i, nbrs, y, beta, epsilon):
    pi = np.ascontiguousarray(pi, np.float64)
    phi_i = np.ascontiguousarray(phi_i, np.float64)
    nbrs = np.ascontiguousarray(nbrs, np.int32)
    y = np.ascontiguousarray(y, np.uint8)
    beta = np.ascontiguousarray(beta, np.float64)
    g = np.zeros(K, np.float64)
    lib().oracle_phi_grad_f64(ctypes.c_int32(K), _p(pi), _p(phi_i), ctypes.c_int32(i), _p(nbrs),
                              _p(y), ctypes.c_int32(nbrs.shape[0]), _p(beta),
                              ctypes.c_double(epsilon), _p(g))
    return g


def update_beta(K, pi, ea, eb, ey, theta, beta, eta, epsilon, eps, scale, noise,
                dtype=np.float32):
    """Literal update_beta; returns (theta, beta, grads)."""
    f64 = dtype == np.float64
    pi = np.ascontiguousarray(pi, dtype)
    th = np.ascontiguousarray(theta, dtype).copy()
    bt = np.ascontiguousarray(beta, dtype).copy()
    ea = np.ascontiguousarray(ea, np.int32)
    eb = np.ascontiguousarray(eb, np.int32)
    ey = np.ascontiguousarray(ey, np.uint8)
    eta = np.ascontiguousarray(eta, dtype)
    noise = np.ascontiguousarray(noise, dtype)
    grads = np.zeros((K, 2), dtype)
    fn = lib().oracle_update_beta_f64 if f64 else lib().oracle_update_beta_f32
    real = ctypes.c_double if f64 else ctypes.c_float
    fn(ctypes.c_int32(K), _p(pi), _p(ea), _p(eb), _p(ey), ctypes.c_int32(ea.shape[0]), _p(th),
       _p(bt), _p(eta), real(epsilon), real(eps), real(scale), _p(noise), _p(grads))
    return th, bt, grads


def edge_likelihood(K, pa, pb, y, beta, epsilon, dtype=np.float64):
    """cal_edge_likelihood (learner.h:100-139) of one pair of pi rows."""
    f64 = dtype == np.float64
    real = ctypes.c_double if f64 else ctypes.c_float
    fn = lib().oracle_edge_likelihood_f64 if f64 else lib().oracle_edge_likelihood_f32
    return fn(ctypes.c_int32(K), _p(np.ascontiguousarray(pa, dtype)),
              _p(np.ascontiguousarray(pb, dtype)), ctypes.c_int(int(y)),
              _p(np.ascontiguousarray(beta, dtype)), real(epsilon))


def normalize(phi, dtype=np.float32):
    phi = np.ascontiguousarray(phi, dtype)
    K = phi.shape[-1]
    out = np.empty_like(phi)
    fn = lib().oracle_normalize_f64 if dtype == np.float64 else lib().oracle_normalize_f32
    for r in range(phi.shape[0]):
        fn(ctypes.c_int32(K), ctypes.c_void_p(phi[r].ctypes.data),
           ctypes.c_void_p(out[r].ctypes.data))
    return out


def perplexity(K, pi, held_out, beta, epsilon, ppx, average_count, mode="f32"):
    """cal_perplexity; ppx is updated in place.  mode: f32 (reference
    accumulation), f64acc (device semantics), f64 (all double)."""
    ha, hb, hy = (np.ascontiguousarray(x) for x in held_out)
    H = ha.shape[0]
    L = lib()
    if mode == "f64":
        return L.oracle_perplexity_f64(ctypes.c_int32(K), _p(np.ascontiguousarray(pi, np.float64)),
                                       _p(ha), _p(hb), _p(hy), ctypes.c_int64(H),
                                       _p(np.ascontiguousarray(beta, np.float64)),
                                       ctypes.c_double(epsilon), _p(ppx),
                                       ctypes.c_uint64(average_count))
    fn = L.oracle_perplexity_f32 if mode == "f32" else L.oracle_perplexity_f64acc
    return fn(ctypes.c_int32(K), _p(np.ascontiguousarray(pi, np.float32)), _p(ha), _p(hb),
              _p(hy), ctypes.c_int64(H), _p(np.ascontiguousarray(beta, np.float32)),
              ctypes.c_float(epsilon), _p(ppx), ctypes.c_uint64(average_count))


class OracleSampler:
    """Whole-iteration CPU sampler (float arithmetic in the reference's
    order, Philox draws): the trajectory reference of the GPU path."""

    def __init__(self, network, K, strategy=0, mini_batch_size=None, num_node_sample=None,
                 alpha=0.0, epsilon=1e-7, eta0=1.0, eta1=1.0, a=0.0, b=1024.0, c=0.5, seed=42,
                 chain=0, max_source=1):
        N = network.N
        self.og = OracleGraph(network)
        self.network = network
        if a == 0.0:
            a = b ** (-c)
        if alpha == 0.0:
            alpha = 1.0 / K
        self.p = Params(K, N, network.num_total_edges, strategy,
                        mini_batch_size or N // 10, num_node_sample or N // 50, alpha, epsilon,
                        eta0, eta1, a, b, c, seed & 0xffffffff, chain, max_source)
        self.K, self.N = K, N
        self.step_count = 1
        self.average_count = 1
        self.ppx = np.zeros(network.held_out[0].shape[0], np.float32)

    def set_state(self, phi, theta):
        self.phi = np.ascontiguousarray(phi, np.float32).copy()
        self.theta = np.ascontiguousarray(theta, np.float32).copy()
        self.beta = (self.theta[:, 1] / (self.theta[:, 0] + self.theta[:, 1])).astype(np.float32)
        self.pi = normalize(self.phi)

    def step(self):
        info = MbInfo()
        rc = lib().oracle_step_f32(ctypes.byref(self.p), ctypes.byref(self.og.g),
                                   ctypes.c_uint32(self.step_count), _p(self.pi), _p(self.phi),
                                   _p(self.theta), _p(self.beta), ctypes.byref(info))
        if rc != 0:
            raise RuntimeError("oracle step failed: %d" % rc)
        self.step_count += 1
        return info

    def init_state_threads(self, seed, threads):
        """phi ~ Gamma(1, 1) and pi = phi / sum(phi) for every node, filled
        on `threads` host threads (oracle_init_state_threads); theta ~
        Gamma(1, 1) (K x 2)."""
        N, K = self.N, self.K
        self.phi = np.empty((N, K), np.float32)
        self.pi = np.empty((N, K), np.float32)
        lib().oracle_init_state_threads(ctypes.c_int64(N), ctypes.c_int32(K),
                                        ctypes.c_uint32(seed & 0xffffffff), _p(self.phi),
                                        _p(self.pi), ctypes.c_int(threads))
        rng = np.random.default_rng(seed)
        self.theta = rng.gamma(1.0, 1.0, (K, 2)).astype(np.float32)
        self.beta = (self.theta[:, 1] / (self.theta[:, 0] + self.theta[:, 1])).astype(np.float32)

    def step_threads(self, threads, max_edges=0):
        """The same iteration with the per-node work on `threads` host
        threads (oracle_step_f32_threads); identical results."""
        info = MbInfo()
        rc = lib().oracle_step_f32_threads(
            ctypes.byref(self.p), ctypes.byref(self.og.g), ctypes.c_uint32(self.step_count),
            _p(self.pi), _p(self.phi), _p(self.theta), _p(self.beta), ctypes.byref(info),
            ctypes.c_int(threads), ctypes.c_int64(max_edges))
        if rc != 0:
            raise RuntimeError("oracle step failed: %d" % rc)
        self.step_count += 1
        return info

    def perplexity(self, mode="f64acc"):
        v = perplexity(self.K, self.pi, self.network.held_out, self.beta, self.p.epsilon,
                       self.ppx, self.average_count, mode)
        self.average_count += 1
        return v


class OracleSampler64(OracleSampler):
    """The same whole-iteration sampler in double arithmetic with the same
    draws: the FP64 trajectory reference of the FP32 and BF16 device paths."""

    def set_state(self, phi, theta):
        self.phi = np.ascontiguousarray(phi, np.float64).copy()
        self.theta = np.ascontiguousarray(theta, np.float64).copy()
        self.beta = self.theta[:, 1] / (self.theta[:, 0] + self.theta[:, 1])
        self.pi = normalize(self.phi, np.float64)
        self.ppx = np.zeros(self.network.held_out[0].shape[0], np.float64)

    def step(self):
        info = MbInfo()
        rc = lib().oracle_step_f64(ctypes.byref(self.p), ctypes.byref(self.og.g),
                                   ctypes.c_uint32(self.step_count), _p(self.pi), _p(self.phi),
                                   _p(self.theta), _p(self.beta), ctypes.byref(info))
        if rc != 0:
            raise RuntimeError("oracle step failed: %d" % rc)
        self.step_count += 1
        return info

    def perplexity(self, mode="f64"):
        v = perplexity(self.K, self.pi, self.network.held_out, self.beta, self.p.epsilon,
                       self.ppx, self.average_count, "f64")
        self.average_count += 1
        return v
