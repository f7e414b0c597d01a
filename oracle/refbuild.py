"""ctypes front end of the reference-built checker (oracle/_ref/libammsb_ref.so,
made by oracle/ref/build_ref.py from the reference sources).

TEST INFRASTRUCTURE ONLY: pins the oracle to the reference's own code and
times the reference's run() loop for bench.py's reference arm.
"""
import ctypes
import os
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libammsb_ref.so")

_lib = None


def available():
    return os.path.exists(LIB)


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(LIB)
        P = ctypes.c_void_p
        L.ref_last_error.restype = ctypes.c_char_p
        L.ref_create.restype = P
        L.ref_create.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)]
        L.ref_destroy.argtypes = [P]
        L.ref_sizes.argtypes = [P] + [ctypes.POINTER(ctypes.c_int64)] * 7
        L.ref_held_out.argtypes = [P, P, P, P]
        L.ref_test_set.argtypes = [P, P, P, P]
        L.ref_edges.restype = ctypes.c_int64
        L.ref_edges.argtypes = [P, P, P]
        L.ref_get_state.argtypes = [P, P, P, P, P]
        L.ref_set_state.argtypes = [P, P, P]
        L.ref_set_step.argtypes = [P, ctypes.c_uint64]
        L.ref_reseed.argtypes = [P, ctypes.c_uint32]
        L.ref_get_step.restype = ctypes.c_uint64
        L.ref_get_step.argtypes = [P]
        L.ref_eps_t.restype = ctypes.c_float
        L.ref_eps_t.argtypes = [P]
        L.ref_update_phi.argtypes = [P, ctypes.c_int32, P, ctypes.c_int32, ctypes.c_float, P, P, P]
        L.ref_update_beta.argtypes = [P, P, P, ctypes.c_int32, ctypes.c_float, P, P, P, P, P]
        L.ref_perplexity.restype = ctypes.c_float
        L.ref_perplexity.argtypes = [P, P]
        L.ref_sample_minibatch.argtypes = [P, P, P, ctypes.c_int32, P, P]
        L.ref_sample_neighbors.argtypes = [P, ctypes.c_int32, P]
        L.ref_run.argtypes = [P, ctypes.c_int64, ctypes.c_int64]
        _lib = L
    return _lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def write_relativity(path, edges):
    """Graph as the reference's relativity text: four header lines, then
    'a<TAB>b' per undirected edge."""
    with open(path, "w") as f:
        f.write("# Undirected graph\n# oracle fixture\n# Nodes Edges\n# FromNodeId\tToNodeId\n")
        for a, b in edges:
            f.write("%d\t%d\n" % (a, b))


class RefSampler:
    """The reference's MCMCSamplerStochastic built from its sources."""

    def __init__(self, edges, argv):
        self._dir = tempfile.mkdtemp(prefix="ammsb_ref_")
        path = os.path.join(self._dir, "graph.txt")
        write_relativity(path, edges)
        args = ["ref", "--mcmc.input.file", path, "--mcmc.input.class", "relativity",
                "--mcmc.input.contiguous"] + list(argv)
        arr = (ctypes.c_char_p * len(args))(*[a.encode() for a in args])
        h = lib().ref_create(len(args), arr)
        if not h:
            raise RuntimeError("reference init failed: %s" % lib().ref_last_error().decode())
        self.h = h
        v = [ctypes.c_int64() for _ in range(7)]
        lib().ref_sizes(h, *[ctypes.byref(x) for x in v])
        self.N, self.K, self.E, self.H, self.T, self.nns, self.mbs = (x.value for x in v)

    def close(self):
        if getattr(self, "h", None):
            lib().ref_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _set(self, fn, n):
        a = np.zeros(n, np.int32)
        b = np.zeros(n, np.int32)
        y = np.zeros(n, np.uint8)
        fn(self.h, _p(a), _p(b), _p(y))
        return a, b, y

    def held_out(self):
        return self._set(lib().ref_held_out, self.H)

    def test_set(self):
        return self._set(lib().ref_test_set, self.T)

    def edges(self):
        a = np.zeros(self.E, np.int32)
        b = np.zeros(self.E, np.int32)
        n = lib().ref_edges(self.h, _p(a), _p(b))
        return a[:n], b[:n]

    def state(self):
        phi = np.zeros((self.N, self.K), np.float32)
        pi = np.zeros((self.N, self.K), np.float32)
        th = np.zeros((self.K, 2), np.float32)
        bt = np.zeros(self.K, np.float32)
        lib().ref_get_state(self.h, _p(phi), _p(pi), _p(th), _p(bt))
        return phi, pi, th, bt

    def set_state(self, phi, theta):
        phi = np.ascontiguousarray(phi, np.float32)
        theta = np.ascontiguousarray(theta, np.float32)
        lib().ref_set_state(self.h, _p(phi), _p(theta))

    def set_step(self, s):
        lib().ref_set_step(self.h, s)

    def reseed(self, s):
        """A fresh random stream for the draws from here on."""
        lib().ref_reseed(self.h, s)

    @property
    def step(self):
        return lib().ref_get_step(self.h)

    def eps_t(self):
        return lib().ref_eps_t(self.h)

    def update_phi(self, node, nbrs, eps):
        nbrs = np.ascontiguousarray(nbrs, np.int32)
        order = np.zeros_like(nbrs)
        noise = np.zeros(self.K, np.float32)
        out = np.zeros(self.K, np.float32)
        rc = lib().ref_update_phi(self.h, int(node), _p(nbrs), nbrs.shape[0], eps, _p(order),
                                  _p(noise), _p(out))
        if rc:
            raise RuntimeError(lib().ref_last_error().decode())
        return order, noise, out

    def update_beta(self, ea, eb, scale):
        ea = np.ascontiguousarray(ea, np.int32)
        eb = np.ascontiguousarray(eb, np.int32)
        oa = np.zeros_like(ea)
        ob = np.zeros_like(eb)
        noise = np.zeros((self.K, 2), np.float32)
        th = np.zeros((self.K, 2), np.float32)
        bt = np.zeros(self.K, np.float32)
        rc = lib().ref_update_beta(self.h, _p(ea), _p(eb), ea.shape[0], scale, _p(oa), _p(ob),
                                   _p(noise), _p(th), _p(bt))
        if rc:
            raise RuntimeError(lib().ref_last_error().decode())
        n = len(set(zip(np.minimum(ea, eb).tolist(), np.maximum(ea, eb).tolist())))
        return oa[:n], ob[:n], noise, th, bt

    def perplexity(self):
        ppx = np.zeros(self.H, np.float32)
        v = lib().ref_perplexity(self.h, _p(ppx))
        return v, ppx

    def sample_minibatch(self, cap):
        ea = np.zeros(cap, np.int32)
        eb = np.zeros(cap, np.int32)
        n = ctypes.c_int32()
        sc = ctypes.c_float()
        rc = lib().ref_sample_minibatch(self.h, _p(ea), _p(eb), cap, ctypes.byref(n),
                                        ctypes.byref(sc))
        if rc:
            raise RuntimeError("reference minibatch failed: %d" % rc)
        return ea[:n.value], eb[:n.value], sc.value

    def sample_neighbors(self, node):
        out = np.zeros(self.nns + 1, np.int32)
        rc = lib().ref_sample_neighbors(self.h, int(node), _p(out))
        if rc:
            raise RuntimeError(lib().ref_last_error().decode())
        return out

    def run(self, n, interval=0):
        rc = lib().ref_run(self.h, n, interval)
        if rc:
            raise RuntimeError(lib().ref_last_error().decode())
