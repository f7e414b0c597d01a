"""Graph, held-out and test sets (the data side of mcmc::Network,
network.h:59-341), prepared by the native host code of libammsb_gpu.so.

``Network`` owns a symmetric CSR graph (sorted rows) and the held-out and
test edge sets as arrays.  Graphs come from the synthetic planted-community
generator, an edge list, or a relativity/SNAP text file
(preprocess/relativity.cc:20-200).
"""
import ctypes

import numpy as np

from . import _native


def _as_np(ptr, n, dtype):
    if n == 0:
        return np.zeros(0, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


class Network:
    def __init__(self, row_ptr, col, held_out=None, test=None, _buf=None):
        self.row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int64)
        self.col = np.ascontiguousarray(col, dtype=np.int32)
        self.N = int(self.row_ptr.shape[0] - 1)
        z = (np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros(0, np.uint8))
        self.held_out = held_out if held_out is not None else z
        self.test = test if test is not None else z
        self._buf = _buf  # native ammsb_graph_buf owning the same CSR, if any

    def __del__(self):
        buf, self._buf = getattr(self, "_buf", None), None
        if buf is not None:
            try:
                _native.lib().ammsb_graph_free(buf)
            except Exception:
                pass

    # -- construction -----------------------------------------------------
    @staticmethod
    def _from_buf(buf):
        """Network over a native graph buffer (takes ownership of it)."""
        L = _native.lib()
        view = _native.AmmsbGraph()
        L.ammsb_graph_view(buf, ctypes.byref(view))
        n = view.n
        row_ptr = _as_np(view.row_ptr, n + 1, np.int64)
        col = _as_np(view.col, int(row_ptr[-1]), np.int32)
        return Network(row_ptr, col, _buf=buf)

    @staticmethod
    def synthetic(n, k_true, size_min=10, size_max=500, zipf_s=1.5, p1=0.7, p2=0.25,
                  intra_degree=4.0, background_frac=0.1, seed=0):
        """Planted-community graph (see ammsb_generate_graph)."""
        L = _native.lib()
        p = _native.AmmsbGenParams(n, k_true, zipf_s, size_min, size_max, p1, p2,
                                   intra_degree, background_frac, seed)
        buf = ctypes.c_void_p()
        _native.check(L.ammsb_generate_graph(ctypes.byref(p), ctypes.byref(buf)))
        return Network._from_buf(buf)

    @staticmethod
    def from_edges(n, a, b):
        L = _native.lib()
        a = np.ascontiguousarray(a, dtype=np.int32)
        b = np.ascontiguousarray(b, dtype=np.int32)
        buf = ctypes.c_void_p()
        _native.check(L.ammsb_graph_from_edges(
            n, a.shape[0], a.ctypes.data_as(_native._I32P), b.ctypes.data_as(_native._I32P),
            ctypes.byref(buf)))
        return Network._from_buf(buf)

    @staticmethod
    def from_relativity(path, contiguous=False):
        L = _native.lib()
        buf = ctypes.c_void_p()
        _native.check(L.ammsb_read_relativity(path.encode(), int(bool(contiguous)),
                                              ctypes.byref(buf)))
        return Network._from_buf(buf)

    @staticmethod
    def load_preprocessed(dirname):
        """A network saved by save_preprocessed (the reference's input class
        "preprocessed", network.cc:49-65): graph, held-out and test sets;
        the held-out ratio it was drawn with is `held_out_ratio`."""
        L = _native.lib()
        g = ctypes.c_void_p()
        sp = ctypes.c_void_p()
        ratio = ctypes.c_double()
        _native.check(L.ammsb_load_preprocessed(str(dirname).encode(), ctypes.byref(g),
                                                ctypes.byref(sp), ctypes.byref(ratio)))
        net = Network._from_buf(g)
        try:
            h = _native.AmmsbEdgeSet()
            t = _native.AmmsbEdgeSet()
            L.ammsb_split_view(sp, ctypes.byref(h), ctypes.byref(t))
            net.held_out = (_as_np(h.a, h.count, np.int32), _as_np(h.b, h.count, np.int32),
                            _as_np(h.y, h.count, np.uint8))
            net.test = (_as_np(t.a, t.count, np.int32), _as_np(t.b, t.count, np.int32),
                        _as_np(t.y, t.count, np.uint8))
        finally:
            L.ammsb_split_free(sp)
        net.held_out_ratio = ratio.value
        return net

    def save_preprocessed(self, dirname, held_out_ratio=None):
        """Network::save (network.cc:136-145): the graph, the held-out and
        test sets and the auxiliary data into directory `dirname` (see
        ammsb_save_preprocessed)."""
        ratio = held_out_ratio if held_out_ratio is not None else getattr(self, "held_out_ratio",
                                                                          0.0)
        ho, _keep_h = Network.native_edge_set(self.held_out)
        te, _keep_t = Network.native_edge_set(self.test)
        g = self.native_graph()
        _native.check(_native.lib().ammsb_save_preprocessed(
            ctypes.byref(g), ctypes.byref(ho), ctypes.byref(te), float(ratio),
            str(dirname).encode()))

    def _with_buf(self, fn):
        """Run fn(graph_buf) on the native graph (built from the CSR if this
        Network was not made by the native library)."""
        L = _native.lib()
        if self._buf is not None:
            return fn(self._buf)
        und = self.undirected_edges()
        buf = ctypes.c_void_p()
        a = np.ascontiguousarray(und[:, 0])
        b = np.ascontiguousarray(und[:, 1])
        _native.check(L.ammsb_graph_from_edges(
            self.N, a.shape[0], a.ctypes.data_as(_native._I32P), b.ctypes.data_as(_native._I32P),
            ctypes.byref(buf)))
        try:
            return fn(buf)
        finally:
            L.ammsb_graph_free(buf)

    def write_relativity(self, path):
        L = _native.lib()
        self._with_buf(lambda buf: _native.check(L.ammsb_write_relativity(buf, path.encode())))

    def make_held_out(self, held_out_ratio, seed=0):
        """network.cc:503-614 (see ammsb_make_held_out); sets held_out, test."""
        L = _native.lib()
        self.held_out_ratio = held_out_ratio

        def run(buf):
            sp = ctypes.c_void_p()
            _native.check(L.ammsb_make_held_out(buf, held_out_ratio, seed, ctypes.byref(sp)))
            try:
                h = _native.AmmsbEdgeSet()
                t = _native.AmmsbEdgeSet()
                L.ammsb_split_view(sp, ctypes.byref(h), ctypes.byref(t))
                self.held_out = (_as_np(h.a, h.count, np.int32), _as_np(h.b, h.count, np.int32),
                                 _as_np(h.y, h.count, np.uint8))
                self.test = (_as_np(t.a, t.count, np.int32), _as_np(t.b, t.count, np.int32),
                             _as_np(t.y, t.count, np.uint8))
            finally:
                L.ammsb_split_free(sp)

        self._with_buf(run)
        return self

    # -- queries ------------------------------------------------------------
    @property
    def num_total_edges(self):
        """Undirected edges of the full graph (network.cc:68)."""
        return int(self.row_ptr[-1]) // 2

    def max_degree(self):
        return int(np.max(np.diff(self.row_ptr))) if self.N else 0

    def undirected_edges(self):
        src = np.repeat(np.arange(self.N, dtype=np.int32), np.diff(self.row_ptr))
        m = self.col > src
        return np.stack([src[m], self.col[m]], axis=1)

    def excluded_keys(self):
        """Sorted keys (min << 32 | max) of the held-out and test pairs."""
        a = np.concatenate([self.held_out[0], self.test[0]]).astype(np.uint64)
        b = np.concatenate([self.held_out[1], self.test[1]]).astype(np.uint64)
        lo = np.minimum(a, b)
        hi = np.maximum(a, b)
        return np.unique((lo << np.uint64(32)) | hi)

    # -- native views ----------------------------------------------------------
    def native_graph(self):
        g = _native.AmmsbGraph()
        g.n = self.N
        g.row_ptr = self.row_ptr.ctypes.data_as(_native._I64P)
        g.col = self.col.ctypes.data_as(_native._I32P)
        return g

    @staticmethod
    def native_edge_set(s):
        a, b, y = (np.ascontiguousarray(s[0], np.int32), np.ascontiguousarray(s[1], np.int32),
                   np.ascontiguousarray(s[2], np.uint8))
        e = _native.AmmsbEdgeSet()
        e.count = a.shape[0]
        e.a = a.ctypes.data_as(_native._I32P)
        e.b = b.ctypes.data_as(_native._I32P)
        e.y = y.ctypes.data_as(_native._U8P)
        return e, (a, b, y)
