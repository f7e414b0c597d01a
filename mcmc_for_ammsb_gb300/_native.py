"""ctypes declarations of the C ABI in include/ammsb_gpu.h.

The product path is the native library; there is no Python or CPU fallback.
If libammsb_gpu.so has not been built, importing this module raises.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libammsb_gpu.so")

AMMSB_OK = 0
ERRORS = {
    -1: "invalid argument",
    -2: "CUDA error",
    -3: "sampling loop cap reached",
    -4: "minibatch exceeds buffer",
    -5: "state / call order error",
    -6: "unsupported option",
}

STRATIFIED_RANDOM_NODE = 0
STRATIFIED_RANDOM_NODE_LINKS = 1
STRATIFIED_RANDOM_NODE_NONLINKS = 2
RANDOM_EDGE = 3

PI_F32 = 0
PI_BF16 = 1

REAL_F32 = 0
REAL_F64 = 1

TUNE_FRESH = 1


class AmmsbOptions(ctypes.Structure):
    _fields_ = [
        ("alpha", ctypes.c_double),
        ("eta0", ctypes.c_double),
        ("eta1", ctypes.c_double),
        ("epsilon", ctypes.c_double),
        ("a", ctypes.c_double),
        ("b", ctypes.c_double),
        ("c", ctypes.c_double),
        ("K", ctypes.c_int64),
        ("mini_batch_size", ctypes.c_int64),
        ("num_node_sample", ctypes.c_int64),
        ("strategy", ctypes.c_int32),
        ("sampler_max_source", ctypes.c_int64),
        ("max_iteration", ctypes.c_int64),
        ("interval", ctypes.c_int64),
        ("stats_print_interval", ctypes.c_int64),
        ("num_updates", ctypes.c_int64),
        ("held_out_ratio", ctypes.c_double),
        ("random_seed", ctypes.c_int32),
        ("convergence_threshold", ctypes.c_double),
        ("pi_dtype", ctypes.c_int32),
        ("chain", ctypes.c_int32),
        ("device", ctypes.c_int32),
        ("use_graph", ctypes.c_int32),
        ("verbose", ctypes.c_int32),
        ("pipeline", ctypes.c_int32),
    ]


class AmmsbGraph(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int64),
        ("row_ptr", ctypes.POINTER(ctypes.c_int64)),
        ("col", ctypes.POINTER(ctypes.c_int32)),
    ]


class AmmsbEdgeSet(ctypes.Structure):
    _fields_ = [
        ("count", ctypes.c_int64),
        ("a", ctypes.POINTER(ctypes.c_int32)),
        ("b", ctypes.POINTER(ctypes.c_int32)),
        ("y", ctypes.POINTER(ctypes.c_uint8)),
    ]


class AmmsbGenParams(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int64),
        ("k_true", ctypes.c_int64),
        ("zipf_s", ctypes.c_double),
        ("size_min", ctypes.c_int64),
        ("size_max", ctypes.c_int64),
        ("p1", ctypes.c_double),
        ("p2", ctypes.c_double),
        ("intra_degree", ctypes.c_double),
        ("background_frac", ctypes.c_double),
        ("seed", ctypes.c_uint32),
    ]


# (name, restype, argtypes) of every exported entry point
_P = ctypes.c_void_p
_I32P = ctypes.POINTER(ctypes.c_int32)
_I64P = ctypes.POINTER(ctypes.c_int64)
_U8P = ctypes.POINTER(ctypes.c_uint8)
_F32P = ctypes.POINTER(ctypes.c_float)
_F64P = ctypes.POINTER(ctypes.c_double)
_U64P = ctypes.POINTER(ctypes.c_uint64)

SIGNATURES = [
    ("ammsb_options_default", None, [ctypes.POINTER(AmmsbOptions)]),
    ("ammsb_create", ctypes.c_int, [ctypes.POINTER(AmmsbOptions), ctypes.POINTER(AmmsbGraph),
                                    ctypes.POINTER(AmmsbEdgeSet), ctypes.POINTER(AmmsbEdgeSet),
                                    ctypes.POINTER(_P)]),
    ("ammsb_destroy", None, [_P]),
    ("ammsb_last_error", ctypes.c_char_p, [_P]),
    ("ammsb_create_error", ctypes.c_char_p, []),
    ("ammsb_init_state", ctypes.c_int, [_P]),
    ("ammsb_set_state", ctypes.c_int, [_P, _F32P, _F64P]),
    ("ammsb_step", ctypes.c_int, [_P, ctypes.c_int64]),
    ("ammsb_step_fed", ctypes.c_int, [_P, ctypes.c_uint32, ctypes.c_int32, _I32P, _I32P, _U8P,
                                      ctypes.c_float, ctypes.c_int32, _I32P, _I32P, _U8P, _F32P,
                                      _F32P]),
    ("ammsb_perplexity", ctypes.c_int, [_P, _F64P]),
    ("ammsb_run", ctypes.c_int, [_P, _F64P]),
    ("ammsb_get_pi", ctypes.c_int, [_P, _F32P]),
    ("ammsb_get_phi", ctypes.c_int, [_P, _F32P]),
    ("ammsb_get_theta", ctypes.c_int, [_P, _F64P]),
    ("ammsb_get_beta", ctypes.c_int, [_P, _F32P]),
    ("ammsb_get_ppx", ctypes.c_int, [_P, _F32P]),
    ("ammsb_get_step", ctypes.c_int, [_P, _U64P, _U64P]),
    ("ammsb_set_step", ctypes.c_int, [_P, ctypes.c_uint64]),
    ("ammsb_get_last_minibatch", ctypes.c_int, [_P, _I32P, _I32P, _I32P, _F32P, _I32P, _I32P,
                                                _U8P, _I32P, _I32P, _U8P]),
    ("ammsb_get_sizes", ctypes.c_int, [_P, _I64P, _I64P, _I64P, _I64P, _I64P, _I64P]),
    ("ammsb_get_options", ctypes.c_int, [_P, ctypes.POINTER(AmmsbOptions)]),
    ("ammsb_profile_step", ctypes.c_int, [_P, _F64P]),
    ("ammsb_stream", _P, [_P]),
    ("ammsb_get_counters", ctypes.c_int, [_P, _U64P, _U64P]),
    ("ammsb_autotune", ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int32]),
    ("ammsb_get_kernel_config", ctypes.c_int, [_P, _I32P]),
    ("ammsb_batch_create", ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int32, ctypes.POINTER(_P)]),
    ("ammsb_batch_destroy", None, [_P]),
    ("ammsb_batch_step", ctypes.c_int, [_P, ctypes.c_int64]),
    ("ammsb_batch_groups", ctypes.c_int32, [_P]),
    ("ammsb_batch_stream", _P, [_P]),
    ("ammsb_batch_last_error", ctypes.c_char_p, [_P]),
    ("ammsb_batch_create_error", ctypes.c_char_p, []),
    ("ammsb_save_checkpoint", ctypes.c_int, [_P, ctypes.c_char_p]),
    ("ammsb_load_checkpoint", ctypes.c_int, [_P, ctypes.c_char_p]),
    ("ammsb_perplexity_noalloc", ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int64, ctypes.c_int64,
                                                ctypes.c_int64, _P, ctypes.c_double, _P, _P, _P,
                                                ctypes.c_int64, _P, ctypes.c_uint64, _P, _F64P]),
    ("ammsb_edge_loglik_workspace_size", ctypes.c_size_t, [ctypes.c_int32, ctypes.c_int64,
                                                          ctypes.c_int64, ctypes.c_int64]),
    ("ammsb_edge_loglik_forward", ctypes.c_int,
     [ctypes.c_int32, ctypes.c_int64, _P, ctypes.c_int64, _P, ctypes.c_int64, ctypes.c_int64, _P,
      ctypes.c_double, _P, ctypes.c_int64, _P, _P, ctypes.c_int64, _P, _P, _P]),
    ("ammsb_edge_loglik_backward", ctypes.c_int,
     [ctypes.c_int32, ctypes.c_int64, _P, ctypes.c_int64, _P, ctypes.c_int64, ctypes.c_int64, _P,
      ctypes.c_double, _P, ctypes.c_int64, _P, _P, ctypes.c_int64, _P, _P, _P, _P, _P, _P, _P, _P,
      _P]),
    ("ammsb_edge_loglik_status", ctypes.c_int, [_P, _P, _I32P]),
    ("ammsb_generate_graph", ctypes.c_int, [ctypes.POINTER(AmmsbGenParams), ctypes.POINTER(_P)]),
    ("ammsb_graph_from_edges", ctypes.c_int, [ctypes.c_int64, ctypes.c_int64, _I32P, _I32P,
                                              ctypes.POINTER(_P)]),
    ("ammsb_read_relativity", ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(_P)]),
    ("ammsb_write_relativity", ctypes.c_int, [_P, ctypes.c_char_p]),
    ("ammsb_graph_view", None, [_P, ctypes.POINTER(AmmsbGraph)]),
    ("ammsb_graph_free", None, [_P]),
    ("ammsb_make_held_out", ctypes.c_int, [_P, ctypes.c_double, ctypes.c_uint32,
                                           ctypes.POINTER(_P)]),
    ("ammsb_split_view", None, [_P, ctypes.POINTER(AmmsbEdgeSet), ctypes.POINTER(AmmsbEdgeSet)]),
    ("ammsb_split_free", None, [_P]),
    ("ammsb_shard_draw", ctypes.c_int, [_P]),
    ("ammsb_shard_update", ctypes.c_int, [_P, ctypes.c_int32, _I32P, _F32P]),
    ("ammsb_shard_commit", ctypes.c_int, [_P, _F32P, ctypes.c_int32, _I32P, _F64P]),
    ("ammsb_shard_theta", ctypes.c_int, [_P, _F64P]),
    ("ammsb_save_preprocessed", ctypes.c_int, [ctypes.POINTER(AmmsbGraph),
                                               ctypes.POINTER(AmmsbEdgeSet),
                                               ctypes.POINTER(AmmsbEdgeSet), ctypes.c_double,
                                               ctypes.c_char_p]),
    ("ammsb_load_preprocessed", ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_P),
                                               ctypes.POINTER(_P),
                                               ctypes.POINTER(ctypes.c_double)]),
]


class AmmsbError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "error"), code, msg))
        self.code = code


_lib = None


def lib():
    """The loaded native library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                "libammsb_gpu.so is not built (%s); run "
                "`python -c 'import __graft_entry__ as g; g.build()'`" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(code, handle=None):
    if code != AMMSB_OK:
        if handle is not None:
            msg = lib().ammsb_last_error(handle)
        else:
            msg = lib().ammsb_create_error()
        raise AmmsbError(code, (msg or b"").decode())
    return code
