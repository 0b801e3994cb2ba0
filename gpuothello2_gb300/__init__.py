"""GB300 batched exact Othello endgame solver -- Python bindings.

Thin ctypes layer over the C ABI in include/gpuothello2.h
(lib/libgpuothello2.so, built in-tree by gpuothello2_gb300.build).  The
product is the native library and the C++ CLI; these bindings exist for
tests, benchmarks and Python callers.  There is no fallback: if the library
is missing, `lib()` raises.
"""
import ctypes
import os

import numpy as np

from . import build as _build

GPO_OK = 0
GPO_ERR_ARG = -1
GPO_ERR_DEPTH = -2
GPO_ERR_BOARD = -3
GPO_ERR_CUDA = -4
GPO_ERR_NOMEM = -5
GPO_ERR_TIMEOUT = -6
GPO_ERR_INTERNAL = -7
GPO_ERR_IO = -8
MOVE_PASS = 64
MOVE_NONE = 65
METHOD_BATCHED = 0
METHOD_PLAIN = 1

EXPORTED_SYMBOLS = (
    "gpo_default_options", "solve_batch", "solve_batch_ex", "solve_batch_device",
    "gpo_generate", "gpo_generate_device", "solve_shutdown", "gpo_strerror",
    "gpo_device_info", "solve_batch_device_noalloc", "gpo_mlp_param_count", "gpo_mlp_init",
    "gpo_mlp_forward", "gpo_mlp_gradients", "gpo_mlp_train", "gpo_mlp_load",
    "gpo_eval_load", "gpo_eval_load_files", "gpo_evaluate", "think_batch",
    "gpo_graph_create", "gpo_graph_launch", "gpo_graph_stats", "gpo_graph_destroy",
)


class Options(ctypes.Structure):
    _fields_ = [
        ("method", ctypes.c_int),
        ("use_table", ctypes.c_int),
        ("use_learned", ctypes.c_int),
        ("threads_per_block", ctypes.c_int),
        ("fastest_first_empties", ctypes.c_int),
        ("learned_min_empties", ctypes.c_int),
        ("node_budget", ctypes.c_uint64),
        ("help_min_empties", ctypes.c_int),
        ("wait_limit_ms", ctypes.c_int),
        ("table_bits", ctypes.c_int),
        ("table_min_empties", ctypes.c_int),
        ("smem_frames", ctypes.c_int),
        ("stability_min_empties", ctypes.c_int),
        ("roots_per_warp", ctypes.c_int),
        ("hard_nodes", ctypes.c_int64),
        ("root_split_plies", ctypes.c_int),
        ("tail_split_positions", ctypes.c_int),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("nodes", ctypes.c_uint64),
        ("table_probes", ctypes.c_uint64),
        ("table_hits", ctypes.c_uint64),
        ("table_updates", ctypes.c_uint64),
        ("learned_calls", ctypes.c_uint64),
        ("splits", ctypes.c_uint64),
        ("kernel_ms", ctypes.c_double),
        ("total_ms", ctypes.c_double),
        ("launches", ctypes.c_uint64),
        ("stability_cuts", ctypes.c_uint64),
        ("table_bits", ctypes.c_uint64),
        ("root_split_positions", ctypes.c_uint64),
        ("tail_positions", ctypes.c_uint64),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class SolverError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        super().__init__("%s: %s (status %d)" % (what or "gpuothello2", strerror(status), status))


_lib = None


def lib():
    """The loaded native library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(_build.LIB):
            raise RuntimeError("native library missing: %s (run gpuothello2_gb300.build)" % _build.LIB)
        L = ctypes.CDLL(_build.LIB)
        vp, i, u64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64
        L.gpo_default_options.argtypes = [ctypes.POINTER(Options)]
        L.gpo_default_options.restype = None
        L.solve_batch.argtypes = [vp, vp, i, i, vp]
        L.solve_batch_ex.argtypes = [vp, vp, i, i, vp, vp, vp, ctypes.POINTER(Options),
                                     ctypes.POINTER(Stats)]
        L.solve_batch_device.argtypes = [vp, vp, i, i, vp, vp, vp, ctypes.POINTER(Options),
                                         ctypes.POINTER(Stats), vp]
        L.gpo_generate.argtypes = [u64, u64, i, i, i, vp, vp]
        L.gpo_generate_device.argtypes = [u64, u64, i, i, i, vp, vp, vp]
        L.solve_shutdown.argtypes = []
        L.solve_shutdown.restype = None
        L.gpo_strerror.argtypes = [i]
        L.gpo_strerror.restype = ctypes.c_char_p
        L.gpo_device_info.argtypes = [ctypes.c_char_p, i, ctypes.POINTER(ctypes.c_int)]
        L.solve_batch_device_noalloc.argtypes = [vp, vp, i, i, vp, vp]
        f32 = ctypes.c_float
        L.gpo_mlp_param_count.argtypes = []
        L.gpo_mlp_init.argtypes = [u64, vp]
        L.gpo_mlp_forward.argtypes = [vp, vp, vp, i, vp]
        L.gpo_mlp_gradients.argtypes = [vp, vp, vp, vp, i, vp, ctypes.POINTER(f32)]
        L.gpo_mlp_train.argtypes = [vp, vp, vp, i, i, i, f32, u64, vp, vp]
        L.gpo_mlp_load.argtypes = [vp]
        L.gpo_eval_load.argtypes = [vp, i, vp, ctypes.c_double]
        L.gpo_eval_load_files.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
        L.gpo_evaluate.argtypes = [vp, vp, i, vp]
        L.think_batch.argtypes = [vp, vp, i, i, vp, vp, vp, ctypes.POINTER(Stats)]
        L.gpo_graph_create.argtypes = [vp, vp, i, i, vp, ctypes.POINTER(Options),
                                       ctypes.POINTER(vp)]
        L.gpo_graph_launch.argtypes = [vp, vp]
        L.gpo_graph_stats.argtypes = [vp, ctypes.POINTER(Stats)]
        L.gpo_graph_destroy.argtypes = [vp]
        L.gpo_graph_destroy.restype = None
        _lib = L
    return _lib


def strerror(status):
    try:
        return lib().gpo_strerror(status).decode()
    except RuntimeError:
        return "status %d" % status


def options(**kw):
    o = Options()
    lib().gpo_default_options(ctypes.byref(o))
    for k, v in kw.items():
        if v is not None:
            setattr(o, k, v)
    return o


def _u64(a):
    return np.ascontiguousarray(a, dtype=np.uint64)


def solve(player, opp, depth, method=None, best=False, nodes=False, check=True, **opts):
    """Exact-solves positions through solve_batch_ex.  Returns (score,
    best_or_None, nodes_or_None, stats, status)."""
    p, o = _u64(player), _u64(opp)
    n = len(p)
    score = np.zeros(n, np.int8)
    bm = np.zeros(n, np.int8) if best else None
    nd = np.zeros(n, np.uint64) if nodes else None
    if method is not None:
        opts["method"] = method
    opt = options(**opts)
    st = Stats()
    rc = lib().solve_batch_ex(p.ctypes.data, o.ctypes.data, n, depth, score.ctypes.data,
                              bm.ctypes.data if bm is not None else None,
                              nd.ctypes.data if nd is not None else None,
                              ctypes.byref(opt), ctypes.byref(st))
    if check and rc != GPO_OK:
        raise SolverError(rc, "solve_batch_ex")
    return score, bm, nd, st, rc


def solve_batch(player, opp, depth):
    """The plain C entry point solve_batch(player, opp, n, depth, score)."""
    p, o = _u64(player), _u64(opp)
    score = np.zeros(len(p), np.int8)
    rc = lib().solve_batch(p.ctypes.data, o.ctypes.data, len(p), depth, score.ctypes.data)
    if rc != GPO_OK:
        raise SolverError(rc, "solve_batch")
    return score


def generate(seed, n, min_empties, max_empties=None, first=0):
    """n positions of the seeded random-playout stream, generated on the GPU."""
    hi = min_empties if max_empties is None else max_empties
    p = np.zeros(n, np.uint64)
    o = np.zeros(n, np.uint64)
    rc = lib().gpo_generate(seed, first, n, min_empties, hi, p.ctypes.data, o.ctypes.data)
    if rc != GPO_OK:
        raise SolverError(rc, "gpo_generate")
    return p, o


def device_info():
    buf = ctypes.create_string_buffer(256)
    sms = ctypes.c_int(0)
    rc = lib().gpo_device_info(buf, 256, ctypes.byref(sms))
    if rc != GPO_OK:
        raise SolverError(rc, "gpo_device_info")
    return buf.value.decode(), sms.value


def shutdown():
    lib().solve_shutdown()


# ---- learned move orderer (mlp.cu) ----
def mlp_init(seed):
    w = np.zeros(lib().gpo_mlp_param_count(), np.float32)
    rc = lib().gpo_mlp_init(seed, w.ctypes.data)
    if rc != GPO_OK:
        raise SolverError(rc, "gpo_mlp_init")
    return w


def mlp_forward(w, player, opp):
    p, o = _u64(player), _u64(opp)
    z = np.zeros((len(p), 64), np.float32)
    w = np.ascontiguousarray(w, np.float32)
    rc = lib().gpo_mlp_forward(w.ctypes.data, p.ctypes.data, o.ctypes.data, len(p), z.ctypes.data)
    if rc != GPO_OK:
        raise SolverError(rc, "gpo_mlp_forward")
    return z


def mlp_gradients(w, player, opp, best):
    p, o = _u64(player), _u64(opp)
    b = np.ascontiguousarray(best, np.int8)
    w = np.ascontiguousarray(w, np.float32)
    g = np.zeros_like(w)
    loss = ctypes.c_float(0.0)
    rc = lib().gpo_mlp_gradients(w.ctypes.data, p.ctypes.data, o.ctypes.data, b.ctypes.data, len(p),
                                 g.ctypes.data, ctypes.byref(loss))
    if rc != GPO_OK:
        raise SolverError(rc, "gpo_mlp_gradients")
    return g, loss.value


def mlp_train(player, opp, best, w, epochs=3, batch=4096, lr=1e-3, seed=0):
    """Trains in place on a copy of w; returns (weights, [(loss, accuracy)] per epoch)."""
    p, o = _u64(player), _u64(opp)
    b = np.ascontiguousarray(best, np.int8)
    w = np.array(w, np.float32)
    hist = np.zeros(2 * epochs, np.float32)
    rc = lib().gpo_mlp_train(p.ctypes.data, o.ctypes.data, b.ctypes.data, len(p), epochs, batch,
                             lr, seed, w.ctypes.data, hist.ctypes.data)
    if rc != GPO_OK:
        raise SolverError(rc, "gpo_mlp_train")
    return w, [(float(hist[2 * e]), float(hist[2 * e + 1])) for e in range(epochs)]


def mlp_load(w):
    """Loads weights for the solver's learned root ordering (None unloads)."""
    if w is None:
        rc = lib().gpo_mlp_load(None)
    else:
        w = np.ascontiguousarray(w, np.float32)
        rc = lib().gpo_mlp_load(w.ctypes.data)
    if rc != GPO_OK:
        raise SolverError(rc, "gpo_mlp_load")


def eval_load(features, values, offset):
    """Loads the think-mode pattern evaluator: square masks, every feature's
    table (3^k values) in order, and the offset."""
    f = np.ascontiguousarray(features, np.uint64)
    v = np.ascontiguousarray(values, np.float64)
    rc = lib().gpo_eval_load(f.ctypes.data, len(f), v.ctypes.data, float(offset))
    if rc != GPO_OK:
        raise SolverError(rc, "gpo_eval_load")


def eval_load_files(features_path, values_path):
    """Loads the evaluator from the reference's feature and value files."""
    rc = lib().gpo_eval_load_files(os.fsencode(features_path), os.fsencode(values_path))
    if rc != GPO_OK:
        raise SolverError(rc, "gpo_eval_load_files")


def evaluate(player, opp):
    p, o = _u64(player), _u64(opp)
    out = np.zeros(len(p), np.float32)
    rc = lib().gpo_evaluate(p.ctypes.data, o.ctypes.data, len(p), out.ctypes.data)
    if rc != GPO_OK:
        raise SolverError(rc, "gpo_evaluate")
    return out


def think(player, opp, depth, check=True):
    """Think mode through think_batch.  Returns (score, best move, nodes,
    stats, status)."""
    p, o = _u64(player), _u64(opp)
    n = len(p)
    score = np.zeros(n, np.int8)
    best = np.zeros(n, np.int8)
    nodes = np.zeros(n, np.uint64)
    st = Stats()
    rc = lib().think_batch(p.ctypes.data, o.ctypes.data, n, depth, score.ctypes.data,
                           best.ctypes.data, nodes.ctypes.data, ctypes.byref(st))
    if check and rc != GPO_OK:
        raise SolverError(rc, "think_batch")
    return score, best, nodes, st, rc
