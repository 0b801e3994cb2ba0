"""ctypes wrapper of the CPU oracle (oracle/oracle.c) -- the checker only."""
import ctypes

import numpy as np

u64 = ctypes.c_uint64


class Oracle:
    def __init__(self, path):
        L = ctypes.CDLL(path)
        vp, i = ctypes.c_void_p, ctypes.c_int
        L.orc_flip.restype = u64
        L.orc_flip.argtypes = [u64, u64, i]
        L.orc_flip_naive.restype = u64
        L.orc_flip_naive.argtypes = [u64, u64, i]
        L.orc_mobility.restype = u64
        L.orc_mobility.argtypes = [u64, u64]
        L.orc_mobility_naive.restype = u64
        L.orc_mobility_naive.argtypes = [u64, u64]
        L.orc_final_score.argtypes = [u64, u64]
        L.orc_encode.argtypes = [u64, u64, ctypes.c_char_p]
        L.orc_decode.argtypes = [ctypes.c_char_p, ctypes.POINTER(u64), ctypes.POINTER(u64)]
        L.orc_generate.argtypes = [u64, u64, i, i, i, vp, vp]
        L.orc_solve_ref.argtypes = [u64, u64, i, ctypes.POINTER(u64), ctypes.POINTER(u64)]
        L.orc_solve_fast.argtypes = [u64, u64, ctypes.POINTER(u64), ctypes.POINTER(ctypes.c_int)]
        L.orc_solve_batch.argtypes = [vp, vp, i, i, i, i, vp, vp, vp, vp]
        L.orc_eval_create.argtypes = [vp, i, vp, ctypes.c_double]
        L.orc_eval_create.restype = vp
        L.orc_eval_free.argtypes = [vp]
        L.orc_eval_free.restype = None
        L.orc_eval.argtypes = [vp, u64, u64]
        L.orc_eval.restype = ctypes.c_float
        L.orc_think_batch.argtypes = [vp, vp, vp, i, i, i, vp, vp, vp, vp]
        self.L = L

    def generate(self, seed, n, lo, hi=None, first=0):
        p = np.zeros(n, np.uint64)
        o = np.zeros(n, np.uint64)
        self.L.orc_generate(seed, first, n, lo, lo if hi is None else hi, p.ctypes.data,
                            o.ctypes.data)
        return p, o

    def encode(self, p, o):
        buf = ctypes.create_string_buffer(17)
        self.L.orc_encode(int(p), int(o), buf)
        return buf.value.decode("latin-1")

    def decode(self, s):
        p, o = u64(), u64()
        rc = self.L.orc_decode(s.encode("latin-1"), ctypes.byref(p), ctypes.byref(o))
        if rc != 0:
            raise ValueError("bad board string %r" % s)
        return p.value, o.value

    def solve_batch(self, p, o, depth=None, mode=0, threads=0):
        """mode 0: reference-order tree (scores, steps, nodes); mode 1: fast
        solver (scores, nodes, best move)."""
        p = np.ascontiguousarray(p, np.uint64)
        o = np.ascontiguousarray(o, np.uint64)
        n = len(p)
        if depth is None:
            depth = 32
        score = np.zeros(n, np.int8)
        steps = np.zeros(n, np.uint64)
        nodes = np.zeros(n, np.uint64)
        best = np.zeros(n, np.int8)
        self.L.orc_solve_batch(p.ctypes.data, o.ctypes.data, n, depth, mode, threads,
                               score.ctypes.data, steps.ctypes.data, nodes.ctypes.data,
                               best.ctypes.data)
        return score, steps, nodes, best


class Evaluator:
    """The oracle's pattern evaluator (orc_eval_create): feature masks, all
    tables as doubles in feature order, and the offset."""

    def __init__(self, oracle, features, values, offset):
        self.L = oracle.L
        f = np.ascontiguousarray(features, np.uint64)
        v = np.ascontiguousarray(values, np.float64)
        self.h = self.L.orc_eval_create(f.ctypes.data, len(f), v.ctypes.data, float(offset))
        if not self.h:
            raise ValueError("bad evaluator arguments")

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_eval_free(self.h)
            self.h = None

    def eval(self, p, o):
        return np.array([self.L.orc_eval(self.h, int(a), int(b)) for a, b in zip(p, o)],
                        np.float32)

    def think(self, p, o, depth, threads=0):
        """(scores, best moves, reference loop steps, nodes) of think mode."""
        p = np.ascontiguousarray(p, np.uint64)
        o = np.ascontiguousarray(o, np.uint64)
        n = len(p)
        score = np.zeros(n, np.int8)
        best = np.zeros(n, np.int8)
        steps = np.zeros(n, np.uint64)
        nodes = np.zeros(n, np.uint64)
        rc = self.L.orc_think_batch(self.h, p.ctypes.data, o.ctypes.data, n, depth, threads,
                                    score.ctypes.data, best.ctypes.data, steps.ctypes.data,
                                    nodes.ctypes.data)
        if rc != 0:
            raise ValueError("think depth must be >= 4")
        return score, best, steps, nodes
