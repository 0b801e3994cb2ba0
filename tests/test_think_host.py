"""The think-mode search and evaluator source the GPU kernels run
(csrc/think.cuh, csrc/evalfile.h), compiled for the CPU
(tests/think_host.cpp), against the reference's fixtures and the oracle:
evaluation bits, scores and best moves equal the reference's, node counts
equal the oracle's, and the file readers read what the reference reads."""
import ctypes
import struct

import numpy as np
import pytest

from tests.golden import think_data as T
from tests.oracle_lib import Evaluator
from tests.test_think_oracle import THINK_FIXTURES, eval_ref, think_ref

GPO_ERR_ARG, GPO_ERR_DEPTH, GPO_ERR_IO = -1, -2, -8


@pytest.fixture(scope="module")
def host(built):
    path = built.build_think_host()
    L = ctypes.CDLL(path)
    vp, i, u64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64
    L.th_load.argtypes = [vp, i, vp, ctypes.c_double]
    L.th_load_files.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
    L.th_read_features.argtypes = [ctypes.c_char_p, vp, i]
    L.th_evaluate.argtypes = [vp, vp, i, vp]
    L.th_think.argtypes = [vp, vp, i, i, vp, vp, vp]
    for name in ("th_transpose", "th_flip_rows"):
        getattr(L, name).argtypes = [u64]
        getattr(L, name).restype = u64
    L.th_mobility.argtypes = [u64, u64]
    L.th_mobility.restype = u64
    L.th_flips.argtypes = [u64, u64, i]
    L.th_flips.restype = u64
    return L


@pytest.fixture(scope="module")
def eval_files(tmp_path_factory):
    d = tmp_path_factory.mktemp("eval")
    feat, val = d / "features.txt", d / "values.bin"
    T.write_features(str(feat))
    T.write_values(str(val))
    return str(feat), str(val)


def think_host(host, p, o, depth):
    n = len(p)
    p = np.ascontiguousarray(p, np.uint64)
    o = np.ascontiguousarray(o, np.uint64)
    score = np.zeros(n, np.int8)
    best = np.zeros(n, np.int8)
    nodes = np.zeros(n, np.uint64)
    rc = host.th_think(p.ctypes.data, o.ctypes.data, n, depth, score.ctypes.data,
                       best.ctypes.data, nodes.ctypes.data)
    return rc, score, best, nodes


def test_board_helpers_match_oracle(host, oracle):
    rng = np.random.default_rng(5)
    for _ in range(2000):
        x, y = (int(v) for v in rng.integers(0, 2**63, 2, dtype=np.uint64) * 2 + 1)
        p, o = x & y, x & ~y & 0xFFFFFFFFFFFFFFFF
        t = 0
        for sq in range(64):
            if (x >> sq) & 1:
                t |= 1 << ((sq % 8) * 8 + sq // 8)
        assert host.th_transpose(x) == t
        assert host.th_flip_rows(x) == int.from_bytes(x.to_bytes(8, "little")[::-1], "little")
        assert host.th_mobility(p, o) == oracle.L.orc_mobility(p, o)
        sq = int(rng.integers(0, 64))
        if not ((p | o) >> sq) & 1:
            assert host.th_flips(p, o, sq) == oracle.L.orc_flip(p, o, sq)


def test_feature_file_reader(host, eval_files, tmp_path):
    masks = np.zeros(32, np.uint64)
    n = host.th_read_features(eval_files[0].encode(), masks.ctypes.data, 32)
    assert n == len(T.PATTERNS)
    assert [int(m) for m in masks[:n]] == T.features()
    # a bitset row may be shorter than 8 digits and rows may share a line
    odd = tmp_path / "odd.txt"
    odd.write_text("1\n101 1 0 0\n0 0 0 11111111\n")
    assert host.th_read_features(str(odd).encode(), masks.ctypes.data, 32) == 1
    assert int(masks[0]) == 0b101 | (1 << 8) | (0xFF << 56)
    bad = tmp_path / "bad.txt"
    bad.write_text("1\n11111111 x\n")
    assert host.th_read_features(str(bad).encode(), masks.ctypes.data, 32) == GPO_ERR_ARG
    assert host.th_read_features(str(tmp_path / "none").encode(), masks.ctypes.data,
                                 32) == GPO_ERR_IO


def test_value_file_reader_rejects_short_files(host, eval_files, tmp_path):
    short = tmp_path / "short.bin"
    short.write_bytes(open(eval_files[1], "rb").read()[:-8])  # no offset
    assert host.th_load_files(eval_files[0].encode(), str(short).encode()) == GPO_ERR_IO
    assert host.th_load_files(eval_files[0].encode(), str(tmp_path / "x").encode()) == GPO_ERR_IO
    assert host.th_load_files(eval_files[0].encode(), eval_files[1].encode()) == 0


def test_too_many_squares_or_tables_are_rejected(host):
    vals = np.zeros(3 ** 13, np.float64)
    big = np.array([(1 << 13) - 1], np.uint64)
    assert host.th_load(big.ctypes.data, 1, vals.ctypes.data, 0.0) == GPO_ERR_ARG
    # 9 features of one square in each of 8 bytes: 72 byte tables > 64
    spread = np.array([0x0101010101010101] * 9, np.uint64)
    v = np.zeros(9 * 3 ** 8, np.float64)
    assert host.th_load(spread.ctypes.data, 9, v.ctypes.data, 0.0) == GPO_ERR_ARG


def test_evaluation_bits_match_reference(host, eval_files):
    assert host.th_load_files(eval_files[0].encode(), eval_files[1].encode()) == 0
    p, o, bits = eval_ref()
    out = np.zeros(len(p), np.float32)
    assert host.th_evaluate(p.ctypes.data, o.ctypes.data, len(p), out.ctypes.data) == 0
    assert np.array_equal(out.view(np.uint32), bits)


@pytest.mark.parametrize("name,depth", THINK_FIXTURES)
def test_think_matches_reference_and_oracle(host, oracle, eval_files, name, depth):
    assert host.th_load_files(eval_files[0].encode(), eval_files[1].encode()) == 0
    p, o, score, best, _ = think_ref(name)
    rc, sc, bm, nodes = think_host(host, p, o, depth)
    assert rc == 0
    assert np.array_equal(sc.astype(int), score)
    assert np.array_equal(bm.astype(int), best)
    ev = Evaluator(oracle, T.features(), T.values(), T.OFFSET)
    _, _, _, onodes = ev.think(p, o, depth)
    assert np.array_equal(nodes, onodes)


def test_depth_limits(host, eval_files):
    assert host.th_load_files(eval_files[0].encode(), eval_files[1].encode()) == 0
    p = np.array([0x0000000810000000], np.uint64)
    o = np.array([0x0000001008000000], np.uint64)
    for d in (3, 25):
        assert think_host(host, p, o, d)[0] == GPO_ERR_DEPTH
    rc, sc, bm, nodes = think_host(host, p, o, 4)
    assert rc == 0 and 0 <= bm[0] < 64 and nodes[0] > 1


def test_values_are_stored_as_float(host, tmp_path):
    # one 1-square feature; values chosen so that double->float rounding matters
    feat = tmp_path / "f.txt"
    feat.write_text("1\n00000001\n0\n0\n0\n0\n0\n0\n0\n")
    val = tmp_path / "v.bin"
    val.write_bytes(struct.pack("=4d", 0.1, 1.0 + 2 ** -30, -0.3, 0.25))
    assert host.th_load_files(str(feat).encode(), str(val).encode()) == 0
    p = np.array([1], np.uint64)
    o = np.array([0], np.uint64)
    out = np.zeros(1, np.float32)
    host.th_evaluate(p.ctypes.data, o.ctypes.data, 1, out.ctypes.data)
    # A1 is `me` in the board and in its transpose; its rotations put the
    # disc on H1, H8, A8 (empty for the mask); float accumulation
    f = np.float32
    acc = f(0)
    for term in (f(1.0 + 2 ** -30), f(1.0 + 2 ** -30), f(0.1), f(0.1), f(0.1), f(0.1),
                 f(0.1), f(0.1)):
        acc = f(acc + term)
    assert out[0] == f(acc + f(0.25))
