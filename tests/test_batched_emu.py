"""The batched search kernel's own source (csrc/batched.cu) run on CPU
threads under the SIMT emulation (tests/batched_emu.cpp,
tests/simt/simt_prelude.h) against the reference's golden scores and the
oracle: the frame placements, the ordering threshold, the transposition
table, the stability cutoff, helping between the lanes of a warp, node
budgets and input rejection -- the code paths a GPU run takes, checked
without a GPU."""
import ctypes

import numpy as np
import pytest

from tests.test_oracle import golden_ref

OVERLAP, DEPTH, BUDGET = 2, 1, 4


class EmuOptions(ctypes.Structure):
    _fields_ = [("warps", ctypes.c_int), ("ff", ctypes.c_int), ("shared_frames", ctypes.c_int),
                ("help_min", ctypes.c_int), ("roots_per_warp", ctypes.c_int),
                ("stab_min", ctypes.c_int), ("stab_gate", ctypes.c_int),
                ("node_budget", ctypes.c_uint64), ("tt_bits", ctypes.c_int),
                ("tt_min", ctypes.c_int), ("order_table", ctypes.c_void_p),
                ("order_bits", ctypes.c_int), ("learned_min", ctypes.c_int)]


@pytest.fixture(scope="module")
def emu(built):
    L = ctypes.CDLL(built.build_batched_emu())
    L.emu_batched.argtypes = ([ctypes.c_void_p] * 2 + [ctypes.c_int] * 2 +
                              [ctypes.POINTER(EmuOptions)] + [ctypes.c_void_p] * 4)

    def run(p, o, depth, **kw):
        p = np.ascontiguousarray(p, np.uint64)
        o = np.ascontiguousarray(o, np.uint64)
        n = len(p)
        score = np.zeros(n, np.int8)
        best = np.zeros(n, np.int8)
        nodes = np.zeros(n, np.uint64)
        stats = np.zeros(7, np.uint64)
        opt = EmuOptions(**{"warps": 1, **kw})
        rc = L.emu_batched(p.ctypes.data, o.ctypes.data, n, depth, ctypes.byref(opt),
                           score.ctypes.data, best.ctypes.data, nodes.ctypes.data,
                           stats.ctypes.data)
        assert rc == 0
        return score, best, nodes, stats

    return run


@pytest.fixture(scope="module")
def c1():
    p, o, scores, _ = golden_ref("c1_seed0_e10")
    return p[:48], o[:48], scores[:48]


def test_scores_and_best_moves(emu, oracle, c1):
    p, o, scores = c1
    sc, bm, nodes, st = emu(p, o, 10, shared_frames=1)
    assert np.array_equal(sc.astype(int), scores)
    assert st[6] == 0 and st[0] == nodes.sum() and (nodes > 0).all()
    # every best move reaches the score
    for i in range(len(p)):
        m = int(bm[i])
        assert 0 <= m < 64
        f = oracle.L.orc_flip(int(p[i]), int(o[i]), m)
        assert f
        cp, co = int(o[i]) ^ f, int(p[i]) ^ f ^ (1 << m)
        v, _, _, _ = oracle.solve_batch(np.array([cp], np.uint64), np.array([co], np.uint64),
                                        mode=1)
        assert -int(v[0]) == int(sc[i])


@pytest.mark.parametrize("ff,shared", [(8, 0), (11, 1), (4, 1)])
def test_ordering_threshold_and_frame_placement(emu, c1, ff, shared):
    p, o, scores = c1
    sc, _, _, st = emu(p, o, 16, ff=ff, shared_frames=shared)
    assert np.array_equal(sc.astype(int), scores) and st[6] == 0


def test_transposition_table(emu, c1):
    p, o, scores = c1
    sc, _, nodes, st = emu(p, o, 10, shared_frames=1, tt_bits=17, tt_min=6)
    assert np.array_equal(sc.astype(int), scores) and st[6] == 0
    probes, hits, updates = int(st[1]), int(st[2]), int(st[3])
    assert probes > 0 and updates > 0 and hits <= probes


def test_stability_cutoff(emu, c1):
    p, o, scores = c1
    sc, _, _, st = emu(p, o, 10, shared_frames=1, stab_min=5, stab_gate=-64)
    assert np.array_equal(sc.astype(int), scores) and st[6] == 0
    assert st[5] > 0  # nodes closed by the cutoff


def test_lopsided_positions_with_passes(emu):
    """Lopsided endgames (|score| >= 40), where one side passes again and
    again, against the reference's own scores: the position after a pass is
    probed in the table, recorded and tried for the stability cutoff like
    any created node."""
    p, o, want, _ = golden_ref("lop_seed21_e11_12")
    sc, _, nodes, st = emu(p, o, 12, warps=2, shared_frames=1, tt_bits=17, tt_min=5,
                           stab_min=4, stab_gate=-64)
    assert np.array_equal(sc.astype(int), want) and st[6] == 0
    assert st[1] > 0 and st[5] > 0  # table probes, stability cutoffs


@pytest.mark.parametrize("rpw,warps,shared", [(1, 1, 1), (3, 2, 0)])
def test_helping_inside_a_warp(emu, oracle, rpw, warps, shared):
    p, o = oracle.generate(11, 8, 11, 13)
    want, _, _, _ = oracle.solve_batch(p, o, mode=1)
    # few positions per warp: the idle lanes receive moves of split nodes
    sc, bm, nodes, st = emu(p, o, 13, warps=warps, shared_frames=shared, help_min=6,
                            roots_per_warp=rpw, tt_bits=17, tt_min=7, stab_min=6, stab_gate=10)
    assert np.array_equal(sc, want) and st[6] == 0
    assert st[4] > 0  # moves handed out
    assert st[0] == nodes.sum()
    # best moves stay optimal although helpers report most of the root's moves
    for i in range(len(p)):
        m = int(bm[i]) & 0xFF
        if m >= 64:
            continue
        f = oracle.L.orc_flip(int(p[i]), int(o[i]), m)
        cp, co = int(o[i]) ^ f, int(p[i]) ^ f ^ (1 << m)
        v, _, _, _ = oracle.solve_batch(np.array([cp], np.uint64), np.array([co], np.uint64),
                                        mode=1)
        assert -int(v[0]) == int(sc[i])


def test_node_budget_fails(emu, c1):
    p, o, scores = c1
    _, _, full_nodes, _ = emu(p, o, 10, shared_frames=1)
    budget = int(np.median(full_nodes))
    _, _, _, st = emu(p, o, 10, shared_frames=1, node_budget=budget)
    assert int(st[6]) & BUDGET
    _, _, _, st = emu(p, o, 10, shared_frames=1, node_budget=int(full_nodes.max()) + 1)
    assert int(st[6]) == 0


def test_rejected_inputs(emu, c1):
    p, o, scores = c1
    p, o = p[:8].copy(), o[:8].copy()
    p[3] |= np.uint64(int(o[3]) & -int(o[3]))  # a square in both bitboards
    sc, _, _, st = emu(p, o, 10, shared_frames=1)
    assert int(st[6]) & OVERLAP and sc[3] == 0
    keep = np.arange(8) != 3
    assert np.array_equal(sc[keep].astype(int), scores[:8][keep])
    _, _, _, st = emu(p[keep], o[keep], 9, shared_frames=1)
    assert int(st[6]) & DEPTH


def pack_list(moves, total):
    """A move list as the learned orderer writes it (mlp.cu order_kernel):
    up to five (slot << 6 | square) entries of 12 bits, unused entries all
    ones, bit 63 set when the position has more legal moves than the list."""
    lst = 0x0FFFFFFFFFFFFFFF
    for slot, sq in enumerate(moves[:5]):
        e = (slot << 6) | sq
        lst = (lst & ~(0xFFF << (12 * slot))) | (e << (12 * slot))
    if total > min(5, len(moves)):
        lst |= 1 << 63
    return lst


M64 = (1 << 64) - 1


def table_key(p, o):
    """The exact position key of table.cuh (tt_key)."""
    x = (p * 0x9E3779B97F4A7C15) & M64
    r = ((x << 32) | (x >> 32)) & M64
    return x, ((o ^ r) * 0xD6E8FEB86659FD93) & M64


def order_table(entries, bits):
    """The learned order table as mlp.cu builds it: {x, y, list, 0} per
    entry, linear probing from the high bits of y."""
    t = np.zeros(4 << bits, np.uint64)
    for (p, o), lst in entries.items():
        x, y = table_key(p, o)
        h = y >> (64 - bits)
        while t[4 * h] or t[4 * h + 1]:
            h = (h + 1) & ((1 << bits) - 1)
        t[4 * h], t[4 * h + 1], t[4 * h + 2] = x, y, lst
    return t


@pytest.mark.parametrize("order", ["high_first", "best_first"])
def test_learned_order_table_keeps_scores_exact(emu, oracle, c1, order):
    """Lists for the roots and their children (nodes with >= 9 empties here)
    replace the fastest-first order: scores stay exact, node counts change."""
    p, o, scores = c1

    def moves_of(a, b):
        legal = oracle.L.orc_mobility(a, b)
        return [k for k in range(64) if (legal >> k) & 1]

    entries = {}
    for i in range(len(p)):
        a, b = int(p[i]), int(o[i])
        nodes = [(a, b)]
        for k in moves_of(a, b):
            f = oracle.L.orc_flip(a, b, k)
            nodes.append((b ^ f, a ^ f ^ (1 << k)))
        for (x, y) in nodes:
            ms = moves_of(x, y)
            if order == "high_first":
                ms = ms[::-1]
            else:  # the move the oracle finds best first
                _, _, _, bst = oracle.solve_batch(np.array([x], np.uint64), np.array([y], np.uint64),
                                                  mode=1)
                if 0 <= int(bst[0]) < 64:
                    ms.remove(int(bst[0]))
                    ms.insert(0, int(bst[0]))
            entries[(x, y)] = pack_list(ms, len(ms))
    table = order_table(entries, 12)
    _, _, plain_nodes, _ = emu(p, o, 10, shared_frames=1)
    sc, bm, nodes, st = emu(p, o, 10, shared_frames=1, order_table=table.ctypes.data,
                            order_bits=12, learned_min=9)
    assert np.array_equal(sc.astype(int), scores) and st[6] == 0
    assert not np.array_equal(nodes, plain_nodes)
