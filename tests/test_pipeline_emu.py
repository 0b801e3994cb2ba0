"""The library's whole solve pipeline -- C ABI, bucketing, batched and plain
search kernels, helping between the lanes of a warp, the allocation-free
entry point, the generator -- compiled as
host C++ and run on CPU threads (tests/pipeline_emu.cpp under the SIMT
emulation), called through the same C ABI the product exports, against the
reference's golden scores and the oracle.  No GPU is involved; this checks
the pipeline's logic (the GPU tests check the real device)."""
import ctypes

import numpy as np
import pytest

import gpuothello2_gb300 as g
from tests.test_oracle import golden_ref


@pytest.fixture(scope="module")
def emu(built):
    L = ctypes.CDLL(built.build_pipeline_emu())
    vp, i, u64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64
    L.gpo_default_options.argtypes = [ctypes.POINTER(g.Options)]
    L.gpo_default_options.restype = None
    L.solve_batch_ex.argtypes = [vp, vp, i, i, vp, vp, vp, ctypes.POINTER(g.Options),
                                 ctypes.POINTER(g.Stats)]
    L.solve_batch_device_noalloc.argtypes = [vp, vp, i, i, vp, vp]
    L.gpo_generate.argtypes = [u64, u64, i, i, i, vp, vp]
    return L


def solve(L, p, o, depth, **kw):
    p = np.ascontiguousarray(p, np.uint64)
    o = np.ascontiguousarray(o, np.uint64)
    n = len(p)
    score = np.zeros(n, np.int8)
    best = np.zeros(n, np.int8)
    nodes = np.zeros(n, np.uint64)
    opt = g.Options()
    L.gpo_default_options(ctypes.byref(opt))
    opt.threads_per_block = 32
    opt.table_bits = 17  # a small table keeps the emulated clears cheap
    for k, v in kw.items():
        setattr(opt, k, v)
    st = g.Stats()
    rc = L.solve_batch_ex(p.ctypes.data, o.ctypes.data, n, depth, score.ctypes.data,
                          best.ctypes.data, nodes.ctypes.data, ctypes.byref(opt),
                          ctypes.byref(st))
    return rc, score, best, nodes, st


def best_moves_reach_scores(oracle, p, o, score, best):
    for i in range(len(p)):
        m = int(best[i])
        if m == g.MOVE_PASS:
            cp, co = int(o[i]), int(p[i])
        else:
            assert 0 <= m < 64
            f = oracle.L.orc_flip(int(p[i]), int(o[i]), m)
            assert f
            cp, co = int(o[i]) ^ f, int(p[i]) ^ f ^ (1 << m)
        v, _, _, _ = oracle.solve_batch(np.array([cp], np.uint64), np.array([co], np.uint64),
                                        mode=1)
        assert -int(v[0]) == int(score[i]), i


@pytest.fixture(scope="module")
def c1():
    p, o, scores, _ = golden_ref("c1_seed0_e10")
    return p[:32], o[:32], scores[:32]


def test_default_pass(emu, oracle, c1):
    p, o, scores = c1
    rc, sc, bm, nodes, st = solve(emu, p, o, 10)
    assert rc == 0 and np.array_equal(sc.astype(int), scores)
    # bucketing (3) and one search launch: no host round trip in between
    assert st.launches == 4
    assert st.nodes == int(nodes.sum())
    assert st.table_probes > 0  # the table is on by default
    best_moves_reach_scores(oracle, p, o, sc, bm)


def test_helping_on_few_positions(emu, oracle):
    """Few deep positions for the warp: one root per warp, the other lanes
    search moves of its split nodes."""
    p, o = oracle.generate(12, 3, 12, 13)
    want, _, _, _ = oracle.solve_batch(p, o, mode=1)
    rc, sc, bm, nodes, st = solve(emu, p, o, 13, roots_per_warp=1, help_min_empties=6)
    assert rc == 0 and np.array_equal(sc, want)
    assert st.splits > 0 and st.nodes == int(nodes.sum())
    best_moves_reach_scores(oracle, p, o, sc, bm)


@pytest.mark.parametrize("plies", [1, 2])
def test_root_split_of_small_batches(emu, oracle, plies):
    """A small batch expanded at the root on the host: every frontier
    position solved by the kernel, values taken back up by negamax; scores,
    best moves (including passes) and node totals as the unsplit solve."""
    p, o = oracle.generate(13, 5, 13, 14)
    p = np.concatenate([p, [np.uint64(0xFFFFFFFF00000000)]])  # a finished game (0 empties)
    o = np.concatenate([o, [np.uint64(0x00000000FFFFFFFF)]])
    want, _, _, _ = oracle.solve_batch(p, o, mode=1)
    rc, sc, bm, nodes, st = solve(emu, p, o, 14, root_split_plies=plies)
    assert rc == 0 and np.array_equal(sc, want)
    assert st.root_split_positions > len(p) and st.nodes == int(nodes.sum())
    best_moves_reach_scores(oracle, p[:-1], o[:-1], sc[:-1], bm[:-1])
    assert int(bm[-1]) == g.MOVE_NONE
    rc, sc2, _, _, st2 = solve(emu, p, o, 14, root_split_plies=-1)
    assert rc == 0 and np.array_equal(sc2, want) and st2.root_split_positions == 0


@pytest.mark.parametrize("seed,n,lo,tail,kw", [(14, 12, 13, 4, {}),
                                                (15, 9, 12, 6, {"threads_per_block": 64}),
                                                (16, 11, 12, 3, {"roots_per_warp": 2})])
def test_tail_handoff(emu, oracle, seed, n, lo, tail, kw):
    """Once the queue is used up and few positions are unfinished, the
    kernel hands them back unsolved, each with its root's lower bound, and a
    root split finishes them with the table kept and the frontier searched
    in windows from those bounds: scores, best moves and node totals as
    without it."""
    p, o = oracle.generate(seed, n, lo, 14)
    want, _, _, _ = oracle.solve_batch(p, o, mode=1)
    rc, sc, bm, nodes, st = solve(emu, p, o, 14, tail_split_positions=tail, root_split_plies=-1,
                                  **kw)
    assert rc == 0 and np.array_equal(sc, want)
    # (positions with <= 12 empties go to the frontier unexpanded)
    assert 1 <= st.tail_positions <= tail and st.root_split_positions >= st.tail_positions
    assert st.nodes == int(nodes.sum())
    best_moves_reach_scores(oracle, p, o, sc, bm)
    if seed == 14:
        rc, sc2, _, _, st2 = solve(emu, p, o, 14, tail_split_positions=-1, root_split_plies=-1)
        assert rc == 0 and np.array_equal(sc2, want) and st2.tail_positions == 0


def test_mixed_empties_without_shared_frames(emu):
    p, o, scores, _ = golden_ref("c3_seed2_mixed")
    small = (64 - np.array([bin(int(a) | int(b)).count("1") for a, b in zip(p, o)])) <= 11
    p, o, scores = p[small][:40], o[small][:40], scores[small][:40]
    rc, sc, _, _, st = solve(emu, p, o, 16, smem_frames=-1)
    assert rc == 0 and np.array_equal(sc.astype(int), scores)


def test_plain_kernel_walks_reference_tree(emu, oracle, c1):
    p, o, scores = c1
    rc, sc, _, nodes, st = solve(emu, p, o, 10, method=g.METHOD_PLAIN)
    assert rc == 0 and np.array_equal(sc.astype(int), scores)
    _, _, onodes, _ = oracle.solve_batch(p, o, 10, mode=0)
    assert np.array_equal(nodes, onodes) and st.launches == 1


@pytest.mark.parametrize("kw", [{"use_table": 1, "table_bits": 17, "table_min_empties": 6},
                                {"use_table": 0, "stability_min_empties": -1,
                                 "help_min_empties": -1},
                                {"roots_per_warp": 4, "threads_per_block": 64},
                                {"fastest_first_empties": 11, "smem_frames": 3}])
def test_options_keep_scores_exact(emu, c1, kw):
    p, o, scores = c1
    rc, sc, _, _, st = solve(emu, p, o, 12, **kw)
    assert rc == 0 and np.array_equal(sc.astype(int), scores)
    if kw.get("use_table") == 1:
        assert st.table_probes > 0 and st.table_updates > 0
    if kw.get("use_table") == 0:
        assert st.table_probes == 0


def test_error_statuses(emu, c1):
    p, o, scores = c1
    assert solve(emu, p, o, 9)[0] == g.GPO_ERR_DEPTH
    q = p.copy()
    q[5] |= np.uint64(int(o[5]) & -int(o[5]))
    rc, sc, _, _, _ = solve(emu, q, o, 10)
    assert rc == g.GPO_ERR_BOARD
    keep = np.arange(len(p)) != 5
    assert np.array_equal(sc[keep].astype(int), scores[keep])
    # the node budget is a watchdog: exceeding it fails the call
    assert solve(emu, p, o, 10, node_budget=500)[0] == g.GPO_ERR_TIMEOUT
    # bad option values
    assert solve(emu, p, o, 10, roots_per_warp=33)[0] == g.GPO_ERR_ARG
    assert solve(emu, p, o, 10, table_bits=40)[0] == g.GPO_ERR_ARG


def test_allocation_free_entry_point(emu, c1):
    p, o, scores = c1
    p = np.ascontiguousarray(p, np.uint64)
    o = np.ascontiguousarray(o, np.uint64)
    sc = np.zeros(len(p), np.int8)
    # device pointers are host pointers in the emulation
    rc = emu.solve_batch_device_noalloc(p.ctypes.data, o.ctypes.data, len(p), 10,
                                        sc.ctypes.data, None)
    assert rc == 0 and np.array_equal(sc.astype(int), scores)


def test_generator_matches_oracle(emu, oracle):
    p = np.zeros(500, np.uint64)
    o = np.zeros(500, np.uint64)
    assert emu.gpo_generate(2, 1000, 500, 8, 16, p.ctypes.data, o.ctypes.data) == 0
    op, oo = oracle.generate(2, 500, 8, 16, first=1000)
    assert np.array_equal(p, op) and np.array_equal(o, oo)


def test_random_option_mixes(emu, oracle):
    """Seeded random batches, depths and option mixes against the oracle."""
    rng = np.random.default_rng(20261203)
    for _ in range(8):
        n = int(rng.integers(1, 24))
        lo = int(rng.integers(1, 11))
        hi = int(rng.integers(lo, 12))
        depth = int(rng.integers(hi, hi + 6))
        p, o = oracle.generate(int(rng.integers(100, 10000)), n, lo, hi)
        want, _, _, _ = oracle.solve_batch(p, o, mode=1)
        kw = {"threads_per_block": int(rng.choice([32, 64]))}
        if rng.random() < 0.5:
            kw["roots_per_warp"] = int(rng.choice([1, 2, 8]))
        if rng.random() < 0.5:
            kw["help_min_empties"] = int(rng.choice([-1, 4, 6, 9]))
        if rng.random() < 0.3:
            kw.update(use_table=int(rng.choice([0, 1])),
                      table_min_empties=int(rng.integers(3, 10)))
        if rng.random() < 0.3:
            kw["stability_min_empties"] = int(rng.choice([-1, 3, 6]))
        if rng.random() < 0.3:
            kw["smem_frames"] = int(rng.choice([-1, 1, 3, 8]))
        if rng.random() < 0.3:
            kw["fastest_first_empties"] = int(rng.integers(3, 13))
        if rng.random() < 0.3:
            kw["tail_split_positions"] = int(rng.choice([-1, 2, 5]))
        rc, sc, _, _, _ = solve(emu, p, o, depth, **kw)
        assert rc == 0 and np.array_equal(sc, want), (n, lo, hi, depth, kw)
