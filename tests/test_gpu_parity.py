"""GPU parity: both CUDA methods against the reference's golden scores and
the CPU oracle, through the C ABI.  Bit-exact everywhere (integer scores)."""
import os
import re
import subprocess

import numpy as np
import pytest

from gpuothello2_gb300 import codec
from tests.conftest import GOLDEN
from tests.test_oracle import FIXTURES, golden_ref

pytestmark = pytest.mark.gpu

PLAIN, BATCHED = 1, 0


@pytest.mark.parametrize("name,seed,count,lo,hi,depth", FIXTURES)
def test_gpu_generator_matches_golden(gpu, name, seed, count, lo, hi, depth):
    path = os.path.join(GOLDEN, name + ".txt")
    if not os.path.exists(path):
        pytest.skip("fixture missing")
    gp, go = codec.read_board_file(path)
    p, o = gpu.generate(seed, count, lo, hi)
    assert np.array_equal(p, gp) and np.array_equal(o, go)


def test_gpu_generator_matches_oracle_stream(gpu, oracle):
    for seed, lo, hi in ((1, 10, 10), (2, 8, 16), (3, 12, 14), (4, 18, 18), (7, 0, 60)):
        p, o = gpu.generate(seed, 3000, lo, hi, first=12345)
        op, oo = oracle.generate(seed, 3000, lo, hi, first=12345)
        assert np.array_equal(p, op) and np.array_equal(o, oo), seed


@pytest.mark.parametrize("name,seed,count,lo,hi,depth", FIXTURES)
@pytest.mark.parametrize("method", [PLAIN, BATCHED])
def test_scores_match_reference(gpu, name, seed, count, lo, hi, depth, method):
    if method == PLAIN and depth > 16:
        pytest.skip("one thread per position in the reference tree: minutes at 18-22 empties")
    p, o, scores, _ = golden_ref(name)
    sc, _, _, st, _ = gpu.solve(p, o, depth, method=method, wait_limit_ms=600000)
    assert np.array_equal(sc.astype(int), scores)
    assert st.nodes > 0
    # plain: the search kernel; batched: bucketing (3) + the search, and the
    # same again for the root split that finishes a handed-back tail
    assert st.launches == (1 if method == PLAIN else (8 if st.tail_positions else 4))


@pytest.mark.parametrize("name,depth", [("c1_seed0_e10", 10), ("c3_seed2_mixed", 16),
                                        ("readme9", 10)])
def test_plain_kernel_walks_reference_tree(gpu, oracle, name, depth):
    """Per-position node counts of the plain kernel equal the oracle's count
    of the reference tree (root + pushed children + pass frames)."""
    p, o, scores, _ = golden_ref(name)
    sc, _, nodes, st, _ = gpu.solve(p, o, depth, method=PLAIN, nodes=True)
    osc, _, onodes, _ = oracle.solve_batch(p, o, depth, mode=0)
    assert np.array_equal(sc, osc)
    assert np.array_equal(nodes, onodes)
    assert st.nodes == int(onodes.sum())


def test_solve_batch_plain_entry_point(gpu):
    p, o, scores, _ = golden_ref("c1_seed0_e10")
    sc = gpu.solve_batch(p, o, 10)
    assert np.array_equal(sc.astype(int), scores)


def test_best_moves_are_optimal(gpu, oracle):
    p, o = oracle.generate(3, 2000, 12, 14)
    sc, best, _, _, _ = gpu.solve(p, o, 14, best=True)
    osc, _, _, _ = oracle.solve_batch(p, o, 14, mode=1)
    assert np.array_equal(sc, osc)
    cp, co, want = [], [], []
    for i in range(len(p)):
        b = int(best[i])
        assert 0 <= b <= 65
        if b >= 64:
            continue
        f = oracle.L.orc_flip(int(p[i]), int(o[i]), b)
        assert f != 0, "best move is not legal"
        cp.append(int(o[i]) ^ f)
        co.append(int(p[i]) ^ f ^ (1 << b))
        want.append(-int(sc[i]))
    csc, _, _, _ = oracle.solve_batch(np.array(cp, np.uint64), np.array(co, np.uint64), 32, mode=1)
    assert np.array_equal(csc.astype(int), np.array(want))


def edge_positions(oracle):
    """Full boards, 1-2 empties, forced passes, game-over positions, an empty
    batch entry duplicate, the start position region."""
    full_p = 0xFFFFFFFF00000000
    full_o = 0x00000000FFFFFFFF
    cases = [
        (full_p, full_o),                       # 0 empties, draw
        (full_p | 0xFFFF, full_o & ~0xFFFF),    # 0 empties, win
        ((full_p | full_o) & ~1, 0),            # one side only, 1 empty, game over
        (0xFFFFFFFFFFFFFFFE & ~(1 << 63), 1 << 63),  # 1 empty, no flips for either? checked by oracle
    ]
    # positions where the side to move must pass: take random 3-10 empty
    # positions and keep those with no legal move but a legal reply
    p, o = oracle.generate(11, 20000, 1, 12)
    for a, b in zip(p, o):
        a, b = int(a), int(b)
        if oracle.L.orc_mobility(a, b) == 0:
            cases.append((a, b))
        if len(cases) > 200:
            break
    return cases


@pytest.mark.parametrize("method", [PLAIN, BATCHED])
def test_edge_positions(gpu, oracle, method):
    cases = edge_positions(oracle)
    p = np.array([c[0] for c in cases] * 2, np.uint64)  # duplicates included
    o = np.array([c[1] for c in cases] * 2, np.uint64)
    sc, best, _, _, _ = gpu.solve(p, o, 12, method=method, best=(method == BATCHED))
    osc, _, _, _ = oracle.solve_batch(p, o, 12, mode=1)
    assert np.array_equal(sc, osc)
    if method == BATCHED:
        for i in range(len(p)):
            if oracle.L.orc_mobility(int(p[i]), int(o[i])) == 0:
                assert int(best[i]) in (64, 65)


def test_errors_are_reported_and_context_survives(gpu):
    g = gpu
    p, o, scores, _ = golden_ref("c1_seed0_e10")
    # a square on both sides
    bp, bo = p[:8].copy(), o[:8].copy()
    low = int(bp[3]) & -int(bp[3])
    bo[3] = np.uint64(int(bo[3]) | low)
    _, _, _, _, rc = g.solve(bp, bo, 10, check=False)
    assert rc == g.GPO_ERR_BOARD
    # more empties than depth
    _, _, _, _, rc = g.solve(p[:8], o[:8], 9, check=False)
    assert rc == g.GPO_ERR_DEPTH
    _, _, _, _, rc = g.solve(p[:8], o[:8], 9, method=PLAIN, check=False)
    assert rc == g.GPO_ERR_DEPTH
    # node budget watchdog
    _, _, _, _, rc = g.solve(p[:64], o[:64], 10, node_budget=5, check=False)
    assert rc == g.GPO_ERR_TIMEOUT
    # the context still works afterwards
    sc, _, _, _, _ = g.solve(p, o, 10)
    assert np.array_equal(sc.astype(int), scores)
    # empty batch
    sc, _, _, _, rc = g.solve(p[:0], o[:0], 10)
    assert rc == 0 and len(sc) == 0


def test_device_entry_point(gpu):
    torch = pytest.importorskip("torch")
    import ctypes

    g = gpu
    p, o, scores, _ = golden_ref("c3_seed2_mixed")
    dp = torch.from_numpy(p.view(np.int64)).cuda()
    do = torch.from_numpy(o.view(np.int64)).cuda()
    ds = torch.zeros(len(p), dtype=torch.int8, device="cuda")
    st = g.Stats()
    opt = g.options()
    stream = torch.cuda.current_stream().cuda_stream
    rc = g.lib().solve_batch_device(dp.data_ptr(), do.data_ptr(), len(p), 16, ds.data_ptr(), None,
                                    None, ctypes.byref(opt), ctypes.byref(st), stream)
    assert rc == 0
    assert np.array_equal(ds.cpu().numpy().astype(int), scores)


def test_cli_output_matches_reference_file(gpu, tmp_path):
    """`solver IN OUT DEPTH` writes the reference's lines: same boards, same
    (player, opponent) order, same scores."""
    from gpuothello2_gb300 import build

    for name, depth in (("c1_seed0_e10", 10), ("c3_seed2_mixed", 16), ("readme9", 10)):
        out = tmp_path / (name + ".out")
        r = subprocess.run([build.SOLVER_BIN, os.path.join(GOLDEN, name + ".txt"), str(out),
                            str(depth)], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        assert "cudaSuccess (no error), elapsed:" in r.stderr and "total nodes:" in r.stderr
        ref = [ln.split()[:2] for ln in open(os.path.join(GOLDEN, name + ".ref"))]
        got = [ln.split() for ln in open(out)]
        assert got == ref
        env = dict(os.environ, GPO_METHOD="plain")
        r = subprocess.run([build.SOLVER_BIN, os.path.join(GOLDEN, name + ".txt"), str(out),
                            str(depth)], capture_output=True, text=True, timeout=300, env=env)
        assert r.returncode == 0, r.stderr
        assert [ln.split() for ln in open(out)] == ref


@pytest.mark.parametrize("name,depth,help_min,rpw", [("c4_seed4_e18", 18, 10, 1),
                                                     ("c3_seed2_mixed", 16, 6, 2),
                                                     ("c3_seed2_mixed", 16, -1, 0),
                                                     ("c1_seed0_e10", 10, 5, 1)])
def test_helping_is_exact(gpu, oracle, name, depth, help_min, rpw):
    """Few positions per warp: idle lanes search moves of their warp's split
    nodes (help_min > 0) or stay idle (help_min < 0); scores stay exact, best
    moves optimal, and the positions' node counts add up to the launch
    total."""
    p, o, scores, _ = golden_ref(name)
    sc, best, nodes, st, _ = gpu.solve(p, o, depth, best=True, nodes=True,
                                       help_min_empties=help_min, roots_per_warp=rpw,
                                       wait_limit_ms=120000)
    assert np.array_equal(sc.astype(int), scores)
    assert int(nodes.sum()) == st.nodes
    if help_min > 0:
        assert st.splits > 0
    else:
        assert st.splits == 0
    cp, co, want = [], [], []
    for i in range(0, len(p), max(1, len(p) // 32)):
        b = int(best[i])
        if b >= 64:
            continue
        f = oracle.L.orc_flip(int(p[i]), int(o[i]), b)
        cp.append(int(o[i]) ^ f)
        co.append(int(p[i]) ^ f ^ (1 << b))
        want.append(-int(sc[i]))
    csc, _, _, _ = oracle.solve_batch(np.array(cp, np.uint64), np.array(co, np.uint64), 32, mode=1)
    assert np.array_equal(csc.astype(int), np.array(want))


@pytest.mark.parametrize("name,depth,bits,tmin", [("c3_seed2_mixed", 16, 20, 9),
                                                  ("c3_seed2_mixed", 16, 17, 5),
                                                  ("c4_seed4_e18", 18, 24, 7),
                                                  ("c1_seed0_e10", 10, 20, 4)])
def test_transposition_table_is_exact(gpu, name, depth, bits, tmin):
    """The 128-bit-CAS table changes node counts only, whatever its size
    and threshold (a small table forces constant eviction)."""
    p, o, scores, _ = golden_ref(name)
    sc, _, _, st, _ = gpu.solve(p, o, depth, use_table=1, table_min_empties=tmin,
                                table_bits=bits, wait_limit_ms=120000)
    assert np.array_equal(sc.astype(int), scores)
    assert st.table_probes > 0 and st.table_updates > 0
    assert st.table_hits <= st.table_probes and st.table_bits == bits


def test_table_options_are_checked(gpu):
    p, o, scores, _ = golden_ref("readme9")
    _, _, _, _, rc = gpu.solve(p, o, 10, use_table=1, table_bits=12, check=False)
    assert rc == gpu.GPO_ERR_ARG
    sc, _, _, st, _ = gpu.solve(p, o, 10, use_table=0)
    assert np.array_equal(sc.astype(int), scores) and st.table_probes == 0


def test_gen_boards_writes_the_golden_board_file(gpu, tmp_path):
    """`gen_boards OUT N SEED MIN [MAX]` writes the stream the golden board
    file holds, byte for byte."""
    from gpuothello2_gb300 import build

    out = tmp_path / "c1.txt"
    r = subprocess.run([build.GEN_BIN, str(out), "4096", "0", "10"], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert out.read_text() == open(os.path.join(GOLDEN, "c1_seed0_e10.txt")).read()


def test_cli_table_counters_and_switches(gpu, tmp_path):
    """The CLI's reference-format stderr line carries the table's counters
    (update count, hit, find) with the table on, zeros with GPO_TABLE=0; the
    learned orderer's weights load by default; the scores stay the
    reference's throughout."""
    from gpuothello2_gb300 import build

    src = os.path.join(GOLDEN, "c3_seed2_mixed.txt")
    ref = [ln.split()[:2] for ln in open(os.path.join(GOLDEN, "c3_seed2_mixed.ref"))]
    pat = re.compile(r"table update count: (\d+), table hit: (\d+), table find: (\d+)")
    for env, on in (({}, True), ({"GPO_TABLE": "0"}, False), ({"GPO_WEIGHTS": "none"}, True),
                    ({"GPO_TABLE_BITS": "20"}, True)):
        out = tmp_path / "out.txt"
        r = subprocess.run([build.SOLVER_BIN, src, str(out), "16"], capture_output=True,
                           text=True, timeout=300, env=dict(os.environ, **env))
        assert r.returncode == 0, r.stderr
        upd, hit, find = map(int, pat.search(r.stderr).groups())
        if on:
            assert upd > 0 and find > 0 and 0 < hit <= find, r.stderr
        else:
            assert upd == hit == find == 0
        assert [ln.split() for ln in open(out)] == ref
    r = subprocess.run([build.SOLVER_BIN, src, str(tmp_path / "x"), "16"], capture_output=True,
                       text=True, timeout=300, env=dict(os.environ, GPO_WEIGHTS="/nonexistent"))
    assert r.returncode != 0 and "weights" in r.stderr
