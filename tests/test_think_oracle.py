"""The oracle's pattern evaluator and think-mode search against the
reference's own (eval.cu, thinker.cu run by oracle/ref_build.sh's
refthink; fixtures made by tests/golden/make_golden.py): evaluation bits,
scores, best moves and the reference's loop-step counts must all match."""
import os

import numpy as np
import pytest

from gpuothello2_gb300 import codec
from tests.conftest import GOLDEN
from tests.golden import think_data as T
from tests.oracle_lib import Evaluator

THINK_FIXTURES = [("think_seed6_e24_34_d6", 6), ("think_seed7_e6_12_d4", 4),
                  ("think_seed8_e20_28_d8", 8), ("think_edge_d5", 5)]


def move_code(s):
    """The reference's move strings (main.cu:31-39) back to square codes."""
    if s == "ps":
        return 64
    return (ord(s[1]) - ord("1")) * 8 + (ord(s[0]) - ord("A"))


def think_ref(name):
    path = os.path.join(GOLDEN, name + ".ref")
    if not os.path.exists(path):
        pytest.skip("fixture %s not generated" % name)
    rows = [ln.split() for ln in open(path) if ln.strip()]
    boards = [codec.decode(r[0]) for r in rows]
    p = np.array([b[0] for b in boards], np.uint64)
    o = np.array([b[1] for b in boards], np.uint64)
    score = np.array([int(r[1]) for r in rows])
    best = np.array([move_code(r[2]) for r in rows])
    steps = np.array([int(r[3]) for r in rows], np.uint64)
    return p, o, score, best, steps


def eval_ref():
    rows = [ln.split() for ln in open(os.path.join(GOLDEN, "eval_vectors.txt")) if ln.strip()]
    p = np.array([int(r[0], 16) for r in rows], np.uint64)
    o = np.array([int(r[1], 16) for r in rows], np.uint64)
    bits = np.array([int(r[2], 16) for r in rows], np.uint32)
    return p, o, bits


@pytest.fixture(scope="module")
def evaluator(oracle):
    return Evaluator(oracle, T.features(), T.values(), T.OFFSET)


def test_evaluation_bits_match_reference(evaluator):
    p, o, bits = eval_ref()
    assert len(p) > 1800
    got = evaluator.eval(p, o).view(np.uint32)
    assert np.array_equal(got, bits)
    v = bits.view(np.float32)
    # the weights exercise the clamp and fractional values
    assert (np.abs(v) == 64).any() and (v != np.round(v)).any()


@pytest.mark.parametrize("name,depth", THINK_FIXTURES)
def test_think_matches_reference(evaluator, name, depth):
    p, o, score, best, steps = think_ref(name)
    sc, bm, st, nodes = evaluator.think(p, o, depth)
    assert np.array_equal(sc.astype(int), score)
    assert np.array_equal(bm.astype(int), best)
    assert np.array_equal(st, steps)
    assert (nodes > 0).all()


def test_edge_boards_cover_passes_and_finished_games():
    p, o, score, best, _ = think_ref("think_edge_d5")
    assert (best == 64).sum() >= 3          # roots that pass
    assert 0 in score and -62 in score      # finished games, one with empties


def test_feature_file_round_trip(tmp_path):
    path = tmp_path / "features.txt"
    T.write_features(str(path))
    tok = path.read_text().split()
    n = int(tok[0])
    masks = []
    for i in range(n):
        rows = tok[1 + 8 * i: 9 + 8 * i]
        masks.append(T.mask_of(rows))
    assert masks == T.features()
    assert T.values().shape == (sum(3 ** bin(f).count("1") for f in T.features()),)
