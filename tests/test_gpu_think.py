"""Think mode and the pattern evaluator on the GPU (think_batch,
gpo_evaluate, the CLI's 4-argument form) against the reference's fixtures
(tests/golden/think_*, eval_vectors.txt, made by the reference's own
eval.cu and thinker.cu) and the oracle.  Bit-exact: evaluation bits,
scores, best moves; node counts equal the oracle's."""
import os
import subprocess

import numpy as np
import pytest

from tests.golden import think_data as T
from tests.oracle_lib import Evaluator
from tests.test_think_oracle import THINK_FIXTURES, eval_ref, think_ref

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eval_dir(tmp_path_factory):
    """The evaluator files under the names the CLI looks for."""
    d = tmp_path_factory.mktemp("think")
    os.makedirs(d / "value")
    T.write_features(str(d / "subboard.txt"))
    T.write_values(str(d / "value" / "value52"))
    return d


@pytest.fixture(scope="module")
def loaded(gpu, eval_dir):
    gpu.eval_load_files(str(eval_dir / "subboard.txt"), str(eval_dir / "value" / "value52"))
    return gpu


def test_evaluation_bits_match_reference(loaded):
    p, o, bits = eval_ref()
    v = loaded.evaluate(p, o)
    assert np.array_equal(v.view(np.uint32), bits)


@pytest.mark.parametrize("name,depth", THINK_FIXTURES)
def test_think_matches_reference(loaded, oracle, name, depth):
    p, o, score, best, _ = think_ref(name)
    sc, bm, nodes, st, _ = loaded.think(p, o, depth)
    assert np.array_equal(sc.astype(int), score)
    assert np.array_equal(bm.astype(int), best)
    ev = Evaluator(oracle, T.features(), T.values(), T.OFFSET)
    _, _, _, onodes = ev.think(p, o, depth)
    assert np.array_equal(nodes, onodes)
    assert st.nodes == int(nodes.sum()) and st.launches == 1


def test_think_batch_against_oracle(loaded, oracle):
    p, o = oracle.generate(10, 1024, 14, 40)
    sc, bm, nodes, _, _ = loaded.think(p, o, 5)
    ev = Evaluator(oracle, T.features(), T.values(), T.OFFSET)
    osc, obm, _, onodes = ev.think(p, o, 5)
    assert np.array_equal(sc, osc) and np.array_equal(bm, obm)
    assert np.array_equal(nodes, onodes)


def test_think_errors(loaded):
    p = np.array([0x0000000810000000], np.uint64)
    o = np.array([0x0000001008000000], np.uint64)
    assert loaded.think(p, o, 3, check=False)[4] == loaded.GPO_ERR_DEPTH
    assert loaded.think(p, o, 25, check=False)[4] == loaded.GPO_ERR_DEPTH
    assert loaded.think(p, p, 5, check=False)[4] == loaded.GPO_ERR_BOARD
    with pytest.raises(loaded.SolverError):
        loaded.evaluate(p, p)


def test_cli_think_mode_writes_reference_lines(loaded, eval_dir, built):
    name, depth = "think_seed6_e24_34_d6", 6
    src = os.path.join(os.path.dirname(__file__), "golden", name + ".txt")
    out = eval_dir / "out.txt"
    r = subprocess.run([built.SOLVER_BIN, src, str(out), "60", str(depth)], cwd=str(eval_dir),
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert r.stderr.startswith("n = ")
    assert "total nodes: " in r.stderr
    ref = os.path.join(os.path.dirname(__file__), "golden", name + ".ref")
    want = [" ".join(ln.split()[:3]) for ln in open(ref) if ln.strip()]
    got = out.read_text().splitlines()
    assert got == want
