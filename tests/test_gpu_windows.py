"""Principal-variation-first expansion (expand_windows = 1) on the GPU:
the first child of a hard position with a full window, its siblings with a
null window, the ones that beat the bound again -- against the reference's
golden scores, with best moves checked by the oracle."""
import numpy as np
import pytest

from tests.test_oracle import golden_ref

pytestmark = pytest.mark.gpu


def best_moves_reach_scores(oracle, p, o, score, best):
    for i in range(len(p)):
        m = int(best[i])
        if m == 64:
            cp, co = int(o[i]), int(p[i])
        else:
            assert 0 <= m < 64
            f = oracle.L.orc_flip(int(p[i]), int(o[i]), m)
            assert f
            cp, co = int(o[i]) ^ f, int(p[i]) ^ f ^ (1 << m)
        v, _, _, _ = oracle.solve_batch(np.array([cp], np.uint64), np.array([co], np.uint64),
                                        mode=1)
        assert -int(v[0]) == int(score[i])


@pytest.mark.parametrize("mode,budget", [(1, 2000), (1, 1 << 16), (2, 1 << 16)])
def test_windowed_expansion_matches_reference(gpu, oracle, mode, budget):
    p, o, scores, _ = golden_ref("c3_seed2_mixed")
    sc, best, _, st, _ = gpu.solve(p, o, 16, best=True, expand_budget=budget,
                                   expand_windows=mode)
    assert np.array_equal(sc.astype(int), scores)
    assert st.splits > 0
    sel = np.arange(0, len(p), 8)
    best_moves_reach_scores(oracle, p[sel], o[sel], sc[sel], best[sel])


def test_windowed_expansion_uses_fewer_nodes(gpu):
    p, o, scores, _ = golden_ref("c3_seed2_mixed")
    full = gpu.solve(p, o, 16, expand_budget=1 << 16)[3]
    win = gpu.solve(p, o, 16, expand_budget=1 << 16, expand_windows=1)[3]
    rec = gpu.solve(p, o, 16, expand_budget=1 << 16, expand_windows=2)[3]
    print("nodes: full-window children %d, windowed %d (%.3f), recursive %d (%.3f)" %
          (full.nodes, win.nodes, win.nodes / full.nodes, rec.nodes, rec.nodes / full.nodes))
    assert win.nodes < full.nodes and rec.nodes < full.nodes
