"""Autotuner on the GPU: every candidate parameter set (block width, frame
placement, fastest-first threshold, warp-split threshold) solves the sample
with identical scores, the winners are cached, and the tuned options give
the oracle's scores on the whole batch."""
import numpy as np
import pytest

from gpuothello2_gb300 import autotune as at
from tests.test_oracle import golden_ref

pytestmark = pytest.mark.gpu

SPACE = (
    ("threads_per_block", (64, 128, 256)),
    ("smem_frames", (0, -1)),
    ("fastest_first_empties", (5, 6, 9)),
    ("help_min_empties", (7, -1)),
)


def test_tuned_parameters_keep_scores_exact(gpu, oracle, tmp_path):
    p, o = gpu.generate(7, 3072, 12, 14)
    path = str(tmp_path / "tuning.json")
    best, src = at.tune_batch(p, o, 14, sample=768, cache_path=path, space=SPACE)
    assert src == "tuned"
    data = at.load_cache(path)
    (entry,) = data.values()
    assert len(entry["candidates"]) == 1 + sum(len(v) - 1 for _, v in SPACE)
    print("tuned:", best, "candidates:", entry["candidates"])

    again, src = at.tune_batch(p, o, 14, sample=768, cache_path=path, space=SPACE)
    assert src == "cache" and again == best

    sc, _, _, st, _ = gpu.solve(p, o, 14, **at.to_options(best))
    osc, _, _, _ = oracle.solve_batch(p, o, 14, mode=1)
    assert np.array_equal(sc, osc)
    assert st.launches >= 4


@pytest.mark.parametrize("smem_frames", [-1, 0])
@pytest.mark.parametrize("threads", [64, 256])
def test_frame_placement_and_block_width_on_reference_scores(gpu, threads, smem_frames):
    p, o, scores, _ = golden_ref("c3_seed2_mixed")
    sc, _, _, _, _ = gpu.solve(p, o, 16, threads_per_block=threads, smem_frames=smem_frames)
    assert np.array_equal(sc.astype(int), scores)
