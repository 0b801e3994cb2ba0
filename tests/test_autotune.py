"""Autotuner host logic on CPU: the coordinate descent, the exactness guard,
the tuning cache and the sample selection, with a synthetic cost in place of
GPU timing (the scores come from the oracle, so the guard sees real ones)."""
import json

import numpy as np
import pytest

from gpuothello2_gb300 import autotune as at


def synthetic_cost(params):
    # separable, minimum at threads 256, smem -1, ff 8, table from 9, help from 6
    t = {64: 3.0, 128: 2.0, 256: 1.0}[params["threads_per_block"]]
    t += {0: 0.5, -1: 0.0}[params["smem_frames"]]
    t += abs(params["fastest_first_empties"] - 8) * 0.25
    t += abs(params["table_min_empties"] - 9) * 0.1
    t += {6: 0.0, 7: 0.05, 9: 0.1, -1: 0.2}[params["help_min_empties"]]
    return t


def test_coordinate_descent_finds_the_separable_minimum():
    calls = []

    def measure(prm):
        calls.append(prm)
        return synthetic_cost(prm), np.zeros(4, np.int8)

    best, t, hist = at.coordinate_descent(measure)
    assert best == {"threads_per_block": 256, "smem_frames": -1, "fastest_first_empties": 8,
                    "table_min_empties": 9, "help_min_empties": 6}
    assert t == pytest.approx(synthetic_cost(best))
    # the start plus every other value of every parameter, each timed once
    assert len(calls) == 1 + sum(len(v) - 1 for _, v in at.SPACE)
    assert len(hist) == len(calls)


def test_repeats_keep_the_fastest_run():
    times = iter([5.0, 3.0, 4.0] + [9.0] * 100)

    def measure(prm):
        return next(times), np.zeros(1, np.int8)

    _, t, hist = at.coordinate_descent(measure, space=(), repeats=3)
    assert t == 3.0 and hist[0][1] == 3.0


def test_a_parameter_that_changes_a_score_stops_tuning():
    def measure(prm):
        s = np.array([2, -4, 0], np.int8)
        if prm["fastest_first_empties"] == 8:
            s[1] = -6
        return 1.0, s

    with pytest.raises(at.TuningError):
        at.coordinate_descent(measure)


def test_tune_batch_caches_by_device_depth_and_empties(oracle, tmp_path):
    p, o = oracle.generate(2, 600, 8, 10)
    ref, _, _, _ = oracle.solve_batch(p, o, 10, mode=1, threads=1)
    seen = []

    def measure(prm, sp, so, depth):
        seen.append(len(sp))
        sc, _, _, _ = oracle.solve_batch(sp, so, depth, mode=1, threads=1)
        return synthetic_cost(prm), sc

    path = tmp_path / "tuning.json"
    best, src = at.tune_batch(p, o, 10, sample=200, cache_path=str(path), measure=measure,
                              device=("GB300-test", 152))
    assert src == "tuned" and best["threads_per_block"] == 256
    assert set(seen) == {200}
    data = json.loads(path.read_text())
    e = at.empties(p[at.sample_indices(600, 200)], o[at.sample_indices(600, 200)])
    key = at.cache_key("GB300-test", 152, 10, int(e.min()), int(e.max()))
    assert list(data) == [key]
    assert data[key]["params"] == best and data[key]["sample"] == 200

    # second call: from the cache, nothing timed
    seen.clear()
    again, src = at.tune_batch(p, o, 10, sample=200, cache_path=str(path), measure=measure,
                               device=("GB300-test", 152))
    assert src == "cache" and again == best and not seen
    # another device or depth is another key
    _, src = at.tune_batch(p, o, 12, sample=200, cache_path=str(path), measure=measure,
                           device=("GB300-test", 152))
    assert src == "tuned"
    assert len(json.loads(path.read_text())) == 2
    # the tuned sample's scores are the oracle's
    sc, _, _, _ = oracle.solve_batch(p, o, 10, mode=1, threads=1)
    assert np.array_equal(sc, ref)


def test_sample_keeps_the_batch_mix(oracle):
    p, o = oracle.generate(2, 4096, 8, 16)
    idx = at.sample_indices(4096, 512)
    assert len(idx) == 512 and idx[0] == 0 and np.all(np.diff(idx) == 8)
    e_all, e_s = at.empties(p, o), at.empties(p[idx], o[idx])
    assert e_s.min() == e_all.min() == 8 and e_s.max() == e_all.max() == 16
    assert np.array_equal(at.sample_indices(10, 64), np.arange(10))


def test_empties_counts_unoccupied_squares():
    p = np.array([0x0000000810000000, 0, 0xFFFFFFFFFFFFFFFF], np.uint64)
    o = np.array([0x0000001008000000, 0, 0], np.uint64)
    assert list(at.empties(p, o)) == [60, 64, 0]


def test_every_candidate_is_a_valid_option_set(built):
    import gpuothello2_gb300 as g

    for name, values in at.SPACE:
        for v in values:
            prm = dict(at.DEFAULTS)
            prm[name] = v
            opt = g.options(**at.to_options(prm))
            assert getattr(opt, name) == v
            tpb = opt.threads_per_block
            assert 32 <= tpb <= 256 and tpb % 32 == 0
    assert at.cache_key("x", 1, 16, 8, 16) == "x|sm1|depth16|e8-16"


def test_unreadable_cache_is_empty(tmp_path):
    bad = tmp_path / "t.json"
    bad.write_text("{not json")
    assert at.load_cache(str(bad)) == {}
    assert at.load_cache(str(tmp_path / "missing.json")) == {}
    at.save_cache(str(tmp_path / "sub" / "t.json"), {"k": {"params": {}}})
    assert at.load_cache(str(tmp_path / "sub" / "t.json")) == {"k": {"params": {}}}
