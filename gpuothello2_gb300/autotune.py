"""Autotuner for the batched solver's launch and search parameters.

The reference fixes its launch shape and stack split as compile-time
constants (nodesPerBlock = 64 and chunk_size = 2048, alphabeta.cuh:4-5;
lower_stack_depth = 9, solver.cu:9).  Here they are gpo_options fields,
chosen per GPU and workload by timing candidates on a bounded sample of the
caller's batch:

  threads_per_block      block width of the persistent search grid
  smem_frames            stack placement: frames in shared memory when they
                         fit (0) or every frame in the global array (-1)
  fastest_first_empties  the empty count from which moves are ordered by
                         the opponent's reply count
  table_min_empties      the empty count from which nodes use the
                         transposition table
  help_min_empties       the warp-split threshold: the empty count a node
                         needs before idle lanes of its warp take its moves
                         (-1 = no helping)

Search: coordinate descent from the library defaults, one parameter at a
time, each candidate timed on the same sample (best of `repeats` runs).
Every candidate's scores must equal the first run's -- the parameters change
only speed, so a different score is a bug and tuning stops with an error.
Winners are kept in a JSON tuning cache keyed by GPU name, SM count, depth
and the sample's empty-count range; a cached key is returned without timing.
"""
import json
import os
import tempfile
import time

import numpy as np

DEFAULTS = {
    "threads_per_block": 128,
    "smem_frames": 0,
    "fastest_first_empties": 6,
    "table_min_empties": 9,
    "help_min_empties": 7,
}

SPACE = (
    ("threads_per_block", (64, 128, 256)),
    ("smem_frames", (0, -1)),
    ("fastest_first_empties", (5, 6, 7, 8)),
    ("table_min_empties", (6, 7, 8, 9)),
    ("help_min_empties", (6, 7, 9, -1)),
)


class TuningError(RuntimeError):
    pass


def default_cache_path():
    """GPO_TUNING_CACHE, else ~/.cache/gpuothello2/tuning.json."""
    env = os.environ.get("GPO_TUNING_CACHE")
    if env:
        return env
    return os.path.join(os.path.expanduser("~"), ".cache", "gpuothello2", "tuning.json")


def cache_key(device_name, sms, depth, min_empties, max_empties):
    return "%s|sm%d|depth%d|e%d-%d" % (device_name, sms, depth, min_empties, max_empties)


def load_cache(path):
    try:
        with open(path) as f:
            data = json.load(f)
    except (OSError, ValueError):
        return {}
    return data if isinstance(data, dict) else {}


def save_cache(path, data):
    """Writes the cache atomically (temporary file + rename)."""
    d = os.path.dirname(os.path.abspath(path))
    os.makedirs(d, exist_ok=True)
    fd, tmp = tempfile.mkstemp(prefix=".tuning", dir=d)
    try:
        with os.fdopen(fd, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except BaseException:
        if os.path.exists(tmp):
            os.unlink(tmp)
        raise


def coordinate_descent(measure, space=SPACE, start=None, repeats=1):
    """Minimises measure(params) -> (seconds, scores) one parameter at a
    time.  Returns (best params, best seconds, history of (params, seconds)).
    Raises TuningError if a candidate's scores differ from the first run's."""
    best = dict(DEFAULTS if start is None else start)
    history = []
    reference = None
    cache = {}

    def run(params):
        key = tuple(sorted(params.items()))
        if key in cache:
            return cache[key]
        t_best = None
        for _ in range(max(1, repeats)):
            seconds, scores = measure(dict(params))
            scores = np.asarray(scores)
            nonlocal reference
            if reference is None:
                reference = scores.copy()
            elif not np.array_equal(scores, reference):
                raise TuningError("parameters %r changed a score" % (params,))
            t_best = seconds if t_best is None else min(t_best, seconds)
        history.append((dict(params), t_best))
        cache[key] = t_best
        return t_best

    best_t = run(best)
    for name, values in space:
        for v in values:
            if v == best.get(name):
                continue
            trial = dict(best)
            trial[name] = v
            t = run(trial)
            if t < best_t:
                best, best_t = trial, t
    return best, best_t, history


def sample_indices(n, sample):
    """Evenly strided indices of a batch: the sample keeps the batch's mix of
    empty counts (a prefix of a bucketed or sorted batch would not)."""
    if sample >= n:
        return np.arange(n)
    return (np.arange(sample, dtype=np.int64) * n) // sample


def empties(player, opp):
    occ = np.bitwise_or(np.asarray(player, np.uint64), np.asarray(opp, np.uint64))
    bits = np.unpackbits(occ.view(np.uint8).reshape(-1, 8), axis=1).sum(axis=1)
    return 64 - bits


def to_options(params):
    """gpo_options keyword arguments for a parameter dict."""
    return {k: int(v) for k, v in params.items()}


def tune_batch(player, opp, depth, sample=4096, cache_path=None, repeats=1, space=SPACE,
               measure=None, device=None, retune=False):
    """Tuned parameters for solving this batch at this depth on this GPU.

    measure(params, p, o, depth) -> (seconds, scores) times one solve of the
    sample (default: solve_batch_ex through the library, wall clock);
    device = (name, sms) (default: gpo_device_info).  Returns (params,
    source) with source "cache" or "tuned"."""
    p = np.ascontiguousarray(player, np.uint64)
    o = np.ascontiguousarray(opp, np.uint64)
    idx = sample_indices(len(p), sample)
    sp, so = p[idx], o[idx]
    e = empties(sp, so)
    if device is None:
        from . import device_info

        device = device_info()
    name, sms = device
    key = cache_key(name, sms, depth, int(e.min()) if len(e) else 0, int(e.max()) if len(e) else 0)
    path = cache_path or default_cache_path()
    data = load_cache(path)
    if not retune and key in data:
        return dict(data[key]["params"]), "cache"
    if measure is None:
        measure = measure_solve
    best, best_t, history = coordinate_descent(lambda prm: measure(prm, sp, so, depth), space,
                                               repeats=repeats)
    data = load_cache(path)
    data[key] = {"params": best, "seconds": best_t, "sample": int(len(sp)),
                 "candidates": [[prm, t] for prm, t in history]}
    save_cache(path, data)
    return best, "tuned"


def measure_solve(params, p, o, depth):
    """One solve of the sample through solve_batch_ex (synchronous), wall
    clock; the scores are returned for the exactness check."""
    from . import solve

    t0 = time.perf_counter()
    score, _, _, _, _ = solve(p, o, depth, **to_options(params))
    return time.perf_counter() - t0, score
