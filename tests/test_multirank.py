"""The bench's multi-rank path on CPU: two gloo ranks each take their slice
of the workload stream (bench.slice_first), solve it with the oracle, and
reduce their times with bench.max_over_ranks.  The slices must be disjoint
and together equal the single-process stream, the gathered scores must equal
a single-process solve, and the reduced time must be the slowest rank's."""
import os
import socket

import numpy as np
import pytest

from tests.conftest import ROOT

torch = pytest.importorskip("torch")

N_PER_RANK, LO, HI, SEED, WORLD = 48, 8, 10, 2, 2


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_main(rank, world, port, oracle_lib, out_dir):
    import sys

    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    from tests.oracle_lib import Oracle

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        orc = Oracle(oracle_lib)
        first = bench.slice_first(rank, N_PER_RANK)
        p, o = orc.generate(SEED, N_PER_RANK, LO, HI, first=first)
        sc, _, _, _ = orc.solve_batch(p, o, HI, mode=1, threads=1)
        # a distinct, known per-rank time so the reduction is checkable
        my_seconds = 1.0 + rank
        slowest = bench.max_over_ranks(my_seconds, world)
        gathered = [None] * world
        dist.all_gather_object(gathered, (first, p.tolist(), o.tolist(), sc.tolist()))
        if rank == 0:
            np.save(os.path.join(out_dir, "slowest.npy"), np.array([slowest]))
            for r, (f, pp, oo, ss) in enumerate(gathered):
                np.save(os.path.join(out_dir, "r%d.npy" % r),
                        np.array([pp, oo, ss], dtype=object), allow_pickle=True)
                np.save(os.path.join(out_dir, "first%d.npy" % r), np.array([f]))
    finally:
        dist.destroy_process_group()


def test_two_ranks_shard_the_stream_and_reduce_the_slowest_time(built, oracle, tmp_path):
    import torch.multiprocessing as mp

    import bench

    mp.start_processes(rank_main, args=(WORLD, free_port(), built.ORACLE_LIB, str(tmp_path)),
                       nprocs=WORLD, join=True, start_method="spawn")
    slowest = float(np.load(tmp_path / "slowest.npy")[0])
    assert slowest == 1.0 + (WORLD - 1)
    assert bench.job_value(WORLD, N_PER_RANK, 1, slowest) == WORLD * N_PER_RANK / slowest

    ps, os_, ss = [], [], []
    for r in range(WORLD):
        assert int(np.load(tmp_path / ("first%d.npy" % r))[0]) == r * N_PER_RANK
        pp, oo, sc = np.load(tmp_path / ("r%d.npy" % r), allow_pickle=True)
        ps += list(pp)
        os_ += list(oo)
        ss += list(sc)
    p1, o1 = oracle.generate(SEED, WORLD * N_PER_RANK, LO, HI)
    assert np.array_equal(np.array(ps, np.uint64), p1)
    assert np.array_equal(np.array(os_, np.uint64), o1)
    s1, _, _, _ = oracle.solve_batch(p1, o1, HI, mode=1, threads=1)
    assert np.array_equal(np.array(ss, np.int8), s1)
