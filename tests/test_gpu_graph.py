"""Repeated batches as a CUDA graph (gpo_graph_*): the captured batched solve
replayed on the same device arrays gives the reference's golden scores, on
two replays in a row and after the inputs are refilled in place."""
import ctypes

import numpy as np
import pytest

from tests.test_oracle import golden_ref

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,depth", [("c1_seed0_e10", 10), ("c3_seed2_mixed", 16)])
def test_graph_replays_match_reference(gpu, oracle, name, depth):
    torch = pytest.importorskip("torch")
    g = gpu
    L = g.lib()
    p, o, scores, _ = golden_ref(name)
    n = len(p)
    dp = torch.from_numpy(p.view(np.int64)).cuda()
    do = torch.from_numpy(o.view(np.int64)).cuda()
    ds = torch.full((n,), 99, dtype=torch.int8, device="cuda")
    stream = torch.cuda.current_stream()
    handle = ctypes.c_void_p()
    opt = g.options(use_learned=0, table_bits=20)
    rc = L.gpo_graph_create(dp.data_ptr(), do.data_ptr(), n, depth, ds.data_ptr(),
                            ctypes.byref(opt), ctypes.byref(handle))
    assert rc == 0, g.strerror(rc)
    try:
        for _ in range(2):
            ds.fill_(99)
            assert L.gpo_graph_launch(handle, stream.cuda_stream) == 0
            stream.synchronize()
            st = g.Stats()
            assert L.gpo_graph_stats(handle, ctypes.byref(st)) == 0
            assert np.array_equal(ds.cpu().numpy().astype(int), scores)
            assert st.nodes > 0 and st.launches == 4 and st.table_bits == 20
        # a new batch of the same size in the same arrays
        q, r = oracle.generate(21, n, 8, min(depth, 12))
        dp.copy_(torch.from_numpy(q.view(np.int64)))
        do.copy_(torch.from_numpy(r.view(np.int64)))
        assert L.gpo_graph_launch(handle, stream.cuda_stream) == 0
        stream.synchronize()
        want, _, _, _ = oracle.solve_batch(q, r, mode=1)
        assert np.array_equal(ds.cpu().numpy(), want)
    finally:
        L.gpo_graph_destroy(handle)


def test_graph_rejects_learned_ordering(gpu):
    torch = pytest.importorskip("torch")
    L = gpu.lib()
    d = torch.zeros(64, dtype=torch.int64, device="cuda")
    s = torch.zeros(64, dtype=torch.int8, device="cuda")
    handle = ctypes.c_void_p()
    opt = gpu.options(use_learned=1)
    assert L.gpo_graph_create(d.data_ptr(), d.data_ptr(), 64, 10, s.data_ptr(), ctypes.byref(opt),
                              ctypes.byref(handle)) == gpu.GPO_ERR_ARG
