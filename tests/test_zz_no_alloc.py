"""solve_batch_device_noalloc: the entry point for callers that cannot
allocate device memory (its scratch is a fixed array inside the library).

Collected last on purpose (file name), so that a run stopping at its first
failure has already run every other test.  Checks the entry point through
the C ABI against solve_batch_device on the same device arrays, exactly
(integer scores), on two calls in a row (the shared scratch keeps the last
call's contents, so the second call checks that it is cleared); against
the reference's own golden scores; and that oversized calls are refused
before any GPU work."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_matches_allocating_entry_point(gpu):
    torch = pytest.importorskip("torch")
    g = gpu
    L = g.lib()
    n, depth = 20000, 16
    dp = torch.empty(n, dtype=torch.int64, device="cuda")
    do = torch.empty(n, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    assert L.gpo_generate_device(2, 0, n, 8, 13, dp.data_ptr(), do.data_ptr(), stream) == 0
    ref = torch.zeros(n, dtype=torch.int8, device="cuda")
    opt = g.options(use_table=0)
    st = g.Stats()
    assert L.solve_batch_device(dp.data_ptr(), do.data_ptr(), n, depth, ref.data_ptr(), None,
                                None, ctypes.byref(opt), ctypes.byref(st), stream) == 0
    want = ref.cpu().numpy()
    for call in range(2):
        out = torch.full((n,), 99, dtype=torch.int8, device="cuda")
        rc = L.solve_batch_device_noalloc(dp.data_ptr(), do.data_ptr(), n, depth, out.data_ptr(),
                                          stream)
        assert rc == 0, g.strerror(rc)
        assert np.array_equal(out.cpu().numpy(), want), "call %d" % call


def test_noalloc_matches_reference_scores(gpu):
    torch = pytest.importorskip("torch")
    from tests.test_oracle import golden_ref

    L = gpu.lib()
    stream = torch.cuda.current_stream().cuda_stream
    for name, depth in (("c3_seed2_mixed", 16), ("c1_seed0_e10", 10)):
        p, o, scores, _ = golden_ref(name)
        dp = torch.from_numpy(p.view(np.int64)).cuda()
        do = torch.from_numpy(o.view(np.int64)).cuda()
        out = torch.full((len(p),), 99, dtype=torch.int8, device="cuda")
        rc = L.solve_batch_device_noalloc(dp.data_ptr(), do.data_ptr(), len(p), depth,
                                          out.data_ptr(), stream)
        assert rc == 0, gpu.strerror(rc)
        assert np.array_equal(out.cpu().numpy().astype(int), scores), name


def test_noalloc_rejects_sizes_beyond_its_limits(gpu):
    L = gpu.lib()
    assert L.solve_batch_device_noalloc(1, 1, (1 << 20) + 1, 16, 1, None) == gpu.GPO_ERR_ARG
    assert L.solve_batch_device_noalloc(1, 1, 16, 17, 1, None) == gpu.GPO_ERR_DEPTH
    assert L.solve_batch_device_noalloc(None, None, 0, 16, None, None) == 0
