"""hora_bf_search_noalloc: exact brute force for callers that cannot allocate
device memory (an engine that owns all device memory through its own pool,
or a latency-critical path where cudaMalloc would synchronise the device).

The entry point takes device buffers only and keeps its scratch in a fixed
file-scope device array.  Its results must equal hora_search's on the same
inputs, on two calls in a row (the array keeps the previous call's contents,
so the second call checks that everything that must start empty is reset).
This file is collected last so a stop-at-first-failure run has already run
every other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _p(t):
    return C.c_void_p(t.data_ptr())


@pytest.mark.parametrize("metric", [3, 1, 2])
def test_noalloc_matches_search(hora, gpu, metric):
    import torch
    rng = np.random.default_rng(100 + metric)
    base = (rng.standard_normal((20000, 64)) * 10).astype(np.float32)
    q = (rng.standard_normal((256, 64)) * 10).astype(np.float32)
    k = 64
    ix = hora.BruteForceIndex(64)
    ix.madd(base, np.arange(base.shape[0], dtype=np.uint64))
    ix.build(hora.Metric(metric))
    ref_ids, ref_d = ix.search_batch(q, k)

    dbase = torch.from_numpy(base).cuda()
    dq = torch.from_numpy(q).cuda()
    ids = torch.empty((256, k), dtype=torch.int64, device="cuda")
    dist = torch.empty((256, k), dtype=torch.float32, device="cuda")
    lib = hora.lib()
    for call in range(2):
        ids.fill_(-7)
        dist.fill_(float("nan"))
        rc = lib.hora_bf_search_noalloc(_p(dbase), base.shape[0], 64, _p(dq), 256, k, metric,
                                        _p(ids), _p(dist), None)
        assert rc == 0, lib.hora_last_error()
        torch.cuda.synchronize()
        # same kernels and the same (distance, row) order: exact equality
        np.testing.assert_array_equal(dist.cpu().numpy(), ref_d, err_msg=f"call {call}")
        np.testing.assert_array_equal(ids.cpu().numpy().view(np.uint64), ref_ids,
                                      err_msg=f"call {call}")


def test_noalloc_rejects_sizes_beyond_maximum(hora, gpu):
    import torch
    lib = hora.lib()
    dbase = torch.zeros((100, 8), device="cuda")
    dq = torch.zeros((300, 8), device="cuda")
    ids = torch.empty((300, 65), dtype=torch.int64, device="cuda")
    dist = torch.empty((300, 65), dtype=torch.float32, device="cuda")
    rc = lib.hora_bf_search_noalloc(_p(dbase), 100, 8, _p(dq), 300, 10, 3, _p(ids), _p(dist), None)
    assert rc == -3 and b"256 queries" in lib.hora_last_error()
    rc = lib.hora_bf_search_noalloc(_p(dbase), 100, 8, _p(dq), 10, 65, 3, _p(ids), _p(dist), None)
    assert rc == -3 and b"k must be <= 64" in lib.hora_last_error()
