"""hora_bf_search_noalloc: exact brute force for callers that cannot allocate
device memory (an engine that owns all device memory through its own pool,
or a latency-critical path where cudaMalloc would synchronise the device).

The entry point takes device buffers only and keeps its scratch in a fixed
file-scope device array.  Its results must equal hora_search's on the same
inputs and the oracle's (distances bit for bit, ids up to ties), on two calls
in a row (the array keeps the previous call's contents, so the second call
checks that everything that must start empty is reset).  The shapes cover
fewer rows than k, fewer rows than the first chunk, a row count that is not a
multiple of the tile, and a base ordered so that every chunk offers more
candidates than a query can hold (the overflow rescan).  This file is
collected last so a stop-at-first-failure run has already run every other
test."""
import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NO_ID = np.iinfo(np.uint64).max


def _p(t):
    return C.c_void_p(t.data_ptr())


def _run_noalloc(hora, base, q, k, metric, calls=2):
    """Calls the entry point `calls` times on the same device buffers (the
    outputs poisoned before each call) and returns the host results of each."""
    import torch
    dbase = torch.from_numpy(base).cuda()
    dq = torch.from_numpy(q).cuda()
    nq = q.shape[0]
    ids = torch.empty((nq, k), dtype=torch.int64, device="cuda")
    dist = torch.empty((nq, k), dtype=torch.float32, device="cuda")
    lib = hora.lib()
    out = []
    for _ in range(calls):
        ids.fill_(-7)
        dist.fill_(float("nan"))
        rc = lib.hora_bf_search_noalloc(_p(dbase), base.shape[0], base.shape[1], _p(dq), nq, k,
                                        metric, _p(ids), _p(dist), None)
        assert rc == 0, lib.hora_last_error()
        torch.cuda.synchronize()
        out.append((ids.cpu().numpy().view(np.uint64).copy(), dist.cpu().numpy().copy()))
    return out


def _check(hora, oracle, base, q, k, metric):
    from test_bf_gpu import same_up_to_ties
    ix = hora.BruteForceIndex(base.shape[1])
    ix.madd(base, np.arange(base.shape[0], dtype=np.uint64))
    ix.build(hora.Metric(metric))
    ref_ids, ref_d = ix.search_batch(q, k)
    oi, od = oracle.bf_search(base, q, k, metric, threads=os.cpu_count() or 4)
    for call, (ids, dist) in enumerate(_run_noalloc(hora, base, q, k, metric)):
        # same kernels and the same (distance, row) order as hora_search: exact equality
        np.testing.assert_array_equal(dist, ref_d, err_msg=f"call {call}")
        np.testing.assert_array_equal(ids, ref_ids, err_msg=f"call {call}")
        # the oracle's restatement of the reference scan: distances bit for bit,
        # ids equal except at ties; empty slots past n are (NO_ID, +inf) here
        # and (-1, +inf) there
        np.testing.assert_array_equal(dist, od, err_msg=f"call {call}")
        gi = np.where(ids == NO_ID, -1, ids.astype(np.int64))
        assert ((gi == -1) == (oi == -1)).all()
        same_up_to_ties(gi, dist, oi, od)


@pytest.mark.parametrize("metric", [3, 1, 2])
def test_noalloc_matches_search_and_oracle(hora, oracle, gpu, metric):
    rng = np.random.default_rng(100 + metric)
    base = (rng.standard_normal((20000, 64)) * 10).astype(np.float32)
    q = (rng.standard_normal((256, 64)) * 10).astype(np.float32)
    _check(hora, oracle, base, q, 64, metric)


@pytest.mark.parametrize("n,dim,nq,k", [
    (40, 16, 17, 64),       # fewer rows than k: the tail is padding
    (700, 8, 256, 10),      # fewer rows than the dense first chunk
    (13337, 12, 33, 64),    # rows not a multiple of the 128-row tile or any chunk
    (1025, 4, 1, 1),        # one row past the first chunk, k = 1
])
def test_noalloc_shapes(hora, oracle, gpu, n, dim, nq, k):
    rng = np.random.default_rng(n + dim)
    base = (rng.standard_normal((n, dim)) * 10).astype(np.float32)
    q = (rng.standard_normal((nq, dim)) * 10).astype(np.float32)
    for metric in (3, 1, 2):
        _check(hora, oracle, base, q, k, metric)


@pytest.mark.parametrize("metric", [3, 1, 2])
def test_noalloc_overflow_rescan(hora, oracle, gpu, metric):
    """Rows ordered from farthest to nearest for every query: each filter
    chunk offers all of its rows (more than the 1,024 candidates a query
    holds), so the overflow collection, the query list and the deduplicating
    rescans run, twice in a row."""
    n, dim = 12000, 64
    u = np.ones(dim, np.float32) / np.float32(np.sqrt(dim))
    t = (1.0 + 0.01 * (n - np.arange(n))).astype(np.float32)
    base = (t[:, None] * u[None, :]).astype(np.float32)
    rng = np.random.default_rng(7)
    q = (rng.standard_normal((64, dim)) * 1e-3).astype(np.float32)
    if metric == 2:  # DotProduct ascends +<q, x> = t <q, u>: queries along +u
        q = (q + u[None, :]).astype(np.float32)
    # the premise: later rows are closer, for every query
    d_first = [oracle.metric(q[0], base[i], metric) for i in (0, n // 2, n - 1)]
    assert d_first[0] > d_first[1] > d_first[2]
    _check(hora, oracle, base, q, 64, metric)


def test_noalloc_rejects_non_finite_input(hora, gpu):
    import torch
    lib = hora.lib()
    base = torch.randn((3000, 8), device="cuda")
    q = torch.randn((5, 8), device="cuda")
    ids = torch.empty((5, 4), dtype=torch.int64, device="cuda")
    dist = torch.empty((5, 4), dtype=torch.float32, device="cuda")
    q[3, 2] = float("nan")
    rc = lib.hora_bf_search_noalloc(_p(base), 3000, 8, _p(q), 5, 4, 3, _p(ids), _p(dist), None)
    assert rc == -5, lib.hora_last_error()
    q[3, 2] = 0.0
    base[2999, 7] = float("inf")
    rc = lib.hora_bf_search_noalloc(_p(base), 3000, 8, _p(q), 5, 4, 3, _p(ids), _p(dist), None)
    assert rc == -5, lib.hora_last_error()
    base[2999, 7] = 0.0
    rc = lib.hora_bf_search_noalloc(_p(base), 3000, 8, _p(q), 5, 4, 3, _p(ids), _p(dist), None)
    assert rc == 0, lib.hora_last_error()


def test_noalloc_rejects_host_buffers(hora, gpu):
    import torch
    lib = hora.lib()
    hbase = np.zeros((100, 8), np.float32)
    dbase = torch.zeros((100, 8), device="cuda")
    dq = torch.zeros((4, 8), device="cuda")
    ids = torch.empty((4, 2), dtype=torch.int64, device="cuda")
    dist = torch.empty((4, 2), dtype=torch.float32, device="cuda")
    rc = lib.hora_bf_search_noalloc(hbase.ctypes.data_as(C.c_void_p), 100, 8, _p(dq), 4, 2, 3,
                                    _p(ids), _p(dist), None)
    assert rc == -1 and b"current device" in lib.hora_last_error()
    rc = lib.hora_bf_search_noalloc(_p(dbase), 100, 8, _p(dq), 4, 2, 3, _p(ids), _p(dist), None)
    assert rc == 0, lib.hora_last_error()


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
