"""Exact FP32 brute force (Euclidean, DotProduct, CosineSimilarity) with the
BF16 tensor-core scan as a certified filter (HORA_OPT_EXACT_TC): the result must be the CUDA-core exact
scan's, bit for bit (distances, and ids including ties), on bases large
enough for pivot clusters, including the queries the certified pass hands
back to the CUDA-core scan (candidate overflow, duplicates at the k-th
distance)."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pair(hora, X, k, q, metric=None, **opts):
    import torch
    out = []
    for xtc in (1, 0):
        ix = hora.BruteForceIndex(X.shape[1])
        ix.madd(torch.from_numpy(X).cuda(), None)
        ix.build(hora.Metric.Euclidean if metric is None else metric)
        ix.set_option(hora.Option.EXACT_TC, xtc)
        for key, v in opts.items():
            ix.set_option(getattr(hora.Option, key), v)
        ids, d = ix.search_batch(q, k)
        info = json.loads(ix.idx_info())
        out.append((ids, d, info["last_threshold_probe"], info["last_fallback_queries"]))
        del ix
    return out


@pytest.mark.parametrize("k", [1, 10, 100, 256])
def test_exact_tc_equals_cuda_core_scan(hora, oracle, gpu, k):
    from hora_gb300 import synth
    X = synth.mixture(131_072, 128, 256, stream=71)
    q = synth.mixture(1_500, 128, 256, stream=72)
    (ia, da, pa, fa), (ib, db, pb, _) = _pair(hora, X, k, q)
    # the certified pass answers (nearly) every query itself; at k = 256 a
    # pivot cluster can hold fewer than k members and its queries go back to
    # the CUDA-core scan
    assert pa in (1, 2) and pb == 0, (pa, pb)
    if k <= 100:
        assert fa <= q.shape[0] // 50, fa
    np.testing.assert_array_equal(da, db)
    np.testing.assert_array_equal(ia, ib)
    # and the oracle's restatement of the reference scan, distances bit for bit
    oi, od = oracle.bf_search(X, q[:48], k, oracle.EUCLIDEAN, threads=os.cpu_count() or 4)
    np.testing.assert_array_equal(da[:48], od)


def test_exact_tc_overflow_and_ties_fall_back_exactly(hora, gpu):
    """A candidate capacity of 256 overflows for most queries at k = 100 (the
    certified window holds a few hundred rows), and 400 copies of one row
    tie at the same distance: both go back to the CUDA-core scan or are
    answered inside the window, with identical results either way."""
    from hora_gb300 import synth
    X = synth.mixture(100_000, 64, 128, stream=73)
    X[50_000:50_400] = X[7]
    q = np.concatenate([synth.mixture(600, 64, 128, stream=74), X[7:8] + 1e-3], axis=0).astype(np.float32)
    for cap in (256, 4096):
        (ia, da, pa, fa), (ib, db, _, _) = _pair(hora, X, 100, q, CAND_CAP=cap)
        assert pa in (1, 2)
        if cap == 256:
            assert fa > 0  # the overflowed queries went back to the CUDA-core scan
        np.testing.assert_array_equal(da, db)
        np.testing.assert_array_equal(ia, ib)


def test_exact_tc_small_base_uses_cuda_cores(hora, gpu):
    from hora_gb300 import synth
    X = synth.mixture(20_000, 32, 64, stream=75)
    (ia, da, pa, _), (ib, db, _, _) = _pair(hora, X, 10, X[:50])
    assert pa == 0
    np.testing.assert_array_equal(da, db)
    np.testing.assert_array_equal(ia, ib)


@pytest.mark.parametrize("k", [1, 10, 100, 256])
@pytest.mark.parametrize("mname", ["DotProduct", "CosineSimilarity"])
def test_exact_tc_dot_and_cosine_equal_cuda_core_scan(hora, oracle, gpu, k, mname):
    """DotProduct and CosineSimilarity through the certified pass: the keys
    are the scan's dot (of unit rows for the cosine), the bound is the
    windowed rerank's; the result is the CUDA-core scan's bit for bit and
    the oracle's distances bit for bit."""
    from hora_gb300 import synth
    X = synth.mixture(131_072, 96, 256, stream=76)
    q = synth.mixture(1_200, 96, 256, stream=77)
    mt = getattr(hora.Metric, mname)
    (ia, da, pa, fa), (ib, db, pb, _) = _pair(hora, X, k, q, metric=mt)
    assert pa in (1, 2) and pb == 0, (pa, pb)
    np.testing.assert_array_equal(da, db)
    np.testing.assert_array_equal(ia, ib)
    om = oracle.DOT if mname == "DotProduct" else oracle.COSINE
    oi, od = oracle.bf_search(X, q[:32], k, om, threads=os.cpu_count() or 4)
    np.testing.assert_array_equal(da[:32], od)


def test_exact_tc_cosine_fallback_queries_keep_their_norms(hora, gpu):
    """400 copies of one row and a candidate capacity of 256 at k = 100: the
    queries beside the copies keep more rows than the capacity and go back
    to the CUDA-core scan, which needs each gathered query's norm; the
    result is still the CUDA-core scan's."""
    from hora_gb300 import synth
    X = synth.mixture(100_000, 64, 128, stream=78)
    X[50_000:50_400] = X[7]
    q = np.concatenate([synth.mixture(400, 64, 128, stream=79) * 3.0, X[7:8] * 2.0 + 1e-3],
                       axis=0).astype(np.float32)
    (ia, da, pa, fa), (ib, db, _, _) = _pair(hora, X, 100, q, metric=hora.Metric.CosineSimilarity, CAND_CAP=256)
    assert pa == 2 and fa > 0, (pa, fa)
    np.testing.assert_array_equal(da, db)
    np.testing.assert_array_equal(ia, ib)
