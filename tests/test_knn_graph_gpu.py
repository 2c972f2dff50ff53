"""All-pairs kNN graph of a brute-force index (SSGIndex::build_knn_graph,
src/index/ssg_idx.rs:69-98) on the GPU against the oracle's brute force."""
import numpy as np
import pytest

from tests.test_bf_gpu import same_up_to_ties

pytestmark = pytest.mark.gpu


def graph_oracle(oracle, X, k, mt):
    ids, d = oracle.bf_search(X, X, k + 1, mt)
    out_i = np.empty((X.shape[0], k), np.int64)
    out_d = np.empty((X.shape[0], k), np.float32)
    for n in range(X.shape[0]):
        keep = [j for j in range(k + 1) if ids[n, j] != n][:k]
        out_i[n], out_d[n] = ids[n, keep], d[n, keep]
    return out_i, out_d


@pytest.mark.parametrize("mt", [3, 1, 2])
def test_exact_graph_matches_oracle(hora, oracle, gpu, mt):
    rng = np.random.default_rng(mt)
    X = rng.standard_normal((1500, 16)).astype(np.float32)
    ix = hora.BruteForceIndex(16)
    ix.madd(X, np.arange(1500, dtype=np.uint64) * 7)  # user ids differ from rows
    ix.build(hora.Metric(mt))
    g = ix.knn_graph(10).astype(np.int64)
    assert g.shape == (1500, 10)
    asc = g[:, ::-1]  # the reference's order is farthest first
    assert not np.any(asc == np.arange(1500)[:, None])  # no self loops
    d = np.array([[oracle.metric(X[n], X[j], mt) for j in asc[n]] for n in range(1500)], np.float32)
    oi, od = graph_oracle(oracle, X, 10, mt)
    np.testing.assert_array_equal(d, od)
    same_up_to_ties(asc, d, oi, od)


def test_bf16_graph_recall(hora, oracle, gpu):
    rng = np.random.default_rng(9)
    cen = (rng.standard_normal((20, 32)) * 3).astype(np.float32)
    X = (cen[rng.integers(0, 20, 4000)] + rng.standard_normal((4000, 32))).astype(np.float32)
    ix = hora.BruteForceIndex(32)
    ix.madd(X, None)
    ix.build(hora.Metric.Euclidean)
    exact = ix.knn_graph(8)
    ix.set_option(hora.Option.PRECISION, 1)
    approx = ix.knn_graph(8)
    hit = sum(len(set(a) & set(b)) for a, b in zip(approx.tolist(), exact.tolist()))
    assert hit / exact.size >= 0.99


def test_graph_errors(hora, gpu):
    X = np.random.default_rng(1).standard_normal((50, 8)).astype(np.float32)
    ix = hora.BruteForceIndex(8)
    ix.madd(X, None)
    with pytest.raises(hora.HoraError):
        ix.knn_graph(5)  # not built
    ix.build(hora.Metric.Euclidean)
    with pytest.raises(hora.HoraError):
        ix.knn_graph(50)  # k must be below n
