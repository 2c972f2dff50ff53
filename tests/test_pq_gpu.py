"""Flat PQIndex (src/index/pq_idx.rs:21-265) on the GPU against the oracle.

- build: codebooks trained on the raw vectors with the build metric
  (train_center, pq_idx.rs:122-149) and the codes of every item equal the
  oracle's restatement bit for bit, for Euclidean, Manhattan and DotProduct;
- search: ADC distances equal the oracle's search_knn_adc (pq_idx.rs:165-193);
  ids equal up to ties;
- CosineSimilarity is rejected at build (the reference's metric is NaN there
  and its heap panics); dump/load keeps the trained index.
"""
import os
import tempfile

import numpy as np
import pytest

from tests.test_bf_gpu import same_up_to_ties

pytestmark = pytest.mark.gpu


def pq(hora, X, n_sub, bits, epochs, mt, seed=0x686F7261):
    ix = hora.PQIndex(X.shape[1], hora.PQParams(n_sub=n_sub, sub_bits=bits, train_epoch=epochs))
    ix.set_option(hora.Option.SEED, seed)
    ix.madd(X, np.arange(X.shape[0], dtype=np.uint64))
    ix.build(hora.Metric(mt))
    return ix


def data(seed, n=3000, d=24, centres=12):
    rng = np.random.default_rng(seed)
    cen = (rng.standard_normal((centres, d)) * 3).astype(np.float32)
    X = (cen[rng.integers(0, centres, n)] + rng.standard_normal((n, d))).astype(np.float32)
    q = (cen[rng.integers(0, centres, 40)] + rng.standard_normal((40, d))).astype(np.float32)
    return X, q


@pytest.mark.parametrize("mt", [3, 1, 2])
def test_build_and_search_match_oracle(hora, oracle, gpu, mt):
    X, q = data(70 + mt)
    ix = pq(hora, X, 6, 5, 6, mt)
    assert ix.name() == "PQIndex"
    ex = ix.export()
    ref = oracle.pq_build(X, 6, 5, 6, mt, 0x686F7261)
    # one list centred at zero, every item in insertion order
    np.testing.assert_array_equal(ex["centers"], np.zeros((1, X.shape[1]), np.float32))
    np.testing.assert_array_equal(ex["offsets"], [0, X.shape[0]])
    np.testing.assert_array_equal(ex["items"], np.arange(X.shape[0]))
    np.testing.assert_array_equal(ex["codebooks"][0], ref["codebooks"])
    np.testing.assert_array_equal(ex["codes"], ref["codes"])
    ids, d = ix.search_batch(q, 10)
    oi, od = oracle.pq_search(ref, q, 10)
    np.testing.assert_array_equal(d, od)
    same_up_to_ties(ids.astype(np.int64), d, oi, od)


def test_uneven_subspaces_and_8bit(hora, oracle, gpu):
    # dim 10 with 4 sub-quantizers: the reference's range formula leaves the
    # last dimensions uncoded (pq_idx.rs:75-88); 8-bit codes
    rng = np.random.default_rng(9)
    X = rng.standard_normal((2500, 10)).astype(np.float32)
    ix = pq(hora, X, 4, 8, 4, 3)
    ref = oracle.pq_build(X, 4, 8, 4, 3, 0x686F7261)
    ex = ix.export()
    np.testing.assert_array_equal(ex["codebooks"][0], ref["codebooks"])
    np.testing.assert_array_equal(ex["codes"], ref["codes"])
    q = rng.standard_normal((20, 10)).astype(np.float32)
    ids, d = ix.search_batch(q, 5)
    oi, od = oracle.pq_search(ref, q, 5)
    np.testing.assert_array_equal(d, od)
    same_up_to_ties(ids.astype(np.int64), d, oi, od)


def test_cosine_rejected(hora, gpu):
    X, _ = data(3, n=500)
    ix = hora.PQIndex(X.shape[1], hora.PQParams(n_sub=4, sub_bits=4, train_epoch=2))
    ix.madd(X, None)
    with pytest.raises(hora.HoraError):
        ix.build(hora.Metric.CosineSimilarity)


def test_rerank_returns_exact_distances(hora, oracle, gpu):
    X, q = data(11)
    ix = pq(hora, X, 6, 5, 6, 3)
    ix.set_option(hora.Option.IVF_RERANK, 200)
    ids, d = ix.search_batch(q, 10)
    for i in range(q.shape[0]):
        exact = [oracle.metric(q[i], X[int(j)], 3) for j in ids[i]]
        np.testing.assert_array_equal(d[i], np.array(exact, np.float32))


def test_dump_load_roundtrip(hora, gpu):
    X, q = data(5)
    ix = pq(hora, X, 6, 4, 4, 1)
    ids, d = ix.search_batch(q, 8)
    with tempfile.TemporaryDirectory() as t:
        path = os.path.join(t, "pq.hora")
        ix.dump(path)
        jx = hora.PQIndex.load(path)
    assert jx.name() == "PQIndex"
    ids2, d2 = jx.search_batch(q, 8)
    np.testing.assert_array_equal(d, d2)
    np.testing.assert_array_equal(ids, ids2)
