"""Mixed-precision brute force (tcgen05 BF16 / FP8 scoring + exact FP32 rerank).

The approximate forms must (a) return exact FP32 distances (the rerank uses
the reference's op order), (b) reach the recall targets against the exact
form on the benchmark's data distribution, and (c) handle ragged shapes and
candidate overflow like the exact path."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def recall(ids, exact, r):
    return np.mean([len(set(a[:r].tolist()) & set(b[:r].tolist())) / r for a, b in zip(ids, exact)])


def bf(hora, base, mt, prec=0):
    ix = hora.BruteForceIndex(base.shape[1])
    ix.madd(base, np.arange(base.shape[0], dtype=np.uint64))
    ix.build(hora.Metric(mt))
    ix.set_option(hora.Option.PRECISION, prec)
    return ix


@pytest.mark.parametrize("prec,r10,r100", [(1, 0.99, 0.98), (2, 0.97, 0.95)])
def test_recall_and_exact_distances_mixture(hora, oracle, gpu, prec, r10, r100):
    from hora_gb300 import synth
    base = synth.mixture(200_000, 128, 1024, stream=21)
    q = synth.mixture(500, 128, 1024, stream=22)
    ix = bf(hora, base, 3)
    e_ids, e_d = ix.search_batch(q, 100)
    ix.set_option(hora.Option.PRECISION, prec)
    ids, d = ix.search_batch(q, 100)
    assert recall(ids, e_ids, 10) >= r10
    assert recall(ids, e_ids, 100) >= r100
    assert (np.diff(d, axis=1) >= 0).all()
    # every returned distance is the exact FP32 one
    for qi in range(0, 500, 50):
        for j in (0, 7, 99):
            assert d[qi, j] == oracle.metric(q[qi], base[int(ids[qi, j])], 3)


@pytest.mark.parametrize("mt", [2, 4])
@pytest.mark.parametrize("prec", [1, 2])
def test_ip_and_cosine(hora, oracle, gpu, mt, prec):
    from hora_gb300 import synth
    base = synth.normal(50_000, 96, 1.0, stream=31)
    q = synth.normal(200, 96, 1.0, stream=32)
    ix = bf(hora, base, mt)
    e_ids, e_d = ix.search_batch(q, 20)
    ix.set_option(hora.Option.PRECISION, prec)
    ix.set_option(hora.Option.RERANK, 200)
    ids, d = ix.search_batch(q, 20)
    assert recall(ids, e_ids, 10) >= 0.95
    j = 0
    assert d[3, j] == oracle.metric(q[3], base[int(ids[3, j])], mt)


@pytest.mark.parametrize("n,dim,nq,k", [(300, 64, 1, 5), (1000, 100, 129, 10), (257, 128, 7, 300),
                                        (70_000, 32, 300, 1), (5000, 200, 50, 10)])
@pytest.mark.parametrize("prec", [1, 2])
def test_ragged_shapes(hora, oracle, gpu, n, dim, nq, k, prec):
    rng = np.random.default_rng(n + dim + nq)
    base = rng.standard_normal((n, dim)).astype(np.float32)
    q = rng.standard_normal((nq, dim)).astype(np.float32)
    ix = bf(hora, base, 3)
    e_ids, e_d = ix.search_batch(q, k)
    ix.set_option(hora.Option.PRECISION, prec)
    ids, d = ix.search_batch(q, k)
    m = min(k, n)
    assert (ids[:, m:] == hora.NO_ID).all()
    assert recall(ids[:, :m], e_ids[:, :m], min(m, 10)) >= 0.9


def test_overflow_rescan_with_ties(hora, oracle, gpu):
    rng = np.random.default_rng(17)
    base = np.repeat(rng.standard_normal((50, 64)).astype(np.float32), 400, axis=0)
    rng.shuffle(base)
    q = rng.standard_normal((40, 64)).astype(np.float32)
    ix = bf(hora, base, 3)
    e_ids, e_d = ix.search_batch(q, 50)
    ix.set_option(hora.Option.PRECISION, 1)
    ix.set_option(hora.Option.CAND_CAP, 256)
    ix.set_option(hora.Option.RERANK, 100)
    ids, d = ix.search_batch(q, 50)
    np.testing.assert_array_equal(d, e_d)


def test_manhattan_runs_exact(hora, oracle, gpu):
    rng = np.random.default_rng(3)
    base = rng.standard_normal((4000, 64)).astype(np.float32)
    q = rng.standard_normal((30, 64)).astype(np.float32)
    ix = bf(hora, base, 1, prec=1)
    ids, d = ix.search_batch(q, 10)
    oi, od = oracle.bf_search(base, q, 10, 1)
    np.testing.assert_array_equal(d, od)
