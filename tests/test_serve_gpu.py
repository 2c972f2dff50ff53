"""Serving loop: requests of uneven batch size, k and index, submitted while
others run, admitted by HBM budget, continuously batched; every result must
equal the same request run alone (all paths are deterministic per query)."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _indexes(hora):
    from hora_gb300 import synth
    X = synth.mixture(100_000, 64, 256, stream=61)
    bf = hora.BruteForceIndex(64)
    bf.madd(X, None)
    bf.build(hora.Metric.Euclidean)
    iv = hora.IVFPQIndex(64, hora.IVFPQParams(n_sub=16, sub_bits=8, n_kmeans_center=128,
                                              search_n_center=8, train_epoch=5))
    iv.madd(X, None)
    iv.build(hora.Metric.Euclidean)
    iv.set_option(hora.Option.IVF_RERANK, 128)
    return X, [bf, iv]


def test_mix_equals_alone(hora, gpu):
    from hora_gb300 import synth
    X, idx = _indexes(hora)
    rng = np.random.default_rng(3)
    reqs = []
    for i in range(120):
        nq = int(np.exp(rng.uniform(0, np.log(256))))  # log-uniform 1..256
        k = int(rng.choice([1, 10, 100]))
        which = int(rng.integers(0, 2))
        q = synth.mixture(nq, 64, 256, stream=1000 + i)
        reqs.append((which, q, k))
    srv = hora.Server(idx, n_slots=4, hbm_budget_bytes=2 << 30)
    out = [None] * len(reqs)

    def client(lo, hi):
        tickets = [(j, srv.submit(reqs[j][0], reqs[j][1], reqs[j][2])) for j in range(lo, hi)]
        for j, t in tickets:
            out[j] = srv.wait(t)

    th = [threading.Thread(target=client, args=(a, a + 30)) for a in range(0, 120, 30)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    st = srv.stats()
    assert st["completed"] == 120 and st["p99_ms"] >= st["p50_ms"] > 0
    assert st["max_admitted_bytes"] <= 2 << 30
    srv.close()
    for j, (which, q, k) in enumerate(reqs):
        ids, dist = idx[which].search_batch(q, k)
        np.testing.assert_array_equal(out[j][0], ids, err_msg=f"request {j}")
        np.testing.assert_array_equal(out[j][1], dist, err_msg=f"request {j}")


def test_budget_rejects_and_limits(hora, gpu):
    X, idx = _indexes(hora)
    srv = hora.Server(idx[:1], n_slots=2, hbm_budget_bytes=64 << 20)
    with pytest.raises(hora.HoraError) as e:
        srv.submit(0, X[:4096], 100)  # working set above 64 MiB
    assert e.value.code == -6
    tickets = [srv.submit(0, X[i * 50:(i + 1) * 50], 10) for i in range(20)]
    for t in tickets:
        ids, d, lat = srv.wait(t)
        assert lat > 0
    st = srv.stats()
    assert st["rejected"] == 1 and st["max_admitted_bytes"] <= 64 << 20
    srv.close()


def test_mixed_k_batches_and_byte_estimate(hora, gpu):
    """Requests of different k on one index share a batch when their search
    keeps the same candidate width (here: exact brute force, and IVF-PQ with
    a rerank of 128 >= every k); each one's result equals the request run
    alone.  On fresh single-slot servers, the bytes a request is charged are
    at least what its search actually reserved in the slot's workspace."""
    from hora_gb300 import synth
    X, idx = _indexes(hora)
    srv = hora.Server(idx, n_slots=1, hbm_budget_bytes=4 << 30)
    reqs = [(w, synth.mixture(int(nq), 64, 256, stream=2000 + i), int(k))
            for i, (w, nq, k) in enumerate([(0, 7, 1), (0, 40, 100), (0, 3, 10), (1, 5, 10), (1, 64, 1),
                                            (1, 9, 100), (0, 100, 10), (1, 33, 100)] * 4)]
    tickets = [srv.submit(w, q, k) for w, q, k in reqs]
    outs = [srv.wait(t) for t in tickets]
    info = srv.info()
    srv.close()
    assert info["mixed_k_batches"] >= 1, info
    for (w, q, k), (ids, dist, _) in zip(reqs, outs):
        a_ids, a_d = idx[w].search_batch(q, k)
        np.testing.assert_array_equal(ids, a_ids)
        np.testing.assert_array_equal(dist, a_d)
    for w in (0, 1):
        for nq, k in ((1, 1), (256, 100), (2048, 10)):
            s = hora.Server([idx[w]], n_slots=1, hbm_budget_bytes=16 << 30)
            est = s.request_bytes(0, nq, k)
            s.wait(s.submit(0, X[:nq], k))
            used = s.info()["slot_workspace_bytes"][0]
            s.close()
            assert 0 < used <= est, (w, nq, k, used, est)
