"""Brute-force parity on the GPU against the oracle, through the C ABI.

Exact FP32 form: distances are bit-identical to the oracle's restatement of
the reference's scalar loops (src/core/simd_metrics.rs), and the id lists
are equal except where distances tie (the reference evicts ties in heap
order, the GPU keeps the lower row)."""
import os
import tempfile

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")
METRICS = [("l2", 3), ("l1", 1), ("ip", 2), ("cos", 4)]


def same_up_to_ties(ids_a, d_a, ids_b, d_b, rtol=1e-6):
    """id sets equal except at ties within rtol relative distance."""
    for qa, da, qb, db in zip(ids_a, d_a, ids_b, d_b):
        m = np.isfinite(da)
        assert (np.isfinite(db) == m).all()
        if set(qa[m].tolist()) == set(qb[m].tolist()):
            continue
        kth = float(np.max(np.abs(da[m]))) if m.any() else 0.0
        diff = set(qa[m].tolist()) ^ set(qb[m].tolist())
        # every differing id must sit at the boundary distance
        bound = da[m][-1]
        for i in diff:
            pos_a = np.where(qa == i)[0]
            pos_b = np.where(qb == i)[0]
            d = da[pos_a[0]] if len(pos_a) else db[pos_b[0]]
            assert abs(d - bound) <= rtol * max(abs(bound), 1e-30) + 1e-30 * kth, (i, d, bound)


def bf(hora, base, mt, ids=None):
    ix = hora.BruteForceIndex(base.shape[1])
    ix.madd(base, np.arange(base.shape[0], dtype=np.uint64) if ids is None else ids)
    ix.build(hora.Metric(mt))
    return ix


def test_golden_fixture(hora, gpu):
    g = np.load(os.path.join(GOLD, "bf_small.npz"))
    for name, mt in METRICS:
        ix = bf(hora, g["base"], mt)
        ids, d = ix.search_batch(g["queries"], 5)
        np.testing.assert_array_equal(d, g[f"{name}_dist"])
        same_up_to_ties(ids.astype(np.int64), d, g[f"{name}_ids"], g[f"{name}_dist"])


@pytest.mark.parametrize("name,mt", METRICS)
def test_config1_parity(hora, oracle, gpu, name, mt):
    """10,000 x 64 Normal(0,10) base, k=10 (the reference's CPU-runnable case)."""
    from hora_gb300 import synth
    base = synth.normal(10000, 64, 10.0, stream=11)
    q = synth.normal(300, 64, 10.0, stream=12)
    ix = bf(hora, base, mt)
    ids, d = ix.search_batch(q, 10)
    oi, od = oracle.bf_search(base, q, 10, mt, threads=os.cpu_count() or 4)
    np.testing.assert_array_equal(d, od)  # bit-identical
    same_up_to_ties(ids.astype(np.int64), d, oi, od)
    # and within 1e-5 relative of the FP64 exact oracle
    ei, ed = oracle.bf_exact_f64(base, q, 10, mt, threads=os.cpu_count() or 4)
    np.testing.assert_allclose(d, ed, rtol=1e-5, atol=1e-5 * np.abs(ed).max())


@pytest.mark.parametrize("n,dim,k", [(1, 5, 3), (7, 3, 7), (129, 33, 10), (1000, 7, 1),
                                     (4099, 130, 100), (300, 64, 300)])
def test_ragged_shapes(hora, oracle, gpu, n, dim, k):
    rng = np.random.default_rng(n * 1000 + dim)
    base = (rng.standard_normal((n, dim)) * 10).astype(np.float32)
    q = (rng.standard_normal((37, dim)) * 10).astype(np.float32)
    for _, mt in METRICS:
        ix = bf(hora, base, mt)
        ids, d = ix.search_batch(q, k)
        oi, od = oracle.bf_search(base, q, k, mt)
        np.testing.assert_array_equal(d, od)
        same_up_to_ties(ids.astype(np.int64), d, oi, od)


def test_k_larger_than_n_pads(hora, gpu):
    base = np.arange(12, dtype=np.float32).reshape(3, 4)
    ix = bf(hora, base, 3)
    ids, d = ix.search_batch(base[:1], 5)
    assert ids[0, :3].tolist() == [0, 1, 2]
    assert (ids[0, 3:] == hora.NO_ID).all() and np.isinf(d[0, 3:]).all()
    assert ix.search(base[0], 5) == [0, 1, 2]


def test_duplicates_ties_and_overflow_rescan(hora, oracle, gpu):
    """Many identical rows (ties) and a tiny candidate capacity force the
    overflow rescan; the result must still be the exact k smallest keys."""
    rng = np.random.default_rng(9)
    base = np.repeat((rng.standard_normal((40, 16)) * 3).astype(np.float32), 250, axis=0)
    rng.shuffle(base)
    q = (rng.standard_normal((20, 16)) * 3).astype(np.float32)
    ix = bf(hora, base, 3)
    ix.set_option(hora.Option.CAND_CAP, 256)
    ids, d = ix.search_batch(q, 100)
    oi, od = oracle.bf_search(base, q, 100, 3)
    np.testing.assert_array_equal(d, od)
    # ties resolve to the lowest rows: check against a stable sort
    for qi in range(q.shape[0]):
        dd = ((base - q[qi]) ** 2).astype(np.float32)
        full = np.array([oracle.metric(q[qi], base[r], 3) for r in range(base.shape[0])], np.float32)
        order = np.lexsort((np.arange(base.shape[0]), full))[:100]
        assert ids[qi].astype(np.int64).tolist() == order.tolist()
        del dd
    info = ix.idx_info()
    assert '"last_overflow_rescans"' in info


def test_user_ids_and_search_nodes(hora, gpu):
    rng = np.random.default_rng(1)
    base = rng.standard_normal((500, 24)).astype(np.float32)
    uid = (np.arange(500, dtype=np.uint64) * 7 + 1000)
    ix = bf(hora, base, 3, ids=uid)
    res = ix.search_nodes(base[17], 4)
    assert res[0][0].idx == 17 * 7 + 1000 and res[0][1] == 0.0
    np.testing.assert_array_equal(res[0][0].vectors, base[17])
    assert ix.search(base[17], 1) == [17 * 7 + 1000]


def test_nan_rejected(hora, gpu):
    ix = hora.BruteForceIndex(4)
    with pytest.raises(hora.HoraError) as e:
        ix.add([1.0, np.nan, 0, 0], 0)
    assert e.value.code == -5
    ix.add([1.0, 2.0, 3.0, 4.0], 0)
    ix.build(hora.Metric.Euclidean)
    with pytest.raises(hora.HoraError):
        ix.search([np.inf, 0, 0, 0], 1)
    # device-resident queries: checked on the device, reported after the search
    import torch
    for prec in (0, 1):
        ix.set_option(hora.Option.PRECISION, prec)
        bad = torch.tensor([[1.0, 2.0, 3.0, 4.0], [0.0, np.nan, 0.0, 0.0]], device="cuda")
        with pytest.raises(hora.HoraError) as e:
            ix.search_batch(bad, 1)
        assert e.value.code == -5
        ids, _ = ix.search_batch(bad[:1].clone(), 1)  # the handle keeps working
        assert int(ids[0, 0]) == 0


def test_search_before_build_and_unknown_metric(hora, gpu):
    ix = hora.BruteForceIndex(4)
    ix.add([1.0, 2.0, 3.0, 4.0], 0)
    with pytest.raises(hora.HoraError) as e:
        ix.search([1, 2, 3, 4], 1)
    assert e.value.code == -8
    with pytest.raises(hora.HoraError) as e:
        ix.build(hora.Metric.Unknown)
    assert e.value.code == -4


def test_device_pointers(hora, oracle, gpu):
    import torch
    rng = np.random.default_rng(2)
    base = rng.standard_normal((3000, 40)).astype(np.float32)
    q = rng.standard_normal((50, 40)).astype(np.float32)
    ix = hora.BruteForceIndex(40)
    ix.madd(torch.from_numpy(base).cuda(), torch.arange(3000, dtype=torch.int64).cuda())
    ix.build(hora.Metric.Manhattan)
    ids_t = torch.empty((50, 8), dtype=torch.int64, device="cuda")
    d_t = torch.empty((50, 8), dtype=torch.float32, device="cuda")
    ix.search_batch(torch.from_numpy(q).cuda(), 8, ids_out=ids_t, dist_out=d_t)
    torch.cuda.synchronize()
    oi, od = oracle.bf_search(base, q, 8, 1)
    np.testing.assert_array_equal(d_t.cpu().numpy(), od)
    same_up_to_ties(ids_t.cpu().numpy(), d_t.cpu().numpy(), oi, od)


def test_dump_load_roundtrip(hora, gpu):
    rng = np.random.default_rng(4)
    base = rng.standard_normal((700, 10)).astype(np.float32)
    ix = bf(hora, base, 4)
    a = ix.search_batch(base[:20], 6)
    with tempfile.TemporaryDirectory() as t:
        p = os.path.join(t, "bf.idx")
        ix.dump(p)
        ix2 = hora.BruteForceIndex.load(p)
        assert ix2.nodes_size() == 700 and ix2.dimension() == 10 and ix2.name() == "BruteForceIndex"
        b = ix2.search_batch(base[:20], 6)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    with pytest.raises(hora.HoraError):
        hora.BruteForceIndex.load("/nonexistent/file")


def test_full_size_sample(hora, oracle, gpu):
    """1,000,000 x 128 mixture, k=100: a sample of queries against the FP64
    exact oracle (distances within 1e-5 relative, ids equal up to ties)."""
    from hora_gb300 import synth
    base = synth.mixture(1_000_000, 128, 1024, stream=1)
    q = synth.mixture(16, 128, 1024, stream=2)
    ix = bf(hora, base, 3)
    ids, d = ix.search_batch(q, 100)
    ei, ed = oracle.bf_exact_f64(base, q, 100, 3, threads=os.cpu_count() or 4)
    np.testing.assert_allclose(d, ed, rtol=1e-5)
    same_up_to_ties(ids.astype(np.int64), d.astype(np.float64), ei, ed, rtol=1e-6)
    # sortedness and idempotence
    assert (np.diff(d, axis=1) >= 0).all()
    ids2, d2 = ix.search_batch(q, 100)
    np.testing.assert_array_equal(ids, ids2)
