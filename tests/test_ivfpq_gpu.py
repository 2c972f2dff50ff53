"""IVF-PQ ("PQIVFIndex") parity on the GPU against the oracle, through the C ABI.

- build: with the same seed, the GPU build (coarse k-means, lists, per-list
  PQ codebooks, codes) equals the oracle's restatement of
  IVFPQIndex::train (src/index/pq_idx.rs:357-396) bit for bit;
- codes: bit-exact given identical codebooks (hora_ivfpq_set_codebooks);
- search: ADC distances equal the oracle's restatement of
  IVFPQIndex::search_knn_adc (pq_idx.rs:408-439); ids equal up to ties.
"""
import os
import tempfile

import numpy as np
import pytest

from tests.test_bf_gpu import same_up_to_ties

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def ivf(hora, X, n_sub, bits, n_list, epochs, mt=3, nprobe=4, seed=0x686F7261):
    p = hora.IVFPQParams(n_sub=n_sub, sub_bits=bits, n_kmeans_center=n_list,
                         search_n_center=nprobe, train_epoch=epochs)
    ix = hora.IVFPQIndex(X.shape[1], p)
    ix.set_option(hora.Option.SEED, seed)
    ix.madd(X, np.arange(X.shape[0], dtype=np.uint64))
    ix.build(hora.Metric(mt))
    return ix


def test_golden_build_and_search(hora, oracle, gpu):
    g = np.load(os.path.join(GOLD, "ivfpq_small.npz"))
    ix = ivf(hora, g["data"], 4, 4, 4, 8, nprobe=2)
    ex = ix.export()
    for k in ("centers", "offsets", "items", "codebooks", "codes", "trained"):
        np.testing.assert_array_equal(ex[k], g[k], err_msg=k)
    ids, d = ix.search_batch(g["data"][:9], 6)
    np.testing.assert_array_equal(d, g["q_dist"])
    same_up_to_ties(ids.astype(np.int64), d, g["q_ids"], g["q_dist"])


@pytest.mark.parametrize("mt", [3, 1, 2, 4])
def test_build_matches_oracle(hora, oracle, gpu, mt):
    rng = np.random.default_rng(40 + mt)
    cen = (rng.standard_normal((12, 24)) * 3).astype(np.float32)
    X = (cen[rng.integers(0, 12, 3000)] + rng.standard_normal((3000, 24))).astype(np.float32)
    ix = ivf(hora, X, 6, 5, 16, 6, mt=mt, nprobe=5)
    ex = ix.export()
    ref = oracle.ivfpq_build(X, 6, 5, 16, 6, mt, 0x686F7261)
    for k in ("centers", "offsets", "items", "codebooks", "codes", "trained"):
        np.testing.assert_array_equal(ex[k], ref[k], err_msg=k)
    q = (cen[rng.integers(0, 12, 40)] + rng.standard_normal((40, 24))).astype(np.float32)
    for nprobe in (1, 3, 16):
        ids, d = ix.search_batch(q, 10, nprobe=nprobe)
        oi, od = oracle.ivfpq_search(ref, q, 10, nprobe)
        np.testing.assert_array_equal(d, od)
        same_up_to_ties(ids.astype(np.int64), d, oi, od)


@pytest.mark.parametrize("mt", [3, 2])
def test_adc_bit_exact_32_subspaces_of_256(hora, oracle, gpu, mt):
    """dim 128 with 32 x 8-bit sub-quantizers (the bench's layout): the
    code-major LUT built for groups of 4 queries, the skewed code-row scan
    with two queries per packed add; ADC distances equal the oracle's bit for
    bit at nprobe 1 and 4."""
    rng = np.random.default_rng(77 + mt)
    cen = (rng.standard_normal((16, 128)) * 3).astype(np.float32)
    X = (cen[rng.integers(0, 16, 12000)] + rng.standard_normal((12000, 128))).astype(np.float32)
    ix = ivf(hora, X, 32, 8, 16, 3, mt=mt, nprobe=4)
    ref = dict(ix.export(), metric=mt)
    q = (X[:64] + 0.1 * rng.standard_normal((64, 128))).astype(np.float32)
    for nprobe in (1, 4):
        ids, d = ix.search_batch(q, 10, nprobe=nprobe)
        oi, od = oracle.ivfpq_search(ref, q, 10, nprobe)
        np.testing.assert_array_equal(d, od)
        same_up_to_ties(ids.astype(np.int64), d, oi, od)


def test_codes_bit_exact_given_codebooks(hora, oracle, gpu):
    rng = np.random.default_rng(5)
    X = rng.standard_normal((4000, 32)).astype(np.float32)
    ref = oracle.ivfpq_build(X[:1500], 8, 8, 8, 3, 3, 99)
    ix = hora.IVFPQIndex(32, hora.IVFPQParams(n_sub=8, sub_bits=8, n_kmeans_center=8,
                                              search_n_center=3, train_epoch=3))
    ix.madd(X, np.arange(4000, dtype=np.uint64))
    ix.build(hora.Metric.Euclidean)
    ix.set_codebooks(ref["centers"], ref["codebooks"])
    ex = ix.export()
    offs, items = ex["offsets"], ex["items"]
    for c in range(8):
        rows = X[items[offs[c]:offs[c + 1]]]
        codes = oracle.pq_encode(rows, ref["centers"][c], ref["codebooks"][c], 8, 8)
        np.testing.assert_array_equal(ex["codes"][offs[c]:offs[c + 1]], codes)
    full = dict(ex, metric=3)
    q = X[:30] + 0.1
    ids, d = ix.search_batch(q, 7)
    oi, od = oracle.ivfpq_search(full, q, 7, 3)
    np.testing.assert_array_equal(d, od)


def test_ranges_non_divisible_dim(hora, oracle, gpu):
    """D=10, n_sub=3 uses the reference's dimension % sub_dimension ranges."""
    rng = np.random.default_rng(8)
    X = rng.standard_normal((900, 10)).astype(np.float32)
    ix = ivf(hora, X, 3, 4, 5, 4, nprobe=2)
    ref = oracle.ivfpq_build(X, 3, 4, 5, 4, 3, 0x686F7261)
    ex = ix.export()
    np.testing.assert_array_equal(ex["codebooks"], ref["codebooks"])
    np.testing.assert_array_equal(ex["codes"], ref["codes"])
    ids, d = ix.search_batch(X[:20], 5)
    oi, od = oracle.ivfpq_search(ref, X[:20], 5, 2)
    np.testing.assert_array_equal(d, od)


def test_empty_lists_and_nprobe_clamp(hora, oracle, gpu):
    """More lists than distinct points leaves lists empty (the reference panics
    there); they are skipped.  nprobe beyond n_list is clamped."""
    X = np.repeat(np.eye(4, 6, dtype=np.float32) * 5, 30, axis=0)
    ix = ivf(hora, X, 2, 2, 16, 3, nprobe=40)
    ex = ix.export()
    assert (ex["trained"] == 0).sum() > 0
    ref = oracle.ivfpq_build(X, 2, 2, 16, 3, 3, 0x686F7261)
    np.testing.assert_array_equal(ex["trained"], ref["trained"])
    ids, d = ix.search_batch(X[:5], 10)
    oi, od = oracle.ivfpq_search(ref, X[:5], 10, 40)
    np.testing.assert_array_equal(d, od)


def test_nprobe_all_lists_equals_flat_adc(hora, oracle, gpu):
    rng = np.random.default_rng(12)
    X = rng.standard_normal((2000, 16)).astype(np.float32)
    ix = ivf(hora, X, 4, 8, 8, 4)
    a_ids, a_d = ix.search_batch(X[:10], 20, nprobe=8)
    ex = dict(ix.export(), metric=3)
    # flat ADC over every list
    for qn in range(10):
        ds = []
        for c in range(8):
            lut = oracle.pq_lut(X[qn], ex["centers"][c], ex["codebooks"][c], 4, 8)
            for r in range(ex["offsets"][c], ex["offsets"][c + 1]):
                dd = np.float32(0)
                for m in range(4):
                    dd = np.float32(dd + lut[m, ex["codes"][r, m]])
                ds.append(dd)
        np.testing.assert_array_equal(a_d[qn], np.sort(np.array(ds, np.float32))[:20])


def test_rerank_option_gives_exact_distances(hora, oracle, gpu):
    rng = np.random.default_rng(13)
    X = rng.standard_normal((5000, 32)).astype(np.float32)
    ix = ivf(hora, X, 8, 8, 16, 5, nprobe=16)
    ix.set_option(hora.Option.IVF_RERANK, 200)
    ids, d = ix.search_batch(X[:25] + 0.05, 10)
    for qn in range(25):
        for j in range(10):
            assert d[qn, j] == oracle.metric(X[qn] + np.float32(0.05), X[int(ids[qn, j])], 3)
    # with every list probed and a wide shortlist this is exact brute force
    ei, ed = oracle.bf_search(X, X[:25] + np.float32(0.05), 10, 3)
    assert np.mean([len(set(a) & set(b)) / 10 for a, b in zip(ids.astype(np.int64), ei)]) > 0.97


def test_dump_load(hora, gpu):
    rng = np.random.default_rng(21)
    X = rng.standard_normal((3000, 16)).astype(np.float32)
    ix = ivf(hora, X, 4, 6, 10, 4)
    a = ix.search_batch(X[:15], 8)
    with tempfile.TemporaryDirectory() as t:
        p = os.path.join(t, "ivf.idx")
        ix.dump(p)
        ix2 = hora.IVFPQIndex.load(p)
        b = ix2.search_batch(X[:15], 8)
        assert ix2.name() == "IVFPQIndex"
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


def test_full_size_config(hora, oracle, gpu):
    """1,000,000 x 128 mixture, 1,024 lists, 32 x 8-bit PQ, trained on the
    first 500,000 items (a few epochs to bound the test): recall grows with
    nprobe, codes of sampled lists are bit-exact with the oracle's encoder."""
    from hora_gb300 import synth
    X = synth.mixture(1_000_000, 128, 1024, stream=1)
    q = synth.mixture(200, 128, 1024, stream=2)
    p = hora.IVFPQParams(n_sub=32, sub_bits=8, n_kmeans_center=1024, search_n_center=16,
                         train_epoch=4)
    ix = hora.IVFPQIndex(128, p)
    ix.set_option(hora.Option.TRAIN_SIZE, 500_000)
    ix.madd(X, None)
    ix.build(hora.Metric.Euclidean)
    ex = ix.export()
    assert ex["offsets"][-1] == 1_000_000
    for c in (0, 511, 1023):
        lo, hi = ex["offsets"][c], ex["offsets"][c + 1]
        if hi == lo:
            continue
        rows = X[ex["items"][lo:hi]]
        codes = oracle.pq_encode(rows, ex["centers"][c], ex["codebooks"][c], 32, 8)
        np.testing.assert_array_equal(ex["codes"][lo:hi], codes)
    ei, _ = oracle.bf_exact_f64(X, q, 10, 3, threads=os.cpu_count() or 4)
    rec = []
    for nprobe in (1, 4, 16, 64):
        ids, d = ix.search_batch(q, 10, nprobe=nprobe)
        assert (np.diff(d, axis=1) >= 0).all()
        rec.append(np.mean([len(set(a) & set(b)) / 10 for a, b in zip(ids.astype(np.int64), ei)]))
    # PQ alone (no rerank, as in the reference) saturates early on this
    # well-separated mixture: ADC error, not probing, limits recall@10
    assert rec == sorted(rec) and rec[-1] > 0.25, rec
    ix.set_option(hora.Option.IVF_RERANK, 400)
    ids, _ = ix.search_batch(q, 10, nprobe=64)
    rr = np.mean([len(set(a) & set(b)) / 10 for a, b in zip(ids.astype(np.int64), ei)])
    assert rr >= 0.95, rr


@pytest.mark.parametrize("metric", [3, 2, 4])
def test_coarse_probe_on_tensor_cores_equals_fp32(hora, gpu, metric):
    """With at least 2,048 lists the coarse probe is a BF16 pass plus the
    exact rescoring of the centres within the certified bound of the
    pmax-th; it returns the FP32 probe's lists: the searches with it (the
    default) and without it (EXACT_TC 0) agree bit for bit, at several
    nprobe."""
    from hora_gb300 import synth
    X = synth.mixture(120_000, 64, 512, stream=71)
    q = synth.mixture(400, 64, 512, stream=72)
    ix = hora.IVFPQIndex(64, hora.IVFPQParams(n_sub=16, sub_bits=8, n_kmeans_center=2048,
                                              search_n_center=4, train_epoch=3))
    ix.madd(X, None)
    ix.build(hora.Metric(metric))
    for nprobe in (1, 4, 37):
        ix.set_option(hora.Option.EXACT_TC, 1)
        ids1, d1 = ix.search_batch(q, 10, nprobe=nprobe)
        ix.set_option(hora.Option.EXACT_TC, 0)
        ids0, d0 = ix.search_batch(q, 10, nprobe=nprobe)
        np.testing.assert_array_equal(ids1, ids0, err_msg=f"nprobe {nprobe}")
        np.testing.assert_array_equal(d1, d0, err_msg=f"nprobe {nprobe}")
