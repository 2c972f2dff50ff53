"""CPU tests of the oracle: the reference's known-answer tests, the golden
fixtures, and properties of the restated algorithms (no GPU needed)."""
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def kat():
    return json.load(open(os.path.join(GOLD, "kat.json")))


def test_kat1_calc_dot(oracle):
    k = kat()["calc_dot_f32"]
    assert oracle.calc_dot(k["a"], k["b"]) == k["expect"]  # src/core/calc.rs:46-50


def test_kat2_manhattan_f64(oracle):
    k = kat()["manhattan_f64"]
    assert oracle.metric_f64(k["a"], k["b"], oracle.MANHATTAN) == k["expect"]  # node.rs:178-186


def test_dot_metric_is_positive_inner_product(oracle):
    # metrics.rs:50-57 negates calc::dot, which already negates
    assert oracle.metric([1, 2, 3], [1, 2, 3], oracle.DOT) == 14.0


def test_euclidean_is_squared(oracle):
    assert oracle.metric([0, 0], [3, 4], oracle.EUCLIDEAN) == 25.0


def test_cosine_intent(oracle):
    assert oracle.metric([1, 0], [1, 0], oracle.COSINE) == -1.0
    assert oracle.metric([1, 0], [0, 1], oracle.COSINE) == 0.0
    assert oracle.metric([0, 0], [0, 1], oracle.COSINE) == 0.0  # zero norm


def test_unknown_metric_is_error(oracle):
    with pytest.raises(ValueError):
        oracle.metric([1.0], [1.0], 0)


def test_heap_tie_order(oracle):
    k = kat()["heap_ties_k2"]
    base = np.zeros((3, 4), np.float32)
    ids, d = oracle.bf_search(base, np.ones((1, 4), np.float32), k["k"], oracle.EUCLIDEAN)
    assert ids[0].tolist() == k["expect_ids"]


def test_bf_golden(oracle):
    g = np.load(os.path.join(GOLD, "bf_small.npz"))
    for mt, name in ((3, "l2"), (1, "l1"), (2, "ip"), (4, "cos")):
        i, d = oracle.bf_search(g["base"], g["queries"], 5, mt)
        np.testing.assert_array_equal(i, g[f"{name}_ids"])
        np.testing.assert_array_equal(d, g[f"{name}_dist"])


@pytest.mark.parametrize("mt", [3, 1, 2, 4])
def test_bf_matches_f64(oracle, mt):
    rng = np.random.default_rng(3)
    base = (rng.standard_normal((3000, 33)) * 10).astype(np.float32)
    q = (rng.standard_normal((11, 33)) * 10).astype(np.float32)
    i, d = oracle.bf_search(base, q, 10, mt)
    ie, de = oracle.bf_exact_f64(base, q, 10, mt)
    np.testing.assert_allclose(d, de, rtol=1e-5, atol=1e-6 * np.abs(de).max())
    assert (i == ie).mean() > 0.99


def test_bf_k_larger_than_n(oracle):
    base = np.arange(12, dtype=np.float32).reshape(3, 4)
    i, d = oracle.bf_search(base, base[:1], 5, oracle.EUCLIDEAN)
    assert i[0, :3].tolist() == [0, 1, 2] and (i[0, 3:] == -1).all() and np.isinf(d[0, 3:]).all()


def test_kmeans_init_two_distinct_centres(oracle):
    # kmeans.rs:72-84: (i & (1 << j)) == 1 only for odd i at j % 64 == 0
    pts = np.random.default_rng(0).standard_normal((50, 130)).astype(np.float32)
    c = oracle.kmeans_init(pts, 0, 130, 8)
    assert len({tuple(r) for r in c}) == 2
    mean = pts.astype(np.float64).mean(0).astype(np.float32)
    np.testing.assert_allclose(c[1, 0], mean[0] + 1, rtol=1e-6)
    np.testing.assert_allclose(c[1, 64], mean[64] + 1, rtol=1e-6)
    np.testing.assert_allclose(c[1, 1], mean[1] - 1, rtol=1e-6)
    np.testing.assert_allclose(c[0, 0], mean[0] - 1, rtol=1e-6)


def test_kmeans_empty_centre_is_zero(oracle):
    pts = np.ones((10, 3), np.float32)
    cent, cnt = oracle.kmeans_update(pts, 0, 3, np.zeros(10, np.int64), 3)
    assert cnt.tolist() == [10, 0, 0] and (cent[1:] == 0).all()


def test_kmeans_split_deterministic(oracle):
    c = np.arange(12, dtype=np.float32).reshape(4, 3)
    cnt = np.array([6, 0, 4, 0])
    a = oracle.kmeans_split(c, cnt, 10, 77)
    b = oracle.kmeans_split(c, cnt, 10, 77)
    np.testing.assert_array_equal(a[0], b[0])
    assert a[1].sum() == 10 and (a[1] >= 0).all()
    assert a[1][1] > 0 or a[1][3] > 0


def test_kmeans_golden(oracle):
    g = np.load(os.path.join(GOLD, "kmeans_small.npz"))
    seed = int(g["seed"])
    np.testing.assert_array_equal(oracle.kmeans_train(g["points"], 0, 8, 6, 12, 3, seed, accum_f64=True),
                                  g["centers_f64"])
    np.testing.assert_array_equal(oracle.kmeans_train(g["points"], 0, 8, 6, 12, 3, seed, accum_f64=False),
                                  g["centers_f32"])


def test_pq_ranges(oracle):
    # pq_idx.rs:75-88, including its dimension % sub_dimension formula
    b, e = oracle.pq_ranges(128, 32)
    assert b.tolist() == list(range(0, 128, 4)) and e.tolist() == list(range(4, 132, 4))
    b, e = oracle.pq_ranges(10, 3)
    assert list(zip(b, e)) == [(0, 4), (4, 7), (7, 10)]
    b, e = oracle.pq_ranges(10, 4)  # dims 8..9 are not covered, as in the reference
    assert list(zip(b, e)) == [(0, 2), (2, 4), (4, 6), (6, 8)]


def test_ivfpq_golden(oracle):
    g = np.load(os.path.join(GOLD, "ivfpq_small.npz"))
    ix = oracle.ivfpq_build(g["data"], 4, 4, 4, 8, 3, 0x686F7261)
    for k in ("centers", "offsets", "items", "codebooks", "codes", "trained"):
        np.testing.assert_array_equal(ix[k], g[k], err_msg=k)
    qi, qd = oracle.ivfpq_search(ix, g["data"][:9], 6, 2)
    np.testing.assert_array_equal(qi, g["q_ids"])
    np.testing.assert_array_equal(qd, g["q_dist"])


def test_ivfpq_codes_reproduce_from_codebooks(oracle):
    g = np.load(os.path.join(GOLD, "ivfpq_small.npz"))
    offs, items = g["offsets"], g["items"]
    for c in range(len(offs) - 1):
        rows = g["data"][items[offs[c]:offs[c + 1]]]
        codes = oracle.pq_encode(rows, g["centers"][c], g["codebooks"][c], 4, 4)
        np.testing.assert_array_equal(codes, g["codes"][offs[c]:offs[c + 1]])


def test_ivfpq_nprobe_all_equals_flat_adc(oracle):
    # probing every list == ADC over every item (pq_idx.rs:408-439)
    g = np.load(os.path.join(GOLD, "ivfpq_small.npz"))
    ix = oracle.ivfpq_build(g["data"], 4, 4, 4, 8, 3, 0x686F7261)
    qi, qd = oracle.ivfpq_search(ix, g["data"][:5], 10, 4)
    for qn in range(5):
        ds = []
        for c in range(4):
            lut = oracle.pq_lut(g["data"][qn], ix["centers"][c], ix["codebooks"][c], 4, 4)
            for r in range(ix["offsets"][c], ix["offsets"][c + 1]):
                d = np.float32(0)
                for m in range(4):
                    d = np.float32(d + lut[m, ix["codes"][r, m]])
                ds.append((d, ix["items"][r]))
        ds.sort(key=lambda t: t[0])
        np.testing.assert_array_equal(qd[qn], np.array([t[0] for t in ds[:10]], np.float32))


@pytest.mark.parametrize("mt", [3, 1, 2])
def test_flat_pq_is_adc_over_its_own_codes(oracle, mt):
    # PQIndex (pq_idx.rs:122-193): every code is the metric's argmin over its
    # subspace's codebook, and search returns the k smallest sequential ADC
    # sums with LUT[m][j] = metric(q[range_m], C[m][j])
    rng = np.random.default_rng(mt)
    X = rng.standard_normal((600, 12)).astype(np.float32)
    ix = oracle.pq_build(X, 3, 3, 4, mt, 7)
    b, e = oracle.pq_ranges(12, 3)
    books, codes = ix["codebooks"], ix["codes"]
    for i in range(0, 600, 37):
        for m in range(3):
            d = [oracle.metric(X[i, b[m]:e[m]], books[m, j, :e[m] - b[m]], mt) for j in range(8)]
            assert codes[i, m] == int(np.argmin(d))  # first minimum, as the strict '<' scan
    q = rng.standard_normal((4, 12)).astype(np.float32)
    qi, qd = oracle.pq_search(ix, q, 6)
    for n in range(4):
        lut = [[oracle.metric(q[n, b[m]:e[m]], books[m, j, :e[m] - b[m]], mt) for j in range(8)]
               for m in range(3)]
        ds = []
        for r in range(600):
            d = np.float32(0)
            for m in range(3):
                d = np.float32(d + np.float32(lut[m][codes[r, m]]))
            ds.append(d)
        np.testing.assert_array_equal(qd[n], np.sort(np.array(ds, np.float32))[:6])


def test_mlp_grad_finite_difference(oracle):
    rng = np.random.default_rng(5)
    f, h1, h2 = 6, 5, 4
    npar = h1 * f + h1 + h2 * h1 + h2 + h2 + 1
    p = (rng.standard_normal(npar) * 0.5).astype(np.float32)
    x = rng.standard_normal((9, f)).astype(np.float32)
    y = rng.standard_normal(9).astype(np.float32)
    loss, g = oracle.mlp_loss_grad(p, x, y, f, h1, h2, alpha=2.0)
    eps = 1e-3
    for i in rng.choice(npar, 12, replace=False):
        pp = p.astype(np.float64).copy()
        pp[i] += eps
        lp, _ = oracle.mlp_loss_grad(pp.astype(np.float32), x, y, f, h1, h2, alpha=2.0)
        pp[i] -= 2 * eps
        lm, _ = oracle.mlp_loss_grad(pp.astype(np.float32), x, y, f, h1, h2, alpha=2.0)
        assert abs((lp - lm) / (2 * eps) - g[i]) < 2e-2 * max(1.0, abs(g[i]))


def test_general_kmeans_oracle_behaviour(oracle):
    """kmeans::general_kmeans (kmeans.rs:216-289) restated: an epoch-0 run
    returns the initial rows as roots, a duplicated initial mean loses every
    tie and becomes 0/0 = NaN with root 0, and well separated clusters seeded
    one row each converge to their means."""
    rng = np.random.default_rng(7)
    cen = np.array([[0, 0], [100, 0], [0, 100]], np.float32)
    lab = rng.integers(0, 3, 600)
    X = (cen[lab] + rng.standard_normal((600, 2))).astype(np.float32)
    init = np.array([int(np.where(lab == c)[0][0]) for c in range(3)], np.int64)
    roots, _ = oracle.general_kmeans(X, 3, 0, 3, init_rows=init)
    np.testing.assert_array_equal(roots, init)
    roots, means = oracle.general_kmeans(X, 3, 5, 3, init_rows=init)
    for c in range(3):
        np.testing.assert_allclose(means[c], X[lab == c].mean(0), atol=1e-3)
        assert lab[roots[c]] == c
    roots, means = oracle.general_kmeans(X, 3, 3, 3, init_rows=np.array([init[0], init[0], init[1]]))
    assert np.isnan(means[1]).all() and roots[1] == 0
    assert np.isfinite(means[[0, 2]]).all()
    a, ma = oracle.general_kmeans(X, 3, 4, 3, seed=3)
    b, mb = oracle.general_kmeans(X, 3, 4, 3, seed=3, threads=4)
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(ma, mb)
