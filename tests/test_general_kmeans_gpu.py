"""kmeans::general_kmeans (src/core/kmeans.rs:216-289; SSG's root selection,
src/index/ssg_idx.rs:388) on the GPU against the oracle's restatement: same
initial rows, so the means must agree bit for bit and the roots exactly."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def index_of(hora, X, mt):
    ix = hora.BruteForceIndex(X.shape[1])
    ix.madd(X, None)
    ix.build(hora.Metric(mt))
    return ix


def mixture(n, d, c, seed, scale=6.0):
    rng = np.random.default_rng(seed)
    cen = (rng.standard_normal((c, d)) * scale).astype(np.float32)
    return (cen[rng.integers(0, c, n)] + rng.standard_normal((n, d))).astype(np.float32)


@pytest.mark.parametrize("mt", [3, 1, 2, 4])
def test_seeded_parity(hora, oracle, gpu, mt):
    X = mixture(3000, 16, 10, mt)
    ix = index_of(hora, X, mt)
    roots, means = ix.general_kmeans(12, epoch=15, seed=5, return_means=True)
    o_roots, o_means = oracle.general_kmeans(X, 12, 15, mt, seed=5)
    np.testing.assert_array_equal(means, o_means)
    np.testing.assert_array_equal(roots.astype(np.int64), o_roots)


def test_duplicate_init_gives_empty_mean(hora, oracle, gpu):
    # the second copy of a mean loses every tie, ends empty (0/0 = NaN) and
    # its root stays at row 0, as in the reference
    X = mixture(2000, 8, 4, 11)
    ix = index_of(hora, X, 3)
    init = np.array([5, 5, 900, 1500], np.uint64)
    roots, means = ix.general_kmeans(4, epoch=6, init_rows=init, return_means=True)
    o_roots, o_means = oracle.general_kmeans(X, 4, 6, 3, init_rows=init.astype(np.int64))
    assert np.isnan(means[1]).all() and roots[1] == 0
    np.testing.assert_array_equal(means, o_means)
    np.testing.assert_array_equal(roots.astype(np.int64), o_roots)


def test_epoch_zero_roots_are_the_init_rows(hora, gpu):
    X = mixture(1000, 8, 3, 2)
    ix = index_of(hora, X, 3)
    init = np.array([3, 999, 400], np.uint64)
    np.testing.assert_array_equal(ix.general_kmeans(3, epoch=0, init_rows=init), init)


def test_larger_parity(hora, oracle, gpu):
    X = mixture(50_000, 64, 40, 3)
    ix = index_of(hora, X, 3)
    roots, means = ix.general_kmeans(32, epoch=8, seed=9, return_means=True)
    o_roots, o_means = oracle.general_kmeans(X, 32, 8, 3, seed=9, threads=8)
    np.testing.assert_array_equal(means, o_means)
    np.testing.assert_array_equal(roots.astype(np.int64), o_roots)


def test_errors(hora, gpu):
    X = mixture(100, 8, 2, 4)
    ix = hora.BruteForceIndex(8)
    ix.madd(X, None)
    with pytest.raises(hora.HoraError):
        ix.general_kmeans(4)  # not built
    ix.build(hora.Metric.Euclidean)
    with pytest.raises(hora.HoraError):
        ix.general_kmeans(0)
    with pytest.raises(hora.HoraError):
        ix.general_kmeans(2, init_rows=np.array([0, 100], np.uint64))
