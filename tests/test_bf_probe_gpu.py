"""Starting thresholds for the low-precision brute force (BF16 and FP8 on
at least 65,536 rows; Euclidean, DotProduct and CosineSimilarity): up to
R = 256 from the query's nearest pivot cluster (a bound), wider R-best lists
(up to 4,096) from a sample of the base (a statistic).

The probed schedule must return exactly what the chunked schedule returns
(the same approximate R-best set, hence the same exact rerank), fall back to
the chunked schedule for a query whose list comes out short, and go through
the overflow rescans when more rows than the candidate capacity tie below a
threshold."""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def build(hora, base, R, prec=1, metric=3):
    ix = hora.BruteForceIndex(base.shape[1])
    ix.madd(base, None)
    ix.build(hora.Metric(metric))
    ix.set_option(hora.Option.PRECISION, prec)
    ix.set_option(hora.Option.RERANK, R)
    return ix


def check_probe_status(info, R, nq):
    """Up to R = 256 the probed thresholds are bounds: no list comes out
    short.  Wider lists take the sampled threshold, a statistic: a few lists
    may come out short (and be answered by the chunked schedule)."""
    if R <= 256:
        assert info["last_threshold_probe"] == 1 and info["last_short_lists"] == 0, info
    else:
        assert info["last_threshold_probe"] in (1, 2) and info["last_short_lists"] <= nq // 50, info


def run(hora, ix, q, k, probe):
    ix.set_option(hora.Option.BF_PROBE, probe)
    ids, d = ix.search_batch(q, k)
    return ids, d, json.loads(ix.idx_info())


@pytest.mark.parametrize("dim,R,k", [(128, 132, 100), (64, 256, 10), (32, 200, 1), (48, 400, 10),
                                     (64, 1000, 100), (128, 4096, 100)])
def test_probe_matches_chunked(hora, oracle, gpu, dim, R, k):
    """Lists up to R = 256 take the cluster threshold, wider ones (400,
    1,000, 4,096) the sampled one; either way the probed pass returns the
    chunked schedule's lists bit for bit."""
    from hora_gb300 import synth
    base = synth.mixture(100_000, dim, 256, stream=41)
    q = synth.mixture(700, dim, 256, stream=42)
    ix = build(hora, base, R)
    ids1, d1, info1 = run(hora, ix, q, k, 1)
    ids0, d0, info0 = run(hora, ix, q, k, 0)
    check_probe_status(info1, R, 700)
    assert info0["last_threshold_probe"] == 0
    np.testing.assert_array_equal(ids1, ids0)
    np.testing.assert_array_equal(d1, d0)
    for qi in range(0, 700, 97):
        assert d1[qi, 0] == oracle.metric(q[qi], base[int(ids1[qi, 0])], 3)


def sample_rows(n, m):
    """The base rows of the first m rows of the sample image the wide lists'
    threshold comes from: floor(frac(j phi) n) for j = 1..m (phi the golden
    ratio), in double precision as the library computes them."""
    f = np.arange(1, m + 1, dtype=np.float64) * 0.6180339887498949
    return np.minimum(((f - np.floor(f)) * n).astype(np.int64), n - 1)


def test_short_lists_fall_back(hora, gpu):
    """A base where exactly the sampled rows lie near the queries: for R =
    4,096 on 65,536 rows the sampled threshold (the 98th of the first 1,024
    sample rows' keys) keeps only ~98 rows, every list comes out short, and
    the chunked schedule answers all of them, with the same result."""
    rng = np.random.default_rng(5)
    n = 65_536
    base = (50.0 + rng.standard_normal((n, 32))).astype(np.float32)
    near = np.unique(sample_rows(n, 1024))
    base[near] = rng.standard_normal((near.size, 32)).astype(np.float32)
    q = rng.standard_normal((40, 32)).astype(np.float32)
    ix = build(hora, base, 4096)
    ids1, d1, info1 = run(hora, ix, q, 10, 1)
    ids0, d0, _ = run(hora, ix, q, 10, 0)
    assert info1["last_threshold_probe"] == 2 and info1["last_short_lists"] == 40, info1
    np.testing.assert_array_equal(ids1, ids0)
    np.testing.assert_array_equal(d1, d0)


def test_far_query_ties(hora, gpu):
    """A blob of 10 rows at rows 0..9 forms a pivot cluster that is dissolved
    (and its pivot dropped); a query far beyond every cluster sees every row
    at the same FP32 distance: the k lowest rows win, probed or not."""
    rng = np.random.default_rng(5)
    base = rng.standard_normal((70_000, 32)).astype(np.float32)
    base[:10] += 100.0
    q = rng.standard_normal((40, 32)).astype(np.float32)
    q[7] = 1e15
    ix = build(hora, base, 132)
    ids1, d1, info1 = run(hora, ix, q, 10, 1)
    ids0, d0, _ = run(hora, ix, q, 10, 0)
    assert info1["last_threshold_probe"] in (1, 2)
    np.testing.assert_array_equal(ids1, ids0)
    np.testing.assert_array_equal(d1, d0)
    assert ids1[7].tolist() == list(range(10))


def test_probe_overflow_with_duplicates(hora, oracle, gpu):
    """5,000 copies of one row tie below the probed threshold of a query at
    that row: more than the 4,096-key candidate capacity, so the overflow
    rescans run; ties go to the lowest rows."""
    rng = np.random.default_rng(6)
    base = rng.standard_normal((70_000, 48)).astype(np.float32)
    rows = np.sort(rng.choice(70_000, 5_000, replace=False))
    base[rows] = base[rows[0]]
    q = rng.standard_normal((64, 48)).astype(np.float32)
    q[3] = base[rows[0]]
    ix = build(hora, base, 132)
    ids1, d1, info1 = run(hora, ix, q, 50, 1)
    ids0, d0, _ = run(hora, ix, q, 50, 0)
    assert info1["last_threshold_probe"] == 1
    assert info1["last_overflow_rescans"] >= 1
    np.testing.assert_array_equal(ids1, ids0)
    np.testing.assert_array_equal(d1, d0)
    assert ids1[3].tolist() == rows[:50].tolist()
    assert d1[3, 0] == oracle.metric(q[3], base[rows[0]], 3)


def test_small_candidate_capacity(hora, gpu):
    """The pivot pass keeps only each query's nearest pivot (no per-pivot
    keys), so a candidate capacity below the pivot count (410 pivots for
    420,000 rows against 256 slots) still runs the probed schedule; the
    small capacity then overflows into rescans, and both answers agree."""
    from hora_gb300 import synth
    base = synth.mixture(420_000, 16, 256, stream=43)
    q = synth.mixture(300, 16, 256, stream=44)
    ix = build(hora, base, 132)
    ids1, d1, info1 = run(hora, ix, q, 20, 1)
    assert info1["last_threshold_probe"] == 1
    ix.set_option(hora.Option.CAND_CAP, 256)
    ids2, d2, info2 = run(hora, ix, q, 20, 1)
    assert info2["last_threshold_probe"] in (1, 2)
    np.testing.assert_array_equal(ids1, ids2)
    np.testing.assert_array_equal(d1, d2)


@pytest.mark.parametrize("dim,R,k", [(128, 256, 100), (128, 132, 100), (64, 200, 10)])
def test_fp8_probe_matches_chunked(hora, oracle, gpu, dim, R, k):
    """FP8 e4m3 scoring (per-row scales): the probe scores the cluster members
    with the scan's FP8 operands and scales; the probed pass returns the
    chunked schedule's lists bit for bit."""
    from hora_gb300 import synth
    base = synth.mixture(100_000, dim, 256, stream=45)
    q = synth.mixture(700, dim, 256, stream=46)
    ix = build(hora, base, R, prec=2)
    ids1, d1, info1 = run(hora, ix, q, k, 1)
    ids0, d0, info0 = run(hora, ix, q, k, 0)
    assert info1["last_threshold_probe"] in (1, 2) and info0["last_threshold_probe"] == 0
    np.testing.assert_array_equal(ids1, ids0)
    np.testing.assert_array_equal(d1, d0)
    for qi in range(0, 700, 97):
        assert d1[qi, 0] == oracle.metric(q[qi], base[int(ids1[qi, 0])], 3)


@pytest.mark.parametrize("metric", [2, 4])
@pytest.mark.parametrize("prec,R,k", [(1, 132, 100), (2, 132, 100), (1, 4096, 100), (2, 300, 10)])
def test_dot_and_cosine_probe_matches_chunked(hora, oracle, gpu, metric, prec, R, k):
    """DotProduct (ascending +<q, x>, the pivot pass reads -q) and
    CosineSimilarity (unit rows) in BF16 and FP8: the probe scores the
    clusters' members with the scan's key formula for the metric, and the
    probed pass returns the chunked schedule's lists bit for bit."""
    from hora_gb300 import synth
    base = synth.mixture(100_000, 64, 256, stream=47)
    q = synth.mixture(500, 64, 256, stream=48)
    ix = build(hora, base, R, prec=prec, metric=metric)
    ids1, d1, info1 = run(hora, ix, q, k, 1)
    ids0, d0, info0 = run(hora, ix, q, k, 0)
    check_probe_status(info1, R, 500)
    assert info0["last_threshold_probe"] == 0
    np.testing.assert_array_equal(ids1, ids0)
    np.testing.assert_array_equal(d1, d0)
    for qi in range(0, 500, 83):
        assert d1[qi, 0] == oracle.metric(q[qi], base[int(ids1[qi, 0])], metric)


@pytest.mark.parametrize("metric", [3, 2, 4])
def test_windowed_rerank_equals_full_rerank(hora, oracle, gpu, metric):
    """A wide BF16 list (R = 4,096 for k = 100) is reranked only within
    T + 2 eps of its k-th scan key (eps the certified bound on scan key vs
    exact distance, per metric); k = 1,100 (R < 4k) reranks all 4,096.  The
    same R-best set, so the first 100 of the wide answer must equal the
    windowed one bit for bit, and both the exact FP32 search's distances."""
    from hora_gb300 import synth
    base = synth.mixture(100_000, 64, 256, stream=49)
    q = synth.mixture(300, 64, 256, stream=50)
    ix = build(hora, base, 4096, metric=metric)
    ids_w, d_w = ix.search_batch(q, 100)
    ids_f, d_f = ix.search_batch(q, 1100)
    np.testing.assert_array_equal(ids_w, ids_f[:, :100])
    np.testing.assert_array_equal(d_w, d_f[:, :100])
    ix.set_option(hora.Option.PRECISION, 0)
    ix.set_option(hora.Option.EXACT_TC, 0)
    ids_e, d_e = ix.search_batch(q, 100)
    np.testing.assert_array_equal(d_w, d_e)


@pytest.mark.parametrize("metric", [3, 2])
def test_fp8_wide_list_holds_exact_top_k(hora, gpu, metric):
    """e4m3 filter passes skip a 32-column slice when a lower bound on its
    distances (from the slice's extreme accumulator and the rows' smallest
    squared norm and scale range) clears the threshold.  With a 4,096-wide
    list the exact 10 best of every query must survive the filter: the
    answer's distances equal the exact FP32 search's."""
    from hora_gb300 import synth
    base = synth.mixture(100_000, 64, 256, stream=51)
    q = synth.mixture(300, 64, 256, stream=52)
    ix = build(hora, base, 4096, prec=2, metric=metric)
    ids8, d8 = ix.search_batch(q, 10)
    ix.set_option(hora.Option.PRECISION, 0)
    ix.set_option(hora.Option.EXACT_TC, 0)
    ids32, d32 = ix.search_batch(q, 10)
    np.testing.assert_array_equal(d8, d32)
