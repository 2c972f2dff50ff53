"""Starting thresholds from pivot clusters (BF16 and FP8 Euclidean brute force
on at least 65,536 rows).

The probed schedule must return exactly what the chunked schedule returns
(the same approximate R-best set, hence the same exact rerank), fall back to
the chunked schedule for a query whose list comes out short, and go through
the overflow rescans when more rows than the candidate capacity tie below a
threshold."""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def build(hora, base, R, prec=1):
    ix = hora.BruteForceIndex(base.shape[1])
    ix.madd(base, None)
    ix.build(hora.Metric.Euclidean)
    ix.set_option(hora.Option.PRECISION, prec)
    ix.set_option(hora.Option.RERANK, R)
    return ix


def run(hora, ix, q, k, probe):
    ix.set_option(hora.Option.BF_PROBE, probe)
    ids, d = ix.search_batch(q, k)
    return ids, d, json.loads(ix.idx_info())


@pytest.mark.parametrize("dim,R,k", [(128, 132, 100), (64, 256, 10), (32, 200, 1), (48, 400, 10)])
def test_probe_matches_chunked(hora, oracle, gpu, dim, R, k):
    """R-best lists wider than 256 keep the chunked schedule; a query whose
    pivot cluster holds fewer than R members is answered by it too."""
    from hora_gb300 import synth
    base = synth.mixture(100_000, dim, 256, stream=41)
    q = synth.mixture(700, dim, 256, stream=42)
    ix = build(hora, base, R)
    ids1, d1, info1 = run(hora, ix, q, k, 1)
    ids0, d0, info0 = run(hora, ix, q, k, 0)
    assert info1["last_threshold_probe"] in ((1, 2) if R <= 256 else (0,))
    assert info0["last_threshold_probe"] == 0
    np.testing.assert_array_equal(ids1, ids0)
    np.testing.assert_array_equal(d1, d0)
    for qi in range(0, 700, 97):
        assert d1[qi, 0] == oracle.metric(q[qi], base[int(ids1[qi, 0])], 3)


def test_short_list_falls_back(hora, gpu):
    """A blob of 10 rows at rows 0..9 takes the first pivot and is dissolved
    (fewer than 512 members); a query far beyond every cluster is nearest to
    that pivot, which has no members, so its list comes out short and the
    chunked schedule answers it.  Every row is then at the same FP32
    distance from it: the k lowest rows win."""
    rng = np.random.default_rng(5)
    base = rng.standard_normal((70_000, 32)).astype(np.float32)
    base[:10] += 100.0
    q = rng.standard_normal((40, 32)).astype(np.float32)
    q[7] = 1e15
    ix = build(hora, base, 132)
    ids1, d1, info1 = run(hora, ix, q, 10, 1)
    ids0, d0, _ = run(hora, ix, q, 10, 0)
    assert info1["last_threshold_probe"] == 2
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
