"""SerializableIndex::load of files in the reference's own bincode layout
(hora_load_reference; layout written by tests/refbin.py from oracle-built
indexes): the loaded index searches exactly like the oracle's restatement of
the reference's search on the same structure.
"""
import os
import tempfile

import numpy as np
import pytest

from tests import refbin
from tests.test_bf_gpu import same_up_to_ties

pytestmark = pytest.mark.gpu


def write(tmp, name, blob):
    p = os.path.join(tmp, name)
    with open(p, "wb") as f:
        f.write(blob)
    return p


@pytest.mark.parametrize("mt", [3, 1, 2, 4])
def test_brute_force(hora, oracle, gpu, mt):
    rng = np.random.default_rng(mt)
    X = rng.standard_normal((700, 20)).astype(np.float32)
    q = rng.standard_normal((9, 20)).astype(np.float32)
    ids = [int(i) * 3 + 1 for i in range(700)]
    with tempfile.TemporaryDirectory() as t:
        ix = hora.load_reference(write(t, "bf.bin", refbin.brute_force(X, ids, mt)), hora.BruteForceIndex)
    assert ix.name() == "BruteForceIndex" and ix.nodes_size() == 700 and ix.dimension() == 20
    got_ids, got_d = ix.search_batch(q, 10)
    oi, od = oracle.bf_search(X, q, 10, mt)
    np.testing.assert_array_equal(got_d, od)
    same_up_to_ties((got_ids.astype(np.int64) - 1) // 3, got_d, oi, od)


@pytest.mark.parametrize("mt", [3, 1, 2])
def test_pq_index(hora, oracle, gpu, mt):
    rng = np.random.default_rng(20 + mt)
    X = rng.standard_normal((1500, 16)).astype(np.float32)
    q = rng.standard_normal((12, 16)).astype(np.float32)
    ref = oracle.pq_build(X, 4, 4, 5, mt, 11)
    blob = refbin.pq_index(X, list(range(1500)), 4, 4, 5, ref["codebooks"], ref["codes"], mt)
    with tempfile.TemporaryDirectory() as t:
        ix = hora.load_reference(write(t, "pq.bin", blob), hora.PQIndex)
    assert ix.name() == "PQIndex"
    ex = ix.export()
    np.testing.assert_array_equal(ex["codes"], ref["codes"])  # codes bit-exact given the codebooks
    ids, d = ix.search_batch(q, 8)
    oi, od = oracle.pq_search(ref, q, 8)
    np.testing.assert_array_equal(d, od)
    same_up_to_ties(ids.astype(np.int64), d, oi, od)


def test_ivfpq_index(hora, oracle, gpu):
    rng = np.random.default_rng(31)
    cen = (rng.standard_normal((10, 24)) * 3).astype(np.float32)
    X = (cen[rng.integers(0, 10, 2500)] + rng.standard_normal((2500, 24))).astype(np.float32)
    q = (cen[rng.integers(0, 10, 15)] + rng.standard_normal((15, 24))).astype(np.float32)
    ref = oracle.ivfpq_build(X, 6, 5, 8, 4, 3, 77)
    blob = refbin.ivfpq_index(X, list(range(2500)), 6, 5, 8, 3, 4, ref, 3)
    with tempfile.TemporaryDirectory() as t:
        ix = hora.load_reference(write(t, "ivf.bin", blob), hora.IVFPQIndex)
    assert ix.name() == "IVFPQIndex"
    ex = ix.export()
    for k in ("centers", "offsets", "items", "codes"):
        np.testing.assert_array_equal(ex[k], ref[k], err_msg=k)
    ids, d = ix.search_batch(q, 10)
    oi, od = oracle.ivfpq_search(ref, q, 10, 3)
    np.testing.assert_array_equal(d, od)
    same_up_to_ties(ids.astype(np.int64), d, oi, od)
