"""Writes the golden fixtures under tests/golden/.

kat.json holds the reference's own known-answer tests, read from its test
sources (the only assertions the reference makes on this path):
  - src/core/calc.rs:46-50   dot::<f32>([1,2,3],[1,2,3]) == -14.0
  - src/core/node.rs:178-186 Manhattan([1,1],[2,2]) == 2.0 (f64)
and a heap-order case derived by hand from std BinaryHeap's push / pop
(the reference's copy is src/core/heap.rs:21-35,54-68,95-112): three rows at
equal distance with k = 2 — the first pushed row is the one evicted.

The .npz fixtures are outputs of the C restatement (oracle/hora_oracle.c) on
small seeded inputs; they pin the restatement against regressions and give
the GPU tests fixed expected values.  Regenerate with
    python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402


def main():
    O.build()
    kat = {
        "calc_dot_f32": {"a": [1, 2, 3], "b": [1, 2, 3], "expect": -14.0,
                         "source": "src/core/calc.rs:46-50"},
        "manhattan_f64": {"a": [1.0, 1.0], "b": [2.0, 2.0], "expect": 2.0,
                          "source": "src/core/node.rs:178-186"},
        "heap_ties_k2": {"distances": [1.0, 1.0, 1.0], "k": 2, "expect_ids": [2, 1],
                         "source": "std BinaryHeap push/pop order, src/core/heap.rs"},
    }
    with open(os.path.join(HERE, "kat.json"), "w") as f:
        json.dump(kat, f, indent=1)

    g = np.random.Generator(np.random.PCG64(20240611))
    base = (g.standard_normal((300, 12)) * 10).astype(np.float32)
    q = (g.standard_normal((7, 12)) * 10).astype(np.float32)
    out = {"base": base, "queries": q}
    for mt, name in ((3, "l2"), (1, "l1"), (2, "ip"), (4, "cos")):
        i, d = O.bf_search(base, q, 5, mt)
        out[f"{name}_ids"] = i
        out[f"{name}_dist"] = d
    np.savez_compressed(os.path.join(HERE, "bf_small.npz"), **out)

    # k-means: one coarse training with the seeded split stream
    cent = (g.standard_normal((6, 8)) * 5).astype(np.float32)
    pts = (cent[g.integers(0, 6, 400)] + g.standard_normal((400, 8))).astype(np.float32)
    seed = O.rng_instance_seed(0x686F7261, 0)
    km = O.kmeans_train(pts, 0, 8, 6, 12, 3, seed, accum_f64=True)
    km32 = O.kmeans_train(pts, 0, 8, 6, 12, 3, seed, accum_f64=False)
    np.savez_compressed(os.path.join(HERE, "kmeans_small.npz"), points=pts, centers_f64=km,
                        centers_f32=km32, seed=np.uint64(seed))

    # IVF-PQ: 1200 x 16, 4 lists, 4 sub-quantizers x 4 bits
    cen = (g.standard_normal((5, 16)) * 4).astype(np.float32)
    X = (cen[g.integers(0, 5, 1200)] + g.standard_normal((1200, 16))).astype(np.float32)
    ix = O.ivfpq_build(X, 4, 4, 4, 8, 3, 0x686F7261)
    qi, qd = O.ivfpq_search(ix, X[:9], 6, 2)
    np.savez_compressed(os.path.join(HERE, "ivfpq_small.npz"), data=X, centers=ix["centers"],
                        offsets=ix["offsets"], items=ix["items"], codebooks=ix["codebooks"],
                        codes=ix["codes"], trained=ix["trained"], q_ids=qi, q_dist=qd)
    print("golden fixtures written")


if __name__ == "__main__":
    main()
