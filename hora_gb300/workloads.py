"""The benchmark configurations as runnable workloads (for profiling runs).

    python -m hora_gb300.workloads ivfpq [--queries N] [--epochs E] [--nprobe P]
                                         [--n ROWS] [--lists C]
    python -m hora_gb300.workloads bf [--queries N] [--precision fp32|bf16|fp8] [--rerank R]

ivfpq: IVFPQIndex over the 1M x 128 Gaussian mixture, 1,024 lists, 32 x
8-bit PQ trained on the first 500k items, then one search of N queries with
an exact rerank of 100 ADC candidates.  bf: BruteForceIndex over the same
data, one search of N queries, k = 100 (R candidates reranked, 0 = auto).
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np


def ivfpq(queries: int = 1024, epochs: int = 25, nprobe: int = 16, n: int = 1_000_000,
          lists: int = 1024):
    import torch

    import hora_gb300 as H
    from hora_gb300 import synth
    X = synth.mixture(n, 128, 1024, stream=1)
    q = synth.mixture(queries, 128, 1024, stream=2)
    ix = H.IVFPQIndex(128, H.IVFPQParams(n_sub=32, sub_bits=8,
                                         n_kmeans_center=lists, search_n_center=nprobe,
                                         train_epoch=epochs))
    ix.set_option(H.Option.TRAIN_SIZE, min(500_000, n))
    ix.madd(torch.from_numpy(X).cuda(), None)
    t0 = time.perf_counter()
    ix.build(H.Metric.Euclidean)
    build_s = time.perf_counter() - t0
    ix.set_option(H.Option.IVF_RERANK, 100)
    ids, d = ix.search_batch(q, 10)
    return {"build_s": build_s, "search_ms": json.loads(ix.idx_info())["last_search_ms"]}


def bf(queries: int = 1024, precision: str = "bf16", n: int = 1_000_000, rerank: int = 0):
    import torch

    import hora_gb300 as H
    from hora_gb300 import synth
    X = synth.mixture(n, 128, 1024, stream=1)
    q = synth.mixture(queries, 128, 1024, stream=2)
    ix = H.BruteForceIndex(128)
    ix.madd(torch.from_numpy(X).cuda(), None)
    ix.build(H.Metric.Euclidean)
    ix.set_option(H.Option.PRECISION, {"fp32": 0, "bf16": 1, "fp8": 2}[precision])
    ix.set_option(H.Option.RERANK, rerank)
    ids, d = ix.search_batch(q, 100)
    return {"search_ms": json.loads(ix.idx_info())["last_search_ms"]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("workload", choices=["ivfpq", "bf"])
    ap.add_argument("--queries", type=int, default=1024)
    ap.add_argument("--epochs", type=int, default=25)
    ap.add_argument("--nprobe", type=int, default=16)
    ap.add_argument("--precision", default="bf16")
    ap.add_argument("--n", type=int, default=1_000_000)
    ap.add_argument("--lists", type=int, default=1024)
    ap.add_argument("--rerank", type=int, default=0)
    a = ap.parse_args()
    if a.workload == "ivfpq":
        print(json.dumps(ivfpq(a.queries, a.epochs, a.nprobe, a.n, a.lists)))
    else:
        print(json.dumps(bf(a.queries, a.precision, a.n, a.rerank)))


if __name__ == "__main__":
    main()
