"""Open-loop load generator for the serving loop (hora_server_*).

Requests arrive as a Poisson process at a target query rate; each request has
a batch size drawn log-uniformly from [1, max_batch], a k drawn uniformly
from k_choices and a target index drawn uniformly.  A submitter thread
releases requests at their arrival times (it never waits for completions:
open loop), a collector thread waits on the tickets.  Reported: achieved
queries/s, request latency p50 / p99 (submit -> completion, measured by the
server), peak in-flight requests and admitted bytes.
"""
from __future__ import annotations

import threading
import time

import numpy as np


def run(server, pools, rate_qps: float, duration_s: float, seed: int = 0,
        k_choices=(1, 10, 100), max_batch: int = 256) -> dict:
    """pools[i] is a (n_pool, dim_i) float32 array of queries for index i."""
    rng = np.random.default_rng(seed)
    mean_b = (max_batch - 1) / np.log(max_batch)  # mean of the log-uniform on [1, max_batch]
    req_rate = rate_qps / mean_b
    reqs = []
    t = 0.0
    while t < duration_s:
        t += rng.exponential(1.0 / req_rate)
        b = int(min(max_batch, max(1, np.floor(np.exp(rng.uniform(0.0, np.log(max_batch + 1)))))))
        which = int(rng.integers(0, len(pools)))
        k = int(rng.choice(k_choices))
        start = int(rng.integers(0, pools[which].shape[0] - b + 1))
        reqs.append((t, which, k, np.ascontiguousarray(pools[which][start:start + b])))
    tickets = [None] * len(reqs)
    lat = [None] * len(reqs)
    submitted = threading.Semaphore(0)

    def submitter():
        t0 = time.perf_counter()
        for i, (ta, which, k, q) in enumerate(reqs):
            delay = ta - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
            tickets[i] = server.submit(which, q, k)
            submitted.release()

    def collector():
        for i in range(len(reqs)):
            submitted.acquire()
            _, _, lat[i] = server.wait(tickets[i])

    t_start = time.perf_counter()
    th = [threading.Thread(target=submitter), threading.Thread(target=collector)]
    for x in th:
        x.start()
    for x in th:
        x.join()
    wall = time.perf_counter() - t_start
    nq = sum(r[3].shape[0] for r in reqs)
    lat = np.array(lat, dtype=np.float64)
    st = server.stats()
    return {"target_qps": rate_qps, "requests": len(reqs), "queries": int(nq),
            "achieved_qps": nq / wall, "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "max_inflight": st["max_inflight"],
            "max_admitted_bytes": st["max_admitted_bytes"], "wall_s": wall}
