#!/usr/bin/env python
"""Benchmark of the brute-force search path on one GB300 (or N replicas).

Workload (the configuration the headline metric is quoted on): a
BruteForceIndex over 1,000,000 x 128 float32 vectors from a Gaussian mixture
(1,024 centres ~ 3*N(0,I), points = centre + N(0,I)), 10,000 queries from the
same mixture, k = 100, Euclidean.  A step is one batched search of all
10,000 queries.  The base (512 MB) is larger than L2 (129 MB), so every step
streams it from HBM; no L2 flush is needed.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`value` is queries/s of the headline form with queries and outputs resident
in HBM; `e2e` is the same through the public API with host buffers (H2D of the
queries and D2H of ids + distances inside the timed region).  The headline
form is the fastest form whose recall@10 against the exact FP32 result is
>= 0.95; every form's QPS and recall is listed under "forms".
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_BASE, DIM, N_Q, K, N_CENTERS = 1_000_000, 128, 10_000, 100, 1024
WORKLOAD = "BruteForceIndex 1Mx128 f32 gaussian-mixture(1024), 10k queries, k=100, Euclidean"


def args_parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--forms", default="fp32,bf16,bf16r132,fp8,fp8r132",
                    help="scoring forms: fp32, bf16, fp8, optionally with an explicit rerank "
                         "width (bf16r132 = BF16 scoring + exact rerank of 132 candidates)")
    ap.add_argument("--cpu-sample", type=int, default=0, help="queries in the CPU baseline sample")
    ap.add_argument("--cpu-shipped-sample", type=int, default=48,
                    help="queries in the one-at-a-time single-thread CPU sample")
    ap.add_argument("--ivf-profile", action="store_true",
                    help="only build the IVF-PQ index of the IVF section and run one search of "
                         "--nq queries at --nprobe (a small case for ncu captures)")
    ap.add_argument("--nprobe", type=int, default=2)
    ap.add_argument("--ivf-lists", type=int, default=1024, help="coarse lists of the --ivf-profile index")
    ap.add_argument("--coarse-fp32", action="store_true",
                    help="--ivf-profile: the FP32 coarse probe (HORA_OPT_EXACT_TC 0) instead of the certified one")
    ap.add_argument("--small", action="store_true", help="tiny workload for a quick check")
    ap.add_argument("--nq", type=int, default=0, help="override the number of queries (profiling)")
    ap.add_argument("--no-ivf", action="store_true", help="skip the IVF-PQ section")
    ap.add_argument("--ivf-epochs", type=int, default=25)
    ap.add_argument("--ivf-train-queries", type=int, default=200_000)
    ap.add_argument("--no-serve", action="store_true", help="skip the serving section")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the 4k-rerank, other-metric and FP64 sections (profiling runs)")
    ap.add_argument("--serve-rates", type=float, nargs="*", default=[20_000.0, 200_000.0])
    ap.add_argument("--serve-seconds", type=float, default=4.0)
    ap.add_argument("--serve-ivf-n", type=int, default=10_000_000,
                    help="rows of the serving mix's PQIVF index (96 dims)")
    return ap.parse_args()


# ---- distributed plumbing (replicas: one process per GPU, no data exchange) ----
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t)
        return float(t.item())


# ---- clocks sampled during the timed region --------------------------------------
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.p = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-i", str(self.idx), "-lms", "200"], stdout=subprocess.PIPE,
                                      stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.p = None

    def _read(self):
        for line in self.p.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict | None:
        if not self.p:
            return None
        time.sleep(0.25)
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        sm, mx, reasons = [], 0.0, set()
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for name, v in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                                "sw_power_cap"), f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# DRAM traffic of the BF16 scan in one step of the headline form (1M x 128,
# 10k queries, R = 132: the pivot pass and the probed pass over the base),
# from an ncu capture of dram__bytes_read.sum + dram__bytes_write.sum of the
# kernel (ncu --metrics ... -k regex:lowp_tile -s 2 -c 2 over this script
# with --forms bf16r132 --no-ivf --no-extras): pivot pass (argmin) 3.0 MB
# read, base pass 292.1 MB read + 12.8 MB written.  Captured while a CTA
# walked 32 tiles and before the MMA issuer polled its barriers; those
# change when the bytes move, not which (the base image is read once, the
# candidates written once).  ncu is not run inside the bench; the value is
# reported beside the live timing as the capture's figure.
SCAN_TRAFFIC_BYTES_PER_STEP = 307.9e6


def peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"],
                "bf16_tflops_sustained": d.get("bf16_tflops_sustained"), "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0,
            "source": "fallback"}


def make_data(small: bool, nq_override: int = 0):
    from hora_gb300 import synth
    n, nq = (20_000, 512) if small else (N_BASE, N_Q)
    if nq_override:
        nq = nq_override
    base = synth.mixture(n, DIM, N_CENTERS, stream=1)
    q = synth.mixture(nq, DIM, N_CENTERS, stream=2)
    return base, q


def form_options(H, form: str):
    """'fp32' | 'bf16' | 'fp8', optionally followed by r<R> (explicit rerank
    width; 0 = the library default) -> (precision, rerank)."""
    base, _, r = form.partition("r")
    prec = {"fp32": H.Precision.FP32, "bf16": H.Precision.BF16, "fp8": H.Precision.FP8}[base]
    return prec, int(r) if r else 0


def recall_at(ids, exact, r=10):
    hit = 0
    for a, b in zip(ids[:, :r], exact[:, :r]):
        hit += len(set(a.tolist()) & set(b.tolist()))
    return hit / (ids.shape[0] * r)


def cpu_sample_qps(base, q, k, n_sample, threads):
    """The oracle (C port of the reference's scan) on a bounded query sample."""
    from oracle import oracle as O
    O.build()
    qs = q[:n_sample]
    t0 = time.perf_counter()
    O.bf_search(base, qs, k, O.EUCLIDEAN, threads=threads)
    dt = time.perf_counter() - t0
    return n_sample / dt, dt


def cpu_as_shipped(base, q, k, n_sample):
    """The reference as its own benchmark drives it (examples/src/ann_bench.rs
    195-218): one query at a time on one thread, each search timed on its own
    and the latencies summed; queries/s = queries / summed latency."""
    from oracle import oracle as O
    O.build()
    lat = []
    for i in range(n_sample):
        t0 = time.perf_counter()
        O.bf_search(base, q[i:i + 1], k, O.EUCLIDEAN, threads=1)
        lat.append(time.perf_counter() - t0)
    tot = sum(lat)
    return {"value": n_sample / tot, "unit": "queries/s", "cores": 1, "kind": "port",
            "sample": f"{n_sample} queries one at a time on one thread against the full "
                      f"{base.shape[0]}x{base.shape[1]} base, k={k}, latency sum {tot:.1f} s",
            "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3)}


# ---- the reference's CPU-runnable case ---------------------------------------------
def run_config1(H, rank0: bool):
    """BruteForceIndex 10,000 x 64, entries Normal(0, 10), 1,000 queries, k = 10,
    Euclidean, exact FP32 on the GPU; the oracle port on the host beside it,
    single-threaded one query at a time (as the reference ships) and on all
    cores."""
    import torch
    from hora_gb300 import synth
    base = synth.normal(10_000, 64, 10.0, stream=11)
    q = synth.normal(1_000, 64, 10.0, stream=12)
    ix = H.BruteForceIndex(64)
    ix.madd(base, None)
    ix.build(H.Metric.Euclidean)
    dq = torch.from_numpy(q).cuda()
    ids = torch.empty((1000, 10), dtype=torch.int64, device="cuda")
    dd = torch.empty((1000, 10), dtype=torch.float32, device="cuda")
    ms = []
    for i in range(13):
        ix.search_batch(dq, 10, ids_out=ids, dist_out=dd)
        if i >= 3:
            ms.append(json.loads(ix.idx_info())["last_search_ms"])
    out = {"workload": "BruteForceIndex 10kx64 Normal(0,10), 1k queries, k=10, Euclidean, exact FP32",
           "gpu_qps": 1000 / (np.median(ms) / 1e3), "gpu_ms": float(np.median(ms))}
    if rank0:
        from oracle import oracle as O
        O.build()
        t0 = time.perf_counter()
        O.bf_search(base, q[:200], 10, O.EUCLIDEAN, threads=1)
        out["cpu_single_thread_qps"] = 200 / (time.perf_counter() - t0)
        th = os.cpu_count() or 1
        t0 = time.perf_counter()
        O.bf_search(base, q, 10, O.EUCLIDEAN, threads=th)
        out["cpu_all_cores_qps"] = 1000 / (time.perf_counter() - t0)
        out["cpu_cores"] = th
    return out


# ---- IVF-PQ (PQIVFIndex) on the same data ---------------------------------------------
def run_ivf(a, H, base, q, exact):
    """1M x 128 mixture, 1,024 lists, 32 x 8-bit PQ trained on the first 500k
    items, k = 10 with an exact FP32 rerank of 100 ADC candidates; QPS and
    recall@10 (against the exact brute-force top-10) for nprobe 1..128 and
    for the learned per-query nprobe trained on separate synthetic queries."""
    import torch
    from hora_gb300 import synth
    n = base.shape[0]
    params = H.IVFPQParams(n_sub=32, sub_bits=8, n_kmeans_center=1024, search_n_center=16,
                           train_epoch=a.ivf_epochs)
    ix = H.IVFPQIndex(DIM, params)
    ix.set_option(H.Option.TRAIN_SIZE, min(500_000, n))
    ix.madd(torch.from_numpy(base).cuda(), None)
    t0 = time.perf_counter()
    ix.build(H.Metric.Euclidean)
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    ix.set_option(H.Option.IVF_RERANK, 100)
    dq = torch.from_numpy(q).cuda()
    nq = q.shape[0]
    ids_d = torch.empty((nq, 10), dtype=torch.int64, device="cuda")
    dist_d = torch.empty((nq, 10), dtype=torch.float32, device="cuda")
    ex10 = exact[:, :10] if exact is not None else None

    def timed(nprobe=0, reps=3):
        ix.search_batch(dq, 10, nprobe=nprobe, ids_out=ids_d, dist_out=dist_d)
        ms = []
        for _ in range(reps):
            ix.search_batch(dq, 10, nprobe=nprobe, ids_out=ids_d, dist_out=dist_d)
            ms.append(json.loads(ix.idx_info())["last_search_ms"])
        torch.cuda.synchronize()
        ids = ids_d.cpu().numpy()
        rec = recall_at(ids, ex10, 10) if ex10 is not None else None
        return {"qps": nq / (np.median(ms) / 1e3), "recall@10": rec, "ms": float(np.median(ms))}

    sweep = {p: timed(p) for p in (1, 2, 4, 8, 16, 32, 64, 128)}
    out = {"workload": "IVFPQIndex 1Mx128 mixture, 1024 lists, 32x8-bit PQ, train 500k, "
                       f"{a.ivf_epochs} epochs, 10k queries, k=10, exact rerank of 100 ADC candidates",
           "build_s": build_s, "sweep": {str(k): v for k, v in sweep.items()}}
    # per-kernel time of one nprobe-2 search (CUDA events on the library stream)
    H._lib.profile_report()
    H._lib.profile(True)
    ix.search_batch(dq, 10, nprobe=2, ids_out=ids_d, dist_out=dist_d)
    H._lib.profile(False)
    out["kernels_nprobe2"] = {k: {"launches": v[0], "ms": v[1]} for k, v in H._lib.profile_report().items()}
    # the reference's CPU search (oracle port, ADC only) on the GPU-built index
    try:
        from oracle import oracle as O
        O.build()
        ex = ix.export()
        ex["metric"] = O.EUCLIDEAN
        ns, threads = 1000, os.cpu_count() or 1
        t0 = time.perf_counter()
        ci, _ = O.ivfpq_search(ex, q[:ns], 10, 2, threads=threads)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"kind": "port", "nprobe": 2, "queries": ns, "cores": threads,
                               "qps": ns / dt, "seconds": dt,
                               "recall@10": recall_at(ci, ex10[:ns], 10) if ex10 is not None else None,
                               "note": "ADC distances only (reference semantics, no rerank)"}
        # as shipped: one query per call on one thread, latency sum
        # (examples/src/ann_bench.rs:195-218; the reference's LUT loop may use
        # rayon threads, this port's is serial)
        lat = []
        for i in range(200):
            t1 = time.perf_counter()
            O.ivfpq_search(ex, q[i:i + 1], 10, 2, threads=1)
            lat.append(time.perf_counter() - t1)
        out["cpu_baseline"]["as_shipped"] = {"value": len(lat) / sum(lat), "unit": "queries/s", "cores": 1,
                                             "kind": "port", "sample": "200 queries one at a time, nprobe 2",
                                             "p50_ms": float(np.percentile(lat, 50) * 1e3)}
        del ex
    except Exception as e:  # the CPU leg is a reported baseline only
        out["cpu_baseline"] = {"error": str(e)}
    # learned nprobe (config 4): labels on 200k training queries from the
    # same mixture (a stream disjoint from the 10k evaluated here) = the
    # smallest nprobe whose top-10 reaches recall 0.95 against exact brute
    # force; the margin is calibrated on the last tenth of the training
    # queries for an aggregate recall@10 of 0.95; evaluated on the 10k
    # held-out bench queries against every fixed nprobe
    try:
        tq = synth.mixture(a.ivf_train_queries, DIM, N_CENTERS, stream=7)
        out["learned_train"] = []
        out["learned"] = []
        for p1 in (0, 1, 4):  # lists probed before the model reads its features
            ix.set_option(H.Option.NPROBE_PHASE1, p1)
            ix.set_option(H.Option.NPROBE_MARGIN, 0.0)
            t0 = time.perf_counter()
            st = ix.train_nprobe(tq, max_nprobe=128, recall_target=0.95, epochs=20)
            train_s = time.perf_counter() - t0
            model = json.loads(ix.idx_info())["ivfpq"]["nprobe_model"]
            ix.set_option(H.Option.LEARNED_NPROBE, 1)
            for extra in (0.0, 0.25):  # on top of the calibrated margin
                ix.set_option(H.Option.NPROBE_MARGIN, extra)
                r = timed(0)
                r["mean_nprobe"] = float(np.maximum(ix.predict_nprobe(q), max(p1, 1)).mean())
                r["margin"] = model["margin"] + extra
                r["phase1_probes"] = p1
                out["learned"].append(r)
            ix.set_option(H.Option.LEARNED_NPROBE, 0)
            ix.set_option(H.Option.NPROBE_MARGIN, 0.0)
            out["learned_train"].append({"phase1_probes": p1, "queries": a.ivf_train_queries,
                                         "seconds": train_s, "final_loss": st[0],
                                         "label_mean_log2": st[1], "model": model})
        ok = [dict(v, nprobe=int(p)) for p, v in sweep.items() if (v["recall@10"] or 0) >= 0.95]
        out["fixed_best_at_0.95"] = max(ok, key=lambda v: v["qps"]) if ok else None
        okl = [v for v in out["learned"] if (v["recall@10"] or 0) >= 0.95]
        out["learned_best_at_0.95"] = max(okl, key=lambda v: v["qps"]) if okl else None
    except H.HoraError as e:
        out["learned_error"] = str(e)
    return out, ix


def build_serving_ivf(a, H):
    """The serving mix's second index: PQIVFIndex over an N x 96 mixture
    (N = 10M by default, drawn on the device), 4,096 lists, 24 x 8-bit PQ,
    trained on the first 2M items; nprobe 16, exact rerank of 100."""
    import torch
    from hora_gb300 import synth
    n = a.serve_ivf_n
    X = synth.mixture_device(n, 96, 1024, stream=5)
    pool = synth.mixture_device(8192, 96, 1024, stream=6).cpu().numpy()
    params = H.IVFPQParams(n_sub=24, sub_bits=8, n_kmeans_center=4096, search_n_center=16,
                           train_epoch=a.ivf_epochs)
    ix = H.PQIVFIndex(96, params)
    ix.set_option(H.Option.TRAIN_SIZE, min(2_000_000, n))
    ix.madd(X, None)
    del X
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ix.build(H.Metric.Euclidean)
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    ix.set_option(H.Option.IVF_RERANK, 100)
    return ix, pool, {"n": n, "dim": 96, "lists": 4096, "pq": "24 x 8-bit", "train": min(2_000_000, n),
                      "epochs": a.ivf_epochs, "nprobe": 16, "rerank": 100, "build_s": build_s}


def run_serving(a, H, bf_index, bf_pool):
    """Open-loop Poisson load on two indexes: the 1M x 128 brute force in its
    headline form and a 10M x 96 PQIVFIndex (4,096 lists, 24 x 256 PQ);
    batch sizes log-uniform 1..256, k in {1, 10, 100}, HBM admission budget
    120 GB."""
    from hora_gb300 import loadgen
    ivx, ivf_pool, ivf_desc = build_serving_ivf(a, H)
    srv = H.Server([bf_index, ivx], n_slots=4, hbm_budget_bytes=120 << 30)
    out = {"workload": f"serving mix: Poisson arrivals, batch 1..256 log-uniform, k in {{1,10,100}}, "
                       f"50/50 brute force 1Mx128 / PQIVF {ivf_desc['n'] // 1_000_000}Mx96 "
                       f"(4096 lists, 24x256 PQ), 4 slots, HBM budget 120 GB",
           "ivf_index": ivf_desc, "rates": []}
    try:
        for rate in a.serve_rates:
            out["rates"].append(loadgen.run(srv, [bf_pool, ivf_pool], rate, a.serve_seconds,
                                            seed=int(rate)))
    finally:
        srv.close()
    return out


def run_form_extras(a, H, ix, base, q, dq, exact, head_prec, head_rerank):
    """Config-2 items beside the headline: the BF16 form with the 4,096-candidate
    rerank the configuration names, the other three metrics (exact FP32 and
    BF16 + rerank; Manhattan has no tensor-core form), and the returned
    distances and ids of a query sample against the FP64 exact oracle."""
    import torch
    from oracle import oracle as O
    nq = q.shape[0]
    out = {}

    def timed(index, k, reps=2):
        ids_d = torch.empty((nq, k), dtype=torch.int64, device="cuda")
        dist_d = torch.empty((nq, k), dtype=torch.float32, device="cuda")
        index.search_batch(dq, k, ids_out=ids_d, dist_out=dist_d)
        ms = []
        for _ in range(reps):
            index.search_batch(dq, k, ids_out=ids_d, dist_out=dist_d)
            ms.append(json.loads(index.idx_info())["last_search_ms"])
        torch.cuda.synchronize()
        return float(np.median(ms)), ids_d.cpu().numpy(), dist_d.cpu().numpy()

    # BF16 with a 4,096-candidate exact rerank
    ix.set_option(H.Option.PRECISION, H.Precision.BF16)
    ix.set_option(H.Option.RERANK, 4096)
    ms, ids, _ = timed(ix, K, reps=1)
    H._lib.profile_report()
    H._lib.profile(True)
    ms, ids, _ = timed(ix, K, reps=1)
    H._lib.profile(False)
    kern = {k: {"launches": v[0], "ms": v[1] / 2} for k, v in H._lib.profile_report().items()}
    out["bf16_rerank_4096"] = {"qps": nq / (ms / 1e3), "ms": ms, "kernels_per_search": kern,
                               "recall@10": recall_at(ids, exact, 10) if exact is not None else None,
                               "recall@100": recall_at(ids, exact, K) if exact is not None else None}
    # narrower rerank widths than the default max(2k, k+64)
    out["bf16_rerank_widths"] = {}
    for R in (132, 164):
        ix.set_option(H.Option.RERANK, R)
        ms, ids, _ = timed(ix, K)
        out["bf16_rerank_widths"][str(R)] = {
            "qps": nq / (ms / 1e3), "recall@10": recall_at(ids, exact, 10) if exact is not None else None,
            "recall@100": recall_at(ids, exact, K) if exact is not None else None}
    ix.set_option(H.Option.RERANK, head_rerank)
    ix.set_option(H.Option.PRECISION, head_prec)

    # the other metrics, each on its own index over the same base
    out["metrics"] = {}
    xb = torch.from_numpy(base).cuda()
    for name, mt in (("DotProduct", H.Metric.DotProduct), ("CosineSimilarity", H.Metric.CosineSimilarity),
                     ("Manhattan", H.Metric.Manhattan)):
        m = H.BruteForceIndex(DIM)
        m.madd(xb, None)
        m.build(mt)
        ms32, ids32, _ = timed(m, K)
        r = {"fp32_qps": nq / (ms32 / 1e3)}
        if mt != H.Metric.Manhattan:
            m.set_option(H.Option.PRECISION, H.Precision.BF16)
            ms16, ids16, _ = timed(m, K)
            r.update(bf16_qps=nq / (ms16 / 1e3), bf16_recall_at_10=recall_at(ids16, ids32, 10),
                     bf16_recall_at_100=recall_at(ids16, ids32, K))
        out["metrics"][name] = r
        del m
    del xb

    # a query sample against the FP64 exact oracle (Euclidean, headline form)
    ns = 32
    ids_h, d_h = ix.search_batch(q[:ns], K)
    O.build()
    i64, d64 = O.bf_exact_f64(base, q[:ns], K, O.EUCLIDEAN, threads=os.cpu_count() or 1)
    rel = np.abs(d_h.astype(np.float64) - d64) / np.maximum(np.abs(d64), 1e-30)
    out["fp64_check"] = {"queries": ns, "recall@10": recall_at(ids_h.astype(np.int64), i64, 10),
                         "recall@100": recall_at(ids_h.astype(np.int64), i64, K),
                         "max_rel_dist_err": float(rel.max()), "mean_rel_dist_err": float(rel.mean())}
    return out


def run_ssg(H, ix, base, cpu_bf_qps):
    """SSG's data-parallel build steps on the 1Mx128 base (SSGParams defaults,
    src/index/ssg_params.rs:40-48): the exact kNN graph with init_k = 100
    (build_knn_graph, ssg_idx.rs:69-98) in the headline form, and the root
    selection general_kmeans(root_size = 100, epoch = 256) (ssg_idx.rs:388)."""
    from oracle import oracle as O
    n = base.shape[0]
    out = {}
    t0 = time.perf_counter()
    g = ix.knn_graph(100)
    dt = time.perf_counter() - t0
    rows = np.random.default_rng(1).choice(n, 64, replace=False)
    threads = os.cpu_count() or 1
    i_ref, _ = O.bf_search(base, base[rows], 101, O.EUCLIDEAN, threads=threads)
    hit = 0
    for r, got in zip(rows, g[rows]):
        want = [j for j in i_ref[list(rows).index(r)] if j != r][:100]
        hit += len(set(want) & set(got.tolist()))
    out["knn_graph"] = {"k": 100, "seconds": dt, "rows_per_s": n / dt, "recall_vs_exact": hit / (64 * 100),
                        "cpu_estimate_s": n / cpu_bf_qps if cpu_bf_qps else None}
    del g
    ex = H.BruteForceIndex(DIM)
    ex.madd(base, None)
    ex.build(H.Metric.Euclidean)
    ex.general_kmeans(100, epoch=1, seed=1)
    t0 = time.perf_counter()
    roots = ex.general_kmeans(100, epoch=256, seed=1)
    dt = time.perf_counter() - t0
    ns = 50_000
    t1 = time.perf_counter()
    O.general_kmeans(base[:ns], 100, 2, O.EUCLIDEAN, seed=1, threads=threads)
    dc = time.perf_counter() - t1
    out["general_kmeans"] = {"k": 100, "epoch": 256, "seconds": dt, "roots_distinct": int(len(set(roots.tolist()))),
                             "cpu_sample": f"{ns} rows, 2 epochs, {threads} threads: {dc:.2f} s",
                             "cpu_estimate_s": dc * (n / ns) * (256 / 2)}
    del ex
    return out


def run_ivf_profile(a, H, base, q):
    """The IVF section's index (1M x 128, 1,024 lists, 32 x 8-bit PQ trained on
    the first 500k items, exact rerank of 100) and one search of the given
    queries at --nprobe."""
    import torch
    params = H.IVFPQParams(n_sub=32, sub_bits=8, n_kmeans_center=a.ivf_lists, search_n_center=a.nprobe,
                           train_epoch=a.ivf_epochs)
    ix = H.IVFPQIndex(DIM, params)
    if a.coarse_fp32:
        ix.set_option(H.Option.EXACT_TC, 0)
    ix.set_option(H.Option.TRAIN_SIZE, min(500_000, base.shape[0]))
    ix.madd(torch.from_numpy(base).cuda(), None)
    H._lib.profile_report()
    H._lib.profile(True)
    t0 = time.perf_counter()
    ix.build(H.Metric.Euclidean)
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    H._lib.profile(False)
    build_kern = {k: {"launches": v[0], "ms": v[1]} for k, v in H._lib.profile_report().items()}
    ix.set_option(H.Option.IVF_RERANK, 100)
    ix.search_batch(q, 10)
    first_ms = json.loads(ix.idx_info())["last_search_ms"]
    # three more searches under the library's per-kernel CUDA-event timing
    H._lib.profile_report()
    H._lib.profile(True)
    for _ in range(3):
        ix.search_batch(q, 10)
    H._lib.profile(False)
    kern = {k: {"launches": v[0] // 3, "ms": v[1] / 3} for k, v in H._lib.profile_report().items()}
    print(json.dumps({"workload": "IVF-PQ profile case", "queries": q.shape[0], "nprobe": a.nprobe,
                      "lists": a.ivf_lists, "coarse": "fp32" if a.coarse_fp32 else "default",
                      "build_s": build_s, "build_kernels": build_kern, "first_search_ms": first_ms,
                      "search_ms": json.loads(ix.idx_info())["last_search_ms"], "kernels_per_search": kern}),
          flush=True)


# ---- our implementation ------------------------------------------------------------
def run_ours(a, dist: Dist):
    import torch

    import hora_gb300 as H
    from hora_gb300 import build as B

    torch.cuda.set_device(dist.local)
    B.build()
    base, q = make_data(a.small, a.nq)
    if a.ivf_profile:
        run_ivf_profile(a, H, base, q)
        return
    n, nq = base.shape[0], q.shape[0]
    ix = H.BruteForceIndex(DIM)
    ix.madd(torch.from_numpy(base).cuda(), None)
    ix.build(H.Metric.Euclidean)
    dq = torch.from_numpy(q).cuda()
    ids_d = torch.empty((nq, K), dtype=torch.int64, device="cuda")
    dist_d = torch.empty((nq, K), dtype=torch.float32, device="cuda")

    # exact FP32 result (reference semantics) and per-form recall
    forms = {}
    exact = None
    order = [f for f in a.forms.split(",") if f]
    for form in order:
        prec, rerank = form_options(H, form)
        try:
            ix.set_option(H.Option.PRECISION, prec)
            ix.set_option(H.Option.RERANK, rerank)
            ix.search_batch(dq, K, ids_out=ids_d, dist_out=dist_d)
        except H.HoraError as e:
            forms[form] = {"error": str(e)}
            continue
        torch.cuda.synchronize()
        ids = ids_d.cpu().numpy()
        if form == "fp32":
            exact = ids
        rec10 = recall_at(ids, exact, 10) if exact is not None else None
        rec100 = recall_at(ids, exact, K) if exact is not None else None
        # warm-up and timing with device-resident inputs
        for _ in range(a.warmup):
            ix.search_batch(dq, K, ids_out=ids_d, dist_out=dist_d)
        torch.cuda.synchronize()
        dist.barrier()
        step_ms = []
        t0 = time.perf_counter()
        for _ in range(a.steps):
            ix.search_batch(dq, K, ids_out=ids_d, dist_out=dist_d)
            step_ms.append(json.loads(ix.idx_info())["last_search_ms"])
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        dist.barrier()
        dev = sum(step_ms) / 1e3
        forms[form] = {"qps": nq * a.steps / dev, "wall_qps": nq * a.steps / wall,
                       "rerank": rerank or "default", "recall@10": rec10, "recall@100": rec100,
                       "p50_ms": float(np.percentile(step_ms, 50)),
                       "p99_ms": float(np.percentile(step_ms, 99))}

    # without the exact form in --forms (profiling runs) recall is unknown and
    # the fastest listed form is timed
    ok = [f for f in order if "qps" in forms.get(f, {}) and
          (exact is None or (forms[f]["recall@10"] or 0) >= 0.95)]
    head = max(ok, key=lambda f: forms[f]["qps"]) if ok else "fp32"
    prec, head_rerank = form_options(H, head)
    ix.set_option(H.Option.PRECISION, prec)
    ix.set_option(H.Option.RERANK, head_rerank)

    # ---- headline timed region: device-resident inputs, kernel timing on ----
    for _ in range(a.warmup):
        ix.search_batch(dq, K, ids_out=ids_d, dist_out=dist_d)
    torch.cuda.synchronize()
    clocks = Clocks(dist.local)
    dist.barrier()
    torch.cuda.synchronize()
    H._lib.profile_report()
    H._lib.profile(True)
    l0 = H.launches()
    clocks.start()
    step_ms = []
    t0 = time.perf_counter()
    for _ in range(a.steps):
        ix.search_batch(dq, K, ids_out=ids_d, dist_out=dist_d)
        step_ms.append(json.loads(ix.idx_info())["last_search_ms"])
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t0
    launches = H.launches() - l0
    clk = clocks.stop()
    H._lib.profile(False)
    prof = H._lib.profile_report()
    dist.barrier()
    t_dev = sum(step_ms) / 1e3
    t_max = dist.max(t_dev)
    value = nq * a.steps * dist.world / t_max

    # ---- e2e through the public API with host buffers ----
    qh = torch.from_numpy(q).pin_memory().numpy()
    ids_h = torch.empty((nq, K), dtype=torch.int64).pin_memory().numpy().view(np.uint64)
    dist_h = torch.empty((nq, K), dtype=torch.float32).pin_memory().numpy()
    ix.search_batch(qh, K, ids_out=ids_h, dist_out=dist_h)
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(a.steps):
        ix.search_batch(qh, K, ids_out=ids_h, dist_out=dist_h)
    t_e2e = dist.max(time.perf_counter() - t0)
    e2e = {"value": nq * a.steps * dist.world / t_e2e, "unit": "queries/s",
           "h2d_bytes_per_step": int(q.nbytes), "d2h_bytes_per_step": int(ids_h.nbytes + dist_h.nbytes)}

    # ---- roofline of the dominant kernel (live CUDA-event timing) ----
    pk = peaks()
    top = max(prof.items(), key=lambda kv: kv[1][1]) if prof else (None, (0, 0.0))
    name, (nl, ms) = top
    roof = None
    if name:
        if name.startswith("fp32_tile"):
            # exact form: sub + mul + add per (query, row, dim), 1 FP32 op/lane/clk
            work = 3.0 * nq * n * DIM * a.steps
            peak_t = 152 * 128 * 2.07e9 / 1e12
            roof = {"bound": "fp32", "achieved": work / (ms / 1e3) / 1e12, "peak": peak_t,
                    "unit": "TFLOP/s", "peak_source": "nominal FP32 issue rate (152 SMs x 128 lanes x 2.07 GHz)"}
        else:
            work = 2.0 * nq * n * DIM * a.steps
            peak_t = pk["bf16_tflops"] * (2.0 if name.startswith("fp8") else 1.0)
            roof = {"bound": "tensor", "achieved": work / (ms / 1e3) / 1e12, "peak": peak_t,
                    "unit": "TFLOP/s", "peak_source": pk["source"] + (" bf16 x2 (fp8)" if name.startswith("fp8") else " bf16")}
        roof["frac"] = roof["achieved"] / roof["peak"]
        roof["kernel"] = name
        roof["launches"] = nl
        roof["kernel_ms_per_step"] = ms / a.steps
        # DRAM bytes of the same kernel's launches, from one ncu capture of
        # this workload; only the BF16 headline form was captured
        roof["traffic"] = SCAN_TRAFFIC_BYTES_PER_STEP * a.steps \
            if name == "bf16_tc_scan" and head == "bf16r132" and not a.small and nq == 10000 else None
        roof["traffic_unit"] = "bytes per timed region (dram__bytes_read.sum + dram__bytes_write.sum)"
        # per base row the image bytes a pass reads: BF16 rows and norm block,
        # or e4m3 rows plus the per-row scale and squared norm the drain reads
        roof["algorithmic_bytes"] = (n * (DIM * 2 + 32)) * a.steps if name == "bf16_tc_scan" else (
            (n * (DIM + 8)) * a.steps if name == "fp8_tc_scan" else None)
        roof["share_of_step"] = ms / (t_dev * 1e3)

    extras = run_form_extras(a, H, ix, base, q, dq, exact, prec, head_rerank) \
        if not a.small and not a.no_extras and dist.rank == 0 else None
    config1 = run_config1(H, dist.rank == 0) if not a.small else None
    ssg = run_ssg(H, ix, base, cpu_sample_qps(base, q, K, 256, os.cpu_count() or 1)[0]) \
        if not a.small and not a.no_extras and dist.rank == 0 else None
    ivf, serving = None, None
    if not a.no_ivf:
        ivf, ivx = run_ivf(a, H, base, q, exact)
        if not a.no_serve:
            del ivx
            serving = run_serving(a, H, ix, q)

    cpu = None
    if dist.rank == 0:
        ns = min(q.shape[0], a.cpu_sample or (32 if a.small else 2048))
        threads = os.cpu_count() or 1
        qps_cpu, dt = cpu_sample_qps(base, q, K, ns, threads)
        cpu = {"value": qps_cpu, "unit": "queries/s", "cores": threads, "kind": "port",
               "sample": f"{ns} of the 10k queries against the full 1Mx128 base, k=100, "
                         f"{threads} threads, {dt:.1f} s",
               "as_shipped": cpu_as_shipped(base, q, K, 4 if a.small else a.cpu_shipped_sample)}

    if dist.rank == 0:
        line = {
            "metric": "QPS at recall@10>=0.95 (brute force, 1Mx128, k=100)",
            "value": value, "unit": "queries/s", "n_gpus": dist.world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": t_max / a.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if head.startswith("fp32") else ("bf16" if head.startswith("bf16") else "e4m3"),
            "data": "synthetic (seeded gaussian mixture; ann-benchmarks sets unavailable offline)",
            "config": {"workload": WORKLOAD if not a.small else "small check", "n": n, "dim": DIM,
                       "queries": nq, "k": K, "form": head, "rerank": head_rerank or "default",
                       "l2_policy": "inputs larger than L2 (512 MB base)",
                       "parallelism": f"replicas x{dist.world}"},
            "forms": forms, "p50_ms": float(np.percentile(step_ms, 50)),
            "p99_ms": float(np.percentile(step_ms, 99)), "wall_s": t_wall,
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk, "ivfpq": ivf,
            "serving": serving, "config1": config1, "form_extras": extras, "ssg_build": ssg,
            "gpu_launches": launches, "kernels": {k: {"launches": v[0], "ms": v[1]} for k, v in prof.items()},
        }
        print(json.dumps(line), flush=True)


# ---- reference arm: the reference's CPU path (C port) on the host cores ------------
def run_reference(a, dist: Dist):
    if dist.rank != 0:
        return
    from oracle import oracle as O
    O.build()
    base, q = make_data(a.small, a.nq)
    threads = os.cpu_count() or 1
    ns = a.cpu_sample or max(threads * 2, 16)
    for i in range(a.warmup):
        O.bf_search(base, q[:threads], K, O.EUCLIDEAN, threads=threads)
    times = []
    for s in range(a.steps):
        qs = q[(s * ns) % q.shape[0]:][:ns]
        t0 = time.perf_counter()
        O.bf_search(base, qs, K, O.EUCLIDEAN, threads=threads)
        times.append(time.perf_counter() - t0)
    qps = ns * a.steps / sum(times)
    sample = f"{ns} queries per step of the 10k against the full 1Mx128 base, k=100, {threads} threads"
    print(json.dumps({
        "impl": "reference", "metric": "QPS at recall@10>=0.95 (brute force, 1Mx128, k=100)",
        "value": qps, "unit": "queries/s", "n_gpus": dist.world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": sum(times) / a.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded gaussian mixture)",
        "config": {"workload": WORKLOAD, "n": base.shape[0], "dim": DIM, "queries": ns, "k": K,
                   "form": "reference CPU scan (C port of src/index/bruteforce_idx.rs:47-73)"},
        "cpu_baseline": {"value": qps, "unit": "queries/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": qps, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def main():
    a = args_parse()
    dist = Dist()
    if a.impl == "reference":
        run_reference(a, dist)
    else:
        run_ours(a, dist)


if __name__ == "__main__":
    main()
