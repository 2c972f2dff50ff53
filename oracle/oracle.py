"""numpy front-end for the CPU oracle (oracle/hora_oracle.c).

TEST INFRASTRUCTURE ONLY — the checker.  tests/, __graft_entry__.smoke() and
bench.py's cpu_baseline / reference legs import this module; the product
package hora_gb300 never does.

Every function restates a piece of the reference; see hora_oracle.h for the
reference file:line each one follows and for the parity status (metrics are
pinned by the reference's known-answer tests; k-means / PQ randomness is
seeded and therefore "parity unpinned" against reference outputs).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "libhora_oracle.so")

EUCLIDEAN, MANHATTAN, DOT, COSINE = 3, 1, 2, 4
_lib = None

f32p = C.POINTER(C.c_float)
f64p = C.POINTER(C.c_double)
i64p = C.POINTER(C.c_int64)
u8p = C.POINTER(C.c_uint8)
u64p = C.POINTER(C.c_uint64)
i64 = C.c_int64


def build() -> str:
    """Compile the oracle with its Makefile (fast; a single C file)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _SO


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(
            os.path.join(_HERE, "hora_oracle.c")
        ):
            build()
        L = C.CDLL(_SO)
        L.horo_calc_dot_f32.restype = C.c_float
        L.horo_calc_dot_f32.argtypes = [f32p, f32p, i64]
        L.horo_calc_dot_f64.restype = C.c_double
        L.horo_calc_dot_f64.argtypes = [f64p, f64p, i64]
        L.horo_metric_f32.restype = C.c_float
        L.horo_metric_f32.argtypes = [f32p, f32p, i64, C.c_int, C.POINTER(C.c_int)]
        L.horo_metric_f64.restype = C.c_double
        L.horo_metric_f64.argtypes = [f64p, f64p, i64, C.c_int, C.POINTER(C.c_int)]
        L.horo_bf_search.argtypes = [f32p, i64, i64, f32p, i64, i64, C.c_int, i64p, f32p, C.c_int]
        L.horo_bf_exact_f64.argtypes = [f32p, i64, i64, f32p, i64, i64, C.c_int, i64p, f64p, C.c_int]
        L.horo_rng_instance_seed.restype = C.c_uint64
        L.horo_rng_instance_seed.argtypes = [C.c_uint64, C.c_uint64]
        L.horo_rng_next.restype = C.c_uint64
        L.horo_rng_next.argtypes = [u64p]
        L.horo_rng_unit.restype = C.c_double
        L.horo_rng_unit.argtypes = [u64p]
        L.horo_kmeans_init.argtypes = [f32p, i64, i64, i64, i64, f32p, i64, C.c_int, f32p]
        L.horo_kmeans_assign.argtypes = [f32p, i64, i64, i64, i64, f32p, f32p, i64, C.c_int, i64p]
        L.horo_kmeans_update.argtypes = [f32p, i64, i64, i64, i64, f32p, i64p, i64, C.c_int, f32p, i64p]
        L.horo_kmeans_split.argtypes = [f32p, i64p, i64, i64, i64, u64p]
        L.horo_kmeans_train.argtypes = [f32p, i64, i64, i64, i64, f32p, i64, i64, C.c_int,
                                        C.c_uint64, C.c_int, f32p]
        L.horo_pq_ranges.argtypes = [i64, i64, i64p, i64p]
        L.horo_ivfpq_build.argtypes = [f32p, i64, i64, i64, i64, i64, i64, C.c_int, C.c_uint64,
                                       C.c_int, i64, f32p, i64p, i64p, f32p, u8p, u8p]
        L.horo_pq_encode.argtypes = [f32p, i64, i64, f32p, f32p, i64, i64, u8p]
        L.horo_pq_lut.argtypes = [f32p, i64, f32p, f32p, i64, i64, f32p]
        L.horo_ivfpq_search.argtypes = [f32p, i64, i64, i64p, i64p, f32p, u8p, u8p, i64, i64,
                                        C.c_int, f32p, i64, i64, i64, i64p, f32p, C.c_int]
        L.horo_ivf_coarse.argtypes = [f32p, i64, i64, C.c_int, f32p, f32p]
        L.horo_pq_build.argtypes = [f32p, i64, i64, i64, i64, i64, C.c_int, C.c_uint64, C.c_int, i64,
                                    f32p, u8p]
        L.horo_pq_search.argtypes = [f32p, u8p, i64, i64, i64, i64, C.c_int, f32p, i64, i64, i64p,
                                     f32p, C.c_int]
        L.horo_general_kmeans.argtypes = [f32p, i64, i64, i64, i64, C.c_int, i64p, C.c_uint64, i64p,
                                          f32p, C.c_int]
        L.horo_mlp_forward.argtypes = [f32p, i64, i64, i64, f32p, i64, f32p]
        L.horo_mlp_loss_grad.restype = C.c_double
        L.horo_mlp_loss_grad.argtypes = [f32p, i64, i64, i64, f32p, f32p, i64, C.c_float, f64p]
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t) if a is not None else None


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def calc_dot(a, b) -> float:
    a, b = _f32(a), _f32(b)
    return float(lib().horo_calc_dot_f32(_p(a, f32p), _p(b, f32p), a.size))


def calc_dot_f64(a, b) -> float:
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    return float(lib().horo_calc_dot_f64(_p(a, f64p), _p(b, f64p), a.size))


def metric(a, b, mt: int) -> float:
    a, b = _f32(a), _f32(b)
    err = C.c_int(0)
    v = lib().horo_metric_f32(_p(a, f32p), _p(b, f32p), a.size, mt, C.byref(err))
    if err.value:
        raise ValueError("unknown method")
    return float(v)


def metric_f64(a, b, mt: int) -> float:
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    err = C.c_int(0)
    v = lib().horo_metric_f64(_p(a, f64p), _p(b, f64p), a.size, mt, C.byref(err))
    if err.value:
        raise ValueError("unknown method")
    return float(v)


def bf_search(base, queries, k: int, mt: int, threads: int = 1):
    base, queries = _f32(base), _f32(queries)
    n, d = base.shape
    nq = queries.shape[0]
    idx = np.empty((nq, k), np.int64)
    dist = np.empty((nq, k), np.float32)
    rc = lib().horo_bf_search(_p(base, f32p), n, d, _p(queries, f32p), nq, k, mt,
                              _p(idx, i64p), _p(dist, f32p), threads)
    if rc:
        raise ValueError("unknown method")
    return idx, dist


def bf_exact_f64(base, queries, k: int, mt: int, threads: int = 1):
    base, queries = _f32(base), _f32(queries)
    n, d = base.shape
    nq = queries.shape[0]
    idx = np.empty((nq, k), np.int64)
    dist = np.empty((nq, k), np.float64)
    lib().horo_bf_exact_f64(_p(base, f32p), n, d, _p(queries, f32p), nq, k, mt,
                            _p(idx, i64p), _p(dist, f64p), threads)
    return idx, dist


def rng_instance_seed(seed: int, inst: int) -> int:
    return int(lib().horo_rng_instance_seed(seed, inst))


def rng_units(state: int, n: int):
    s = C.c_uint64(state)
    return [float(lib().horo_rng_unit(C.byref(s))) for _ in range(n)]


def kmeans_init(data, begin, end, n_center, residual=None, accum_f64=True):
    data = _f32(data)
    res = _f32(residual) if residual is not None else None
    out = np.empty((n_center, end - begin), np.float32)
    lib().horo_kmeans_init(_p(data, f32p), data.shape[0], data.shape[1], begin, end,
                           _p(res, f32p), n_center, int(accum_f64), _p(out, f32p))
    return out


def kmeans_assign(data, begin, end, centers, mt, residual=None):
    data, centers = _f32(data), _f32(centers)
    res = _f32(residual) if residual is not None else None
    out = np.empty(data.shape[0], np.int64)
    lib().horo_kmeans_assign(_p(data, f32p), data.shape[0], data.shape[1], begin, end,
                             _p(res, f32p), _p(centers, f32p), centers.shape[0], mt, _p(out, i64p))
    return out


def kmeans_update(data, begin, end, assign, n_center, residual=None, accum_f64=True):
    data = _f32(data)
    res = _f32(residual) if residual is not None else None
    assign = np.ascontiguousarray(assign, np.int64)
    cent = np.empty((n_center, end - begin), np.float32)
    cnt = np.empty(n_center, np.int64)
    lib().horo_kmeans_update(_p(data, f32p), data.shape[0], data.shape[1], begin, end,
                             _p(res, f32p), _p(assign, i64p), n_center, int(accum_f64),
                             _p(cent, f32p), _p(cnt, i64p))
    return cent, cnt


def kmeans_split(centers, counts, batch_size, rng_state):
    centers = _f32(centers).copy()
    counts = np.ascontiguousarray(counts, np.int64).copy()
    s = C.c_uint64(rng_state)
    rc = lib().horo_kmeans_split(_p(centers, f32p), _p(counts, i64p), centers.shape[0],
                                 centers.shape[1], batch_size, C.byref(s))
    if rc:
        raise RuntimeError("split_center failed")
    return centers, counts, int(s.value)


def kmeans_train(data, begin, end, n_center, n_epoch, mt, seed, residual=None, accum_f64=True):
    data = _f32(data)
    res = _f32(residual) if residual is not None else None
    out = np.empty((n_center, end - begin), np.float32)
    rc = lib().horo_kmeans_train(_p(data, f32p), data.shape[0], data.shape[1], begin, end,
                                 _p(res, f32p), n_center, n_epoch, mt, seed, int(accum_f64),
                                 _p(out, f32p))
    if rc:
        raise RuntimeError("kmeans failed")
    return out


def pq_ranges(dim, n_sub):
    b = np.empty(n_sub, np.int64)
    e = np.empty(n_sub, np.int64)
    lib().horo_pq_ranges(dim, n_sub, _p(b, i64p), _p(e, i64p))
    return b, e


def pq_dmax(dim, n_sub):
    sd = dim // n_sub
    return sd + (1 if dim % sd else 0)


def ivfpq_build(data, n_sub, sub_bits, n_list, n_epoch, mt, seed, accum_f64=True, train_size=0):
    data = _f32(data)
    n, d = data.shape
    K = 1 << sub_bits
    dm = pq_dmax(d, n_sub)
    centers = np.empty((n_list, d), np.float32)
    offs = np.empty(n_list + 1, np.int64)
    items = np.empty(n, np.int64)
    books = np.empty((n_list, n_sub, K, dm), np.float32)
    codes = np.empty((n, n_sub), np.uint8)
    trained = np.empty(n_list, np.uint8)
    rc = lib().horo_ivfpq_build(_p(data, f32p), n, d, n_sub, sub_bits, n_list, n_epoch, mt, seed,
                                int(accum_f64), train_size, _p(centers, f32p), _p(offs, i64p),
                                _p(items, i64p), _p(books, f32p), _p(codes, u8p), _p(trained, u8p))
    if rc:
        raise RuntimeError(f"ivfpq build failed rc={rc}")
    return dict(centers=centers, offsets=offs, items=items, codebooks=books, codes=codes,
                trained=trained, n_sub=n_sub, sub_bits=sub_bits, metric=mt)


def pq_build(data, n_sub, sub_bits, n_epoch, mt, seed, accum_f64=True, train_size=0):
    """Flat PQIndex build (pq_idx.rs:122-149): codebooks [n_sub, K, dmax], codes [n, n_sub]."""
    data = _f32(data)
    n, d = data.shape
    K = 1 << sub_bits
    books = np.empty((n_sub, K, pq_dmax(d, n_sub)), np.float32)
    codes = np.empty((n, n_sub), np.uint8)
    rc = lib().horo_pq_build(_p(data, f32p), n, d, n_sub, sub_bits, n_epoch, mt, seed, int(accum_f64),
                             train_size, _p(books, f32p), _p(codes, u8p))
    if rc:
        raise RuntimeError(f"pq build failed rc={rc}")
    return dict(codebooks=books, codes=codes, n_sub=n_sub, sub_bits=sub_bits, metric=mt, dim=d)


def pq_search(ix, queries, k, threads=1):
    """Flat PQIndex search_knn_adc (pq_idx.rs:165-193): ids ascending by ADC distance."""
    queries = _f32(queries)
    nq, d = queries.shape
    idx = np.empty((nq, k), np.int64)
    dist = np.empty((nq, k), np.float32)
    lib().horo_pq_search(_p(ix["codebooks"], f32p), _p(ix["codes"], u8p), ix["codes"].shape[0], d,
                         ix["n_sub"], ix["sub_bits"], ix["metric"], _p(queries, f32p), nq, k,
                         _p(idx, i64p), _p(dist, f32p), threads)
    return idx, dist


def general_kmeans(data, k, epoch, mt, seed=0, init_rows=None, threads=1):
    """kmeans::general_kmeans (kmeans.rs:216-289): (roots [k] int64, means [k, dim])."""
    data = _f32(data)
    n, d = data.shape
    roots = np.zeros(k, np.int64)
    means = np.zeros((k, d), np.float32)
    init = None if init_rows is None else np.ascontiguousarray(init_rows, dtype=np.int64)
    rc = lib().horo_general_kmeans(_p(data, f32p), n, d, k, epoch, mt, _p(init, i64p), seed,
                                   _p(roots, i64p), _p(means, f32p), threads)
    if rc:
        raise ValueError("init row out of range")
    return roots, means


def pq_encode(data, list_center, codebook, n_sub, sub_bits):
    data, list_center, codebook = _f32(data), _f32(list_center), _f32(codebook)
    out = np.empty((data.shape[0], n_sub), np.uint8)
    lib().horo_pq_encode(_p(data, f32p), data.shape[0], data.shape[1], _p(list_center, f32p),
                         _p(codebook, f32p), n_sub, sub_bits, _p(out, u8p))
    return out


def pq_lut(query, list_center, codebook, n_sub, sub_bits):
    query, list_center, codebook = _f32(query), _f32(list_center), _f32(codebook)
    out = np.empty((n_sub, 1 << sub_bits), np.float32)
    lib().horo_pq_lut(_p(query, f32p), query.size, _p(list_center, f32p), _p(codebook, f32p),
                      n_sub, sub_bits, _p(out, f32p))
    return out


def ivfpq_search(ix, queries, k, nprobe, threads=1):
    queries = _f32(queries)
    nq, d = queries.shape
    idx = np.empty((nq, k), np.int64)
    dist = np.empty((nq, k), np.float32)
    c = ix
    lib().horo_ivfpq_search(_p(c["centers"], f32p), c["centers"].shape[0], d,
                            _p(c["offsets"], i64p), _p(c["items"], i64p), _p(c["codebooks"], f32p),
                            _p(c["codes"], u8p), _p(c["trained"], u8p), c["n_sub"], c["sub_bits"],
                            c["metric"], _p(queries, f32p), nq, k, nprobe, _p(idx, i64p),
                            _p(dist, f32p), threads)
    return idx, dist


def ivf_coarse(centers, query, mt):
    centers, query = _f32(centers), _f32(query)
    out = np.empty(centers.shape[0], np.float32)
    lib().horo_ivf_coarse(_p(centers, f32p), centers.shape[0], centers.shape[1], mt,
                          _p(query, f32p), _p(out, f32p))
    return out


def mlp_forward(params, x, f, h1, h2):
    params, x = _f32(params), _f32(x)
    out = np.empty(x.shape[0], np.float32)
    lib().horo_mlp_forward(_p(params, f32p), f, h1, h2, _p(x, f32p), x.shape[0], _p(out, f32p))
    return out


def mlp_loss_grad(params, x, y, f, h1, h2, alpha=1.0):
    params, x, y = _f32(params), _f32(x), _f32(y)
    g = np.empty(params.size, np.float64)
    loss = lib().horo_mlp_loss_grad(_p(params, f32p), f, h1, h2, _p(x, f32p), _p(y, f32p),
                                    x.shape[0], alpha, _p(g, f64p))
    return float(loss), g
