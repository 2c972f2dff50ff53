"""Python mirror of hora's index API over the C ABI.

The classes follow trait ANNIndex (src/core/ann_index.rs:25-121) and
SerializableIndex (:141-158) method for method: add / madd / build / built /
rebuild / search / search_nodes / name / nodes_size / clear / idx_info /
dimension / dump / load, plus batched forms (search_batch) that expose the
GPU.  Ids are uint64 (the reference's T = usize in its bindings).

Inputs may be numpy arrays (host memory; copied by the library) or CUDA
tensors exposing data_ptr() (device memory; used in place).
"""
from __future__ import annotations

import ctypes as C
import enum
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import IVFPQParamsC, PQParamsC, check, lib

NO_ID = np.uint64(0xFFFFFFFFFFFFFFFF)


class Metric(enum.IntEnum):
    """Same variant order as src/core/metrics.rs:5-13."""
    Unknown = 0
    Manhattan = 1
    DotProduct = 2
    Euclidean = 3
    CosineSimilarity = 4
    Angular = 5


class Precision(enum.IntEnum):
    FP32 = 0
    BF16 = 1
    FP8 = 2


class Option(enum.IntEnum):
    PRECISION = 1
    RERANK = 2
    SEED = 3
    TRAIN_SIZE = 4
    ACCUM_F64 = 5
    CAND_CAP = 6
    LEARNED_NPROBE = 7
    NPROBE_MARGIN = 8
    NPROBE_MAX = 9
    IVF_RERANK = 10
    NPROBE_PHASE1 = 11
    BF_PROBE = 12
    EXACT_TC = 13


@dataclass
class BruteForceParams:
    """BruteForceParams {} (src/index/bruteforce_params.rs:5-14)."""


@dataclass
class IVFPQParams:
    """IVFPQParams with the reference defaults (src/index/pq_params.rs:80-91)
    and its consuming builder setters (:52-78)."""
    n_sub: int = 25
    sub_bits: int = 4
    n_kmeans_center: int = 256
    search_n_center: int = 8
    train_epoch: int = 100

    def with_n_sub(self, v):
        self.n_sub = v
        return self

    def with_sub_bits(self, v):
        self.sub_bits = v
        return self

    def with_n_kmeans_center(self, v):
        self.n_kmeans_center = v
        return self

    def with_search_n_center(self, v):
        self.search_n_center = v
        return self

    def with_train_epoch(self, v):
        self.train_epoch = v
        return self


@dataclass
class PQParams:
    """PQParams with the reference defaults (src/index/pq_params.rs:32-41)
    and its consuming builder setters (:15-30)."""
    n_sub: int = 4
    sub_bits: int = 4
    train_epoch: int = 100

    def with_n_sub(self, v):
        self.n_sub = v
        return self

    def with_sub_bits(self, v):
        self.sub_bits = v
        return self

    def with_train_epoch(self, v):
        self.train_epoch = v
        return self


@dataclass
class Node:
    """core::node::Node: a vector and its optional id (src/core/node.rs:93-97)."""
    vectors: np.ndarray
    idx: int | None = None


def _ptr(a):
    """(pointer, keepalive, is_device) for numpy arrays or CUDA tensors."""
    if a is None:
        return None, None, False
    if hasattr(a, "data_ptr") and getattr(a, "is_cuda", False):
        return C.c_void_p(a.data_ptr()), a, True
    arr = np.ascontiguousarray(a)
    return C.c_void_p(arr.ctypes.data), arr, False


class _Index:
    kind = 0

    def __init__(self, dimension: int, params=None, _handle=None):
        self._h = C.c_void_p()
        if _handle is not None:
            self._h = _handle
            return
        p = None
        if isinstance(params, IVFPQParams):
            self._cp = IVFPQParamsC(params.n_sub, params.sub_bits, params.n_kmeans_center,
                                    params.search_n_center, params.train_epoch)
            p = C.cast(C.pointer(self._cp), C.c_void_p)
        elif isinstance(params, PQParams):
            self._cp = PQParamsC(params.n_sub, params.sub_bits, params.train_epoch)
            p = C.cast(C.pointer(self._cp), C.c_void_p)
        check(lib().hora_index_create(self.kind, dimension, p, C.byref(self._h)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib._lib is not None:
            _lib._lib.hora_index_free(h)
            self._h = C.c_void_p()

    # ---- ANNIndex -------------------------------------------------------------
    def add(self, vs, idx: int):
        """add (ann_index.rs:41-43)."""
        v = np.asarray(vs, dtype=np.float32).reshape(1, -1)
        self._add(v, np.array([idx], dtype=np.uint64))

    def add_node(self, node: Node):
        """add_node (ann_index.rs:36)."""
        self.add(node.vectors, node.idx if node.idx is not None else self.nodes_size())

    def madd(self, vss, indices):
        """madd (ann_index.rs:48-59): all vectors at once.  indices=None numbers
        the rows from the current size."""
        if indices is None:
            n = vss.shape[0] if hasattr(vss, "shape") else len(vss)
            indices = np.arange(self.nodes_size(), self.nodes_size() + n, dtype=np.uint64)
        if len(vss) != len(indices):
            raise _lib.HoraError(-12, "vector's size is different with index")
        if hasattr(vss, "data_ptr"):
            self._add(vss, indices)
        else:
            self._add(np.asarray(vss, dtype=np.float32), np.asarray(indices, dtype=np.uint64))

    def _add(self, vecs, ids):
        n = vecs.shape[0]
        if vecs.shape[1] != self.dimension():
            raise _lib.HoraError(-2, "dimension is different")
        pv, kv, _ = _ptr(vecs if hasattr(vecs, "data_ptr") else np.ascontiguousarray(vecs, np.float32))
        pi, ki, _ = _ptr(ids if ids is None or hasattr(ids, "data_ptr") else np.ascontiguousarray(ids, np.uint64))
        check(lib().hora_add(self._h, pv, pi, n))

    def build(self, mt: Metric):
        check(lib().hora_build(self._h, int(mt)))

    def built(self) -> bool:
        o = C.c_int()
        check(lib().hora_built(self._h, C.byref(o)))
        return bool(o.value)

    def rebuild(self, mt: Metric):
        check(lib().hora_rebuild(self._h, int(mt)))

    def search_batch(self, queries, k: int, nprobe: int = 0, ids_out=None, dist_out=None):
        """Batched search: (ids [nq,k] uint64, distances [nq,k] float32).
        Missing results (k > items) have id NO_ID and distance +inf."""
        if hasattr(queries, "data_ptr"):
            nq = queries.shape[0]
            pq_, kq, _ = _ptr(queries)
        else:
            q = np.ascontiguousarray(queries, dtype=np.float32).reshape(-1, self.dimension())
            nq = q.shape[0]
            pq_, kq, _ = _ptr(q)
        ids = ids_out if ids_out is not None else np.empty((nq, k), np.uint64)
        dist = dist_out if dist_out is not None else np.empty((nq, k), np.float32)
        pi, ki, _ = _ptr(ids)
        pd, kd, _ = _ptr(dist)
        if nprobe:
            check(lib().hora_search_nprobe(self._h, pq_, nq, k, nprobe, pi, pd))
        else:
            check(lib().hora_search(self._h, pq_, nq, k, pi, pd))
        return ids, dist

    def search(self, item, k: int):
        """search (ann_index.rs:91-97): ids of the k nearest, ascending."""
        item = np.asarray(item, dtype=np.float32)
        assert item.size == self.dimension()
        ids, _ = self.search_batch(item.reshape(1, -1), k)
        return [int(i) for i in ids[0] if i != NO_ID]

    def search_nodes(self, item, k: int):
        """search_nodes (ann_index.rs:81-84): [(Node, distance)] ascending."""
        item = np.ascontiguousarray(item, dtype=np.float32).reshape(1, -1)
        assert item.shape[1] == self.dimension()
        d = self.dimension()
        ids = np.empty((1, k), np.uint64)
        dist = np.empty((1, k), np.float32)
        vecs = np.empty((1, k, d), np.float32)
        check(lib().hora_search_nodes(self._h, C.c_void_p(item.ctypes.data), 1, k,
                                      C.c_void_p(ids.ctypes.data), C.c_void_p(dist.ctypes.data),
                                      C.c_void_p(vecs.ctypes.data)))
        return [(Node(vecs[0, j].copy(), int(ids[0, j])), float(dist[0, j]))
                for j in range(k) if ids[0, j] != NO_ID]

    def name(self) -> str:
        s = C.c_char_p()
        check(lib().hora_name(self._h, C.byref(s)))
        return s.value.decode()

    def nodes_size(self) -> int:
        o = C.c_uint64()
        check(lib().hora_nodes_size(self._h, C.byref(o)))
        return o.value

    def dimension(self) -> int:
        o = C.c_uint64()
        check(lib().hora_dimension(self._h, C.byref(o)))
        return o.value

    def clear(self):
        check(lib().hora_clear(self._h))

    def idx_info(self) -> str:
        buf = C.create_string_buffer(1 << 16)
        check(lib().hora_idx_info(self._h, buf, len(buf)))
        return buf.value.decode()

    # ---- GPU options ------------------------------------------------------------
    def set_option(self, key: Option, value: float):
        check(lib().hora_set_option(self._h, int(key), float(value)))

    def get_option(self, key: Option) -> float:
        o = C.c_double()
        check(lib().hora_get_option(self._h, int(key), C.byref(o)))
        return o.value

    # ---- SerializableIndex --------------------------------------------------------
    def dump(self, path: str):
        check(lib().hora_dump(self._h, path.encode()))

    @classmethod
    def load(cls, path: str):
        h = C.c_void_p()
        check(lib().hora_load(path.encode(), C.byref(h)))
        obj = cls.__new__(cls)
        _Index.__init__(obj, 0, None, _handle=h)
        return obj


class BruteForceIndex(_Index):
    """BruteForceIndex<f32, u64> (src/index/bruteforce_idx.rs)."""
    kind = 0

    def __init__(self, dimension: int, params: BruteForceParams | None = None, _handle=None):
        super().__init__(dimension, params, _handle)


def _knn_graph(self, k: int):
    """SSGIndex::build_knn_graph (src/index/ssg_idx.rs:69-98): [n, k] row
    numbers of each row's k nearest other rows, farthest first."""
    out = np.empty((self.nodes_size(), k), np.uint64)
    check(lib().hora_knn_graph(self._h, k, C.c_void_p(out.ctypes.data)))
    return out


def _general_kmeans(self, k: int, epoch: int = 256, seed: int = 0, init_rows=None, return_means: bool = False):
    """kmeans::general_kmeans (src/core/kmeans.rs:216-289) over this index's
    rows with its metric: the row number nearest to each of the k means after
    `epoch` rounds (SSG calls it with epoch 256, ssg_idx.rs:388).  The means
    start at init_rows (k row numbers) or at k rows drawn with replacement
    from the seeded stream.  Returns roots [k] (uint64), and the means [k, dim]
    (float32, NaN for a mean that lost all its rows) when return_means."""
    dim = self.dimension()
    if self.nodes_size() == 0 and self.built():
        empty = np.empty(0, np.uint64)
        return (empty, np.empty((0, dim), np.float32)) if return_means else empty
    roots = np.empty(k, np.uint64)
    means = np.empty((k, dim), np.float32) if return_means else None
    init = None
    if init_rows is not None:
        init = np.ascontiguousarray(init_rows, dtype=np.uint64)
        if init.shape != (k,):
            raise _lib.HoraError(-1, "init_rows must hold k row numbers")
    check(lib().hora_general_kmeans(self._h, k, epoch, None if init is None else C.c_void_p(init.ctypes.data),
                                    seed, C.c_void_p(roots.ctypes.data),
                                    None if means is None else C.c_void_p(means.ctypes.data)))
    return (roots, means) if return_means else roots


BruteForceIndex.knn_graph = _knn_graph
BruteForceIndex.general_kmeans = _general_kmeans


class IVFPQIndex(_Index):
    """IVFPQIndex<f32, u64> (src/index/pq_idx.rs:267-523), a.k.a. PQIVFIndex."""
    kind = 1

    def __init__(self, dimension: int, params: IVFPQParams | None = None, _handle=None):
        super().__init__(dimension, params if params is not None else IVFPQParams(), _handle)

    def layout(self):
        a = [C.c_uint64() for _ in range(4)]
        check(lib().hora_ivfpq_layout(self._h, *[C.byref(x) for x in a]))
        return tuple(x.value for x in a)  # n_list, n_sub, sub_bits, dmax

    def export(self):
        n_list, n_sub, sub_bits, dmax = self.layout()
        n, d = self.nodes_size(), self.dimension()
        K = 1 << sub_bits
        out = dict(
            centers=np.empty((n_list, d), np.float32), offsets=np.empty(n_list + 1, np.int64),
            items=np.empty(n, np.int64), codebooks=np.empty((n_list, n_sub, K, dmax), np.float32),
            codes=np.empty((n, n_sub), np.uint8), trained=np.empty(n_list, np.uint8))
        check(lib().hora_ivfpq_export(self._h, *[C.c_void_p(out[k].ctypes.data) for k in
                                                 ("centers", "offsets", "items", "codebooks",
                                                  "codes", "trained")]))
        out.update(n_sub=n_sub, sub_bits=sub_bits)
        return out

    def set_codebooks(self, centers, codebooks):
        c = np.ascontiguousarray(centers, np.float32)
        b = np.ascontiguousarray(codebooks, np.float32)
        check(lib().hora_ivfpq_set_codebooks(self._h, C.c_void_p(c.ctypes.data),
                                             C.c_void_p(b.ctypes.data)))

    def train_nprobe(self, train_queries, max_nprobe=128, recall_target=0.95, epochs=30):
        q = np.ascontiguousarray(train_queries, np.float32)
        stats = (C.c_double * 4)()
        check(lib().hora_ivfpq_train_nprobe(self._h, C.c_void_p(q.ctypes.data), q.shape[0],
                                            max_nprobe, recall_target, epochs, stats))
        return list(stats)

    def nprobe_features(self, queries):
        q = np.ascontiguousarray(queries, np.float32)
        out = np.empty((q.shape[0], 40), np.float32)
        check(lib().hora_ivfpq_nprobe_features(self._h, C.c_void_p(q.ctypes.data), q.shape[0],
                                               C.c_void_p(out.ctypes.data)))
        return out

    def predict_nprobe(self, queries):
        q = np.ascontiguousarray(queries, np.float32)
        out = np.empty(q.shape[0], np.uint32)
        check(lib().hora_ivfpq_predict_nprobe(self._h, C.c_void_p(q.ctypes.data), q.shape[0],
                                              C.c_void_p(out.ctypes.data)))
        return out


PQIVFIndex = IVFPQIndex


class PQIndex(IVFPQIndex):
    """PQIndex<f32, u64> (src/index/pq_idx.rs:21-265): product quantization of
    the raw vectors, codebooks trained with the build metric, every item
    scanned by ADC.  layout()/export() report one list centred at zero."""
    kind = 2

    def __init__(self, dimension: int, params: PQParams | None = None, _handle=None):
        _Index.__init__(self, dimension, params if params is not None else PQParams(), _handle)


def load_reference(path: str, kind):
    """SerializableIndex::load of a file the reference wrote (bincode of
    BruteForceIndex / PQIndex / IVFPQIndex<f32, usize>); `kind` is the class."""
    h = C.c_void_p()
    check(lib().hora_load_reference(path.encode(), kind.kind, C.byref(h)))
    obj = kind.__new__(kind)
    _Index.__init__(obj, 0, None, _handle=h)
    return obj


class Server:
    """Continuous-batching request loop over built indexes (hora_server_*).

    submit() queues a request (host buffers; they must stay alive until
    wait() returns) and returns a ticket; wait() blocks until it finished and
    returns its latency in ms.  stats() gives completed requests / queries,
    p50 / p99 latency (ms), peak in-flight requests, peak admitted bytes and
    rejected requests."""

    def __init__(self, indexes, n_slots: int = 4, hbm_budget_bytes: int = 120 << 30):
        self._idx = list(indexes)
        arr = (C.c_void_p * len(self._idx))(*[ix._h for ix in self._idx])
        self._h = C.c_void_p()
        check(lib().hora_server_create(arr, len(self._idx), n_slots, hbm_budget_bytes,
                                       C.byref(self._h)))
        self._keep = {}

    def submit(self, index_no: int, queries, k: int):
        q = np.ascontiguousarray(queries, dtype=np.float32)
        ids = np.empty((q.shape[0], k), np.uint64)
        dist = np.empty((q.shape[0], k), np.float32)
        t = C.c_uint64()
        check(lib().hora_server_submit(self._h, index_no, C.c_void_p(q.ctypes.data), q.shape[0], k,
                                       C.c_void_p(ids.ctypes.data), C.c_void_p(dist.ctypes.data),
                                       C.byref(t)))
        self._keep[t.value] = (q, ids, dist)
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1):
        lat = C.c_double()
        rc = lib().hora_server_wait(self._h, ticket, timeout_ms, C.byref(lat))
        q, ids, dist = self._keep.pop(ticket) if rc != -11 else self._keep[ticket]
        check(rc)
        return ids, dist, lat.value

    def stats(self) -> dict:
        o = (C.c_double * 7)()
        check(lib().hora_server_stats(self._h, o))
        keys = ("completed", "queries", "p50_ms", "p99_ms", "max_inflight", "max_admitted_bytes",
                "rejected")
        return dict(zip(keys, list(o)))

    def request_bytes(self, index_no: int, nq: int, k: int) -> int:
        out = C.c_uint64()
        check(lib().hora_server_request_bytes(self._h, index_no, nq, k, C.byref(out)))
        return out.value

    def info(self) -> dict:
        import json
        buf = C.create_string_buffer(1 << 14)
        check(lib().hora_server_info(self._h, buf, len(buf)))
        return json.loads(buf.value.decode())

    def close(self):
        if self._h:
            lib().hora_server_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        if getattr(self, "_h", None) and _lib._lib is not None:
            self.close()
